// Fused raymarch (RaymarchGridTransform) forward and adjoint.
//
// Forward semantics: kRaymarchGridTransformLindepth (raymarch_grid.cu.cc:107-143).
// One thread per pixel; the rays of all (batch, camera) pairs of a call run in
// one launch (grid.z = pair), where the reference launches once per camera
// with a host constant-buffer upload in between.  A warp covers an 8x4 pixel
// tile so that the 32 rays of a warp gather from neighbouring voxels.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "gft_internal.h"

namespace gft {

// 128 threads, warp = 8x4 pixels (measured at 480x270x192: 16x2 and 32x1
// pixel warps gather and scatter over more cells, 3 % and 9 % slower steps)
constexpr int RM_BX = 8, RM_BY = 16;

// Ray clipping.  Under BORDER a LINEAR or NEAREST sample is 0 outside
// (-1, dims + 0.5) in grid coordinates (the NEAREST domain int(p) in [0, dims)
// reaches down to -1, the reference-normalised scatter window -1 < p - 0.5 <
// dims up to dims + 0.5), and blending a zero sample leaves the accumulator
// unchanged.  So a ray only needs the steps i whose position p0 + i*st can lie
// in that box: [i_lo, i_hi] from a slab test, widened by a margin (0.05 voxels
// and one step) far above the rounding of the positions.  Sample i lies at
// fmaf(i, step, p0) (ray_sample), so the processed samples sit exactly where
// the full march puts them.  Returns false when no step can reach the box.
__device__ __forceinline__ bool ray_clip(float3 p0, float3 st, int n, Dims d, int& i_lo, int& i_hi) {
    float t0 = 0.f, t1 = (float)(n - 1);
    const float lo = -1.05f;
    auto axis = [&](float p, float s, float hi) {
        if (fabsf(s) < 1e-20f) {
            if (!(p >= lo && p <= hi)) t0 = 2.f * t1 + 2.f;  // never inside (NaN positions too)
            return;
        }
        const float a = (lo - p) / s, b = (hi - p) / s;
        t0 = fmaxf(t0, fminf(a, b));
        t1 = fminf(t1, fmaxf(a, b));
    };
    axis(p0.x, st.x, (float)d.x + 0.55f);
    axis(p0.y, st.y, (float)d.y + 0.55f);
    axis(p0.z, st.z, (float)d.z + 0.55f);
    if (!(t0 <= t1)) return false;
    i_lo = max(0, (int)floorf(t0) - 1);
    i_hi = min(n - 1, (int)ceilf(t1) + 1);
    return true;
}

// The blocks of one launch tile the images of all its pairs (8x16 pixels per
// block, row-major per pair, pairs one after another, tab.tile0): pairs may
// differ in image size and sample count.  Sets this thread's pair, pixel and
// the pair's geometry; false for pixels outside the pair's image.
struct RayPix {
    int tile;  // pixel tile of the launch (set by the caller)
    int p, x, y, W, H, D;
};

// Position of sample i of a ray: near + i * step with one rounding per
// coordinate.  The reference walks the ray by repeated addition
// (raymarch_grid.cu.cc:122-140, its adjoint by repeated subtraction from the far
// end, :354-370), whose rounding error grows along the ray: at 960x540x256 on a
// 256x455x256 grid that drift changes the unnormalised (exact) adjoint by
// ~3e-4 rel-L2 against fp64 positions, against ~2e-5 here.  The forward and
// every adjoint pass evaluate the same expression, so they sample the same
// points bit for bit.
__device__ __forceinline__ float3 ray_sample(float3 nearp, float3 step, int i) {
    const float t = (float)i;
    return make_float3(fmaf(t, step.x, nearp.x), fmaf(t, step.y, nearp.y), fmaf(t, step.z, nearp.z));
}
__device__ __forceinline__ bool ray_pixel(const PairTable& tab, RayPix& r) {
    const int b = r.tile;
    int p = 0;
    while (p + 1 < tab.n && b >= tab.tile0[p + 1]) ++p;
    r.p = p;
    r.W = tab.rw[p];
    r.H = tab.rh[p];
    r.D = tab.rd[p];
    const int tiles_x = (r.W + RM_BX - 1) / RM_BX;
    const int t = b - tab.tile0[p];
    const int ty = t / tiles_x;
    r.x = (t - ty * tiles_x) * RM_BX + threadIdx.x;
    r.y = ty * RM_BY + threadIdx.y;
    return r.x < r.W && r.y < r.H;
}

// Warp-aligned march: every lane of the warp walks the union [w0, w1] of the
// lanes' clipped step ranges and processes only its own [i0, i1].  Lanes that
// march the same step index sit at neighbouring positions (the rays of an 8x4
// pixel tile at one depth), so a warp's gathers and reductions at one step hit
// a few neighbouring cells; with per-lane ranges the lanes' entry steps differ
// by 1-3 (up to ~10) steps, 1.6 voxels each at 480x270x192 on a 128^3-voxel
// scale, and their samples scatter over as many cells.  The union costs about
// 0.1 % more warp iterations there.  All 32 lanes of the warp must call this
// (no lane has returned before); a lane without samples passes hit = false.
__device__ __forceinline__ void warp_clip_range(bool hit, int D, int& i0, int& i1, int& w0, int& w1) {
    if (!hit) {
        i0 = D;
        i1 = -1;
    }
    w0 = __reduce_min_sync(0xffffffffu, i0);
    w1 = __reduce_max_sync(0xffffffffu, i1);
}

static int ray_tiles(int W, int H) { return ((W + RM_BX - 1) / RM_BX) * ((H + RM_BY - 1) / RM_BY); }

// Fills tab.tile0 and the sample store offsets tab.smp0 (host side; *cells:
// the store cells of the pairs of earlier tables, advanced past this table's)
// and returns the blocks of the launch.  Sample store layout, in cells of C
// floats: per pair, per tile block, per step i (front to back), the block's
// 128 lanes: cell smp0[p] + ((block - tile0[p]) * D + i) * 128 + lane, so that
// a warp's step is 32 consecutive cells (512 bytes for C == 4).
static unsigned set_ray_tiles(PairTable& t, int64_t* cells = nullptr) {
    int b = 0;
    int64_t f = cells ? *cells : 0;
    for (int k = 0; k < t.n; ++k) {
        t.tile0[k] = b;
        t.smp0[k] = f;
        const int tiles = ray_tiles(t.rw[k], t.rh[k]);
        b += tiles;
        f += (int64_t)tiles * t.rd[k] * (RM_BX * RM_BY);
    }
    t.tile0[t.n] = b;
    if (cells) *cells = f;
    return (unsigned)b;
}

// ---- sample store ----------------------------------------------------------------
// The differentiable forward keeps the samples it blends for the adjoint.  Only
// samples that can be non-zero are written: a sample whose 8 corners lie in a
// 4^3-voxel block without a non-zero voxel (grown by one voxel at its upper
// faces, so that it holds every corner of a sample with its base cell in the
// block) is exactly zero, and the forward neither fetches nor stores it; per
// warp and step a ballot word records which lanes have a non-zero sample, and
// the adjoint uses zero where a lane's bit is clear.
//
// The samples go into a pool that warps fill in chunks: a warp takes
// STORE_CHUNK cells from the store's counter when its current chunk cannot
// hold a step's samples, writes them at consecutive cells (in lane order) and
// records the step's first cell beside its ballot word.  A pool smaller than
// every sample the launch could store is allowed: once a chunk request goes
// past the pool's end the warp records STORE_OVERFLOW for its remaining steps
// of the tile, and the adjoint re-samples the grid there.
//
// Layout: [counter (one uint64), 256 bytes][ballot words][first cells][occupancy
// maps][empty-space distance maps][their scratch][pool]: the words and first
// cells hold one uint32 per pair, pixel tile, step and warp; the maps one byte
// per input slice and block.
constexpr int OCC_SHIFT = 2;  // 4^3-voxel occupancy blocks
constexpr uint32_t STORE_CHUNK = 256;
constexpr uint32_t STORE_OVERFLOW = 0xffffffffu;

static int64_t store_cells(const std::vector<Pair>& pairs) {
    int64_t f = 0;
    for (const Pair& p : pairs) f += (int64_t)ray_tiles(p.W, p.H) * p.D * (RM_BX * RM_BY);
    return f;
}
static Dims occ_dims(Dims d) {
    const int b = 1 << OCC_SHIFT;
    return Dims{(d.x + b - 1) / b, (d.y + b - 1) / b, (d.z + b - 1) / b};
}
static size_t align256u(size_t n) { return (n + 255) & ~size_t(255); }

// bytes before the pool
static size_t store_meta_bytes(const std::vector<Pair>& pairs, int N, Dims din) {
    const int64_t cells = store_cells(pairs);
    return 256 + 2 * align256u(sizeof(uint32_t) * (cells / 32)) + 3 * align256u((size_t)voxels(occ_dims(din)) * N);
}
size_t raymarch_store_min_bytes(const std::vector<Pair>& pairs, int N, Dims din) {
    return store_meta_bytes(pairs, N, din);
}
// Pool cells that hold every sample the launch could store: a warp abandons a
// chunk only when a step's samples (at most 32) do not fit its rest, so each
// abandoned chunk holds at least STORE_CHUNK - 31 samples, and each warp's
// last chunk of a tile may be mostly empty.
static int64_t store_pool_full_cells(const std::vector<Pair>& pairs) {
    int64_t f = 0;
    for (const Pair& p : pairs) {
        const int64_t tiles = ray_tiles(p.W, p.H), cells = tiles * p.D * (RM_BX * RM_BY);
        f += (cells * STORE_CHUNK + (STORE_CHUNK - 32)) / (STORE_CHUNK - 31) +
             tiles * (RM_BX * RM_BY / 32) * STORE_CHUNK;
    }
    return f;
}
size_t raymarch_store_bytes(const std::vector<Pair>& pairs, int C, int N, Dims din) {
    return store_meta_bytes(pairs, N, din) + align256u(sizeof(float) * store_pool_full_cells(pairs) * C);
}

RaymarchArgs::Store raymarch_store_layout(void* base, size_t bytes, const std::vector<Pair>& pairs, int C, int N,
                                          Dims din) {
    RaymarchArgs::Store st;
    const int64_t cells = store_cells(pairs);
    char* p = static_cast<char*>(base);
    st.count = reinterpret_cast<unsigned long long*>(p);
    p += 256;
    st.words = reinterpret_cast<uint32_t*>(p);
    p += align256u(sizeof(uint32_t) * (cells / 32));
    st.first = reinterpret_cast<uint32_t*>(p);
    p += align256u(sizeof(uint32_t) * (cells / 32));
    st.occ = reinterpret_cast<uint8_t*>(p);
    const Dims od = occ_dims(din);
    st.nbx = od.x;
    st.nby = od.y;
    st.nbz = od.z;
    p += align256u((size_t)voxels(od) * N);
    st.dist = reinterpret_cast<uint8_t*>(p);
    p += align256u((size_t)voxels(od) * N);
    st.dist_tmp = reinterpret_cast<uint8_t*>(p);
    p += align256u((size_t)voxels(od) * N);
    st.samples = reinterpret_cast<float*>(p);
    const size_t meta = store_meta_bytes(pairs, N, din);
    const uint64_t cap = bytes > meta ? (uint64_t)((bytes - meta) / (sizeof(float) * (size_t)C)) : 0;
    st.capacity = (uint32_t)std::min<uint64_t>(cap, STORE_OVERFLOW - 1);
    return st;
}

// Index of this lane's warp's ballot word (and first cell) for step i (a
// pair's words start at smp0 / 32).
__device__ __forceinline__ int64_t sample_word_index(const PairTable& tab, int tile, int p, int D, int i) {
    const int tid = threadIdx.y * RM_BX + threadIdx.x;
    return (tab.smp0[p] >> 5) + ((int64_t)(tile - tab.tile0[p]) * D + i) * (RM_BX * RM_BY / 32) + (tid >> 5);
}

// Rank of this lane among the set bits of a warp's ballot word.
__device__ __forceinline__ uint32_t lane_rank(unsigned word, unsigned lane) {
    return (uint32_t)__popc(word & ((1u << lane) - 1u));
}

// Occupancy of one input slice per block: a non-zero voxel marks the blocks
// whose grown region holds it (its own, and the lower neighbour along each axis
// where it lies on the block's lower face); all writers store 1.
template <int C, typename S, int L>
__global__ void k_raymarch_occupancy(const S* __restrict__ in, Dims d, uint8_t* __restrict__ occ, Dims od) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= voxels(d)) return;
    const int n = blockIdx.y;
    int x, y, z;
    unflat32(v, d, x, y, z);
    const Vec<C> a = Load<C, S>::at(in + (size_t)n * slice_cells<L>(d) * C, cell_index<L>(x, y, z, d));
    bool nonzero = false;
#pragma unroll
    for (int c = 0; c < C; ++c) nonzero = nonzero || a.v[c] != 0.f;  // NaN counts as non-zero
    if (!nonzero) return;
    const int bx = x >> OCC_SHIFT, by = y >> OCC_SHIFT, bz = z >> OCC_SHIFT;
    const int mask = (1 << OCC_SHIFT) - 1;
    const int ex = (x & mask) == 0 && bx > 0, ey = (y & mask) == 0 && by > 0, ez = (z & mask) == 0 && bz > 0;
    uint8_t* o = occ + (size_t)n * voxels(od);
    for (int k = 0; k <= ez; ++k)
        for (int j = 0; j <= ey; ++j)
            for (int i = 0; i <= ex; ++i) o[((size_t)(bz - k) * od.y + (by - j)) * od.x + (bx - i)] = 1;
}

// Brick layout: one thread per 2x2x2-voxel brick (its 8 cells contiguous); a
// non-zero brick marks its block and, where it lies on the block's lower face
// along an axis (even brick coordinate), the lower neighbour too: at least
// every block that a non-zero voxel of it marks (more is safe).
template <int C, typename S>
__global__ void k_raymarch_occupancy_bricks(const S* __restrict__ in, Dims d, uint8_t* __restrict__ occ, Dims od) {
    const Dims bd{(d.x + 1) / 2, (d.y + 1) / 2, (d.z + 1) / 2};
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= voxels(bd)) return;
    const int n = blockIdx.y;
    const S* g = in + (size_t)n * brick_cells(d) * C + (size_t)b * 8 * C;
    bool nonzero = false;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const Vec<C> a = Load<C, S>::at(g, k);  // cells outside the grid hold zeros or are never read
#pragma unroll
        for (int c = 0; c < C; ++c) nonzero = nonzero || a.v[c] != 0.f;  // NaN counts as non-zero
    }
    if (!nonzero) return;
    int x2, y2, z2;
    unflat32(b, bd, x2, y2, z2);
    const int bx = x2 >> (OCC_SHIFT - 1), by = y2 >> (OCC_SHIFT - 1), bz = z2 >> (OCC_SHIFT - 1);
    const int ex = (x2 & 1) == 0 && bx > 0, ey = (y2 & 1) == 0 && by > 0, ez = (z2 & 1) == 0 && bz > 0;
    uint8_t* o = occ + (size_t)n * voxels(od);
    for (int k = 0; k <= ez; ++k)
        for (int j = 0; j <= ey; ++j)
            for (int i = 0; i <= ex; ++i) o[((size_t)(bz - k) * od.y + (by - j)) * od.x + (bx - i)] = 1;
}

template <int C, typename S, int L>
static void occ_launch(const RaymarchArgs& a, cudaStream_t s) {
    const Dims od{a.store.nbx, a.store.nby, a.store.nbz};
    if constexpr (L == LAYOUT_BRICK) {
        const dim3 grid((unsigned)((brick_cells(a.din) / 8 + 255) / 256), (unsigned)a.N);
        k_raymarch_occupancy_bricks<C, S><<<grid, 256, 0, s>>>((const S*)a.input, a.din, a.store.occ, od);
    } else {
        const dim3 grid((unsigned)((voxels(a.din) + 255) / 256), (unsigned)a.N);
        k_raymarch_occupancy<C, S, L><<<grid, 256, 0, s>>>((const S*)a.input, a.din, a.store.occ, od);
    }
}

// Empty-space distance of each block: the Chebyshev distance, in blocks, to
// the nearest block the occupancy map marks (capped at DIST_CAP), so that the
// storing forward can step over samples that are all zero.  Three 1D passes:
// along x the distance to the nearest marked block of the row; along y and z
// the smallest max(|offset|, previous distance) over the offsets up to the cap
// -- the min-max composition is exactly the Chebyshev distance.  Blocks
// outside the map are never looked up (positions are clamped to the grid).
constexpr int DIST_CAP = 7;
template <int AXIS>
__global__ void k_empty_distance(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, Dims od) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= voxels(od)) return;
    const size_t base = (size_t)blockIdx.y * voxels(od);
    int x, y, z;
    unflat32(v, od, x, y, z);
    const int c = AXIS == 0 ? x : AXIS == 1 ? y : z;
    const int n = AXIS == 0 ? od.x : AXIS == 1 ? od.y : od.z;
    const int64_t stride = AXIS == 0 ? 1 : AXIS == 1 ? od.x : (int64_t)od.x * od.y;
    const uint8_t* row = src + base + v - (int64_t)c * stride;
    int best = DIST_CAP;
    for (int o = -(DIST_CAP - 1); o <= DIST_CAP - 1; ++o) {
        const int k = c + o;
        if (k < 0 || k >= n) continue;
        const int val = row[(int64_t)k * stride];
        const int dd = AXIS == 0 ? (val != 0 ? abs(o) : DIST_CAP) : max(abs(o), (int)val);
        best = min(best, dd);
    }
    dst[base + v] = (uint8_t)best;
}

bool launch_raymarch_occupancy(const RaymarchArgs& a, cudaStream_t s) {
    const Dims od{a.store.nbx, a.store.nby, a.store.nbz};
    if (!cuda_ok(cudaMemsetAsync(a.store.occ, 0, (size_t)voxels(od) * a.N, s), "zero occupancy")) return false;
    // ballot words of steps no warp marches stay 0, so the store is fully
    // defined; the pool counter starts at 0
    const size_t words = reinterpret_cast<const char*>(a.store.first) - reinterpret_cast<const char*>(a.store.words);
    if (!cuda_ok(cudaMemsetAsync(a.store.words, 0, words, s), "zero sample words") ||
        !cuda_ok(cudaMemsetAsync(a.store.count, 0, sizeof(unsigned long long), s), "zero sample counter"))
        return false;
    const bool brick = a.layout == LAYOUT_BRICK;
    if (a.dtype == 0) {
        if (a.C == 4) brick ? occ_launch<4, float, LAYOUT_BRICK>(a, s) : occ_launch<4, float, LAYOUT_FLAT>(a, s);
        else if (a.C == 2) brick ? occ_launch<2, float, LAYOUT_BRICK>(a, s) : occ_launch<2, float, LAYOUT_FLAT>(a, s);
        else brick ? occ_launch<1, float, LAYOUT_BRICK>(a, s) : occ_launch<1, float, LAYOUT_FLAT>(a, s);
    } else {
        if (a.C == 4) brick ? occ_launch<4, __nv_bfloat16, LAYOUT_BRICK>(a, s) : occ_launch<4, __nv_bfloat16, LAYOUT_FLAT>(a, s);
        else if (a.C == 2) brick ? occ_launch<2, __nv_bfloat16, LAYOUT_BRICK>(a, s) : occ_launch<2, __nv_bfloat16, LAYOUT_FLAT>(a, s);
        else brick ? occ_launch<1, __nv_bfloat16, LAYOUT_BRICK>(a, s) : occ_launch<1, __nv_bfloat16, LAYOUT_FLAT>(a, s);
    }
    if (!launched(1, "raymarch occupancy launch")) return false;
    // occupancy -> distance along x (dist) -> y (dist_tmp) -> z (dist, the
    // map the forward reads)
    const dim3 grid((unsigned)((voxels(od) + 255) / 256), (unsigned)a.N);
    k_empty_distance<0><<<grid, 256, 0, s>>>(a.store.occ, a.store.dist, od);
    k_empty_distance<1><<<grid, 256, 0, s>>>(a.store.dist, a.store.dist_tmp, od);
    k_empty_distance<2><<<grid, 256, 0, s>>>(a.store.dist_tmp, a.store.dist, od);
    return launched(3, "raymarch empty-distance launch");
}

// The sample at p is exactly zero by the occupancy map, without a fetch, where
// its corners that the boundary mode reads lie in the grown region of one
// block without a non-zero voxel.  BORDER and CLAMP: the block of the base
// cell clamped to the grid (corners outside read 0 resp. the clamped border
// voxels, which that block holds); WRAP: interior base cells only (all 8
// corners inside).  Non-finite positions are fetched.  sample_distance
// returns that block's empty-space distance (>= 1: the sample is zero), or 0
// where the sample must be fetched.
template <int BM>
__device__ __forceinline__ int sample_distance(Dims d, float px, float py, float pz, const uint8_t* __restrict__ dist,
                                               int nbx, int nby) {
    if (!(fabsf(px) <= 3.0e9f && fabsf(py) <= 3.0e9f && fabsf(pz) <= 3.0e9f)) return 0;
    int x0 = (int)floorf(px), y0 = (int)floorf(py), z0 = (int)floorf(pz);
    if constexpr (BM == BM_WRAP) {
        if (!((unsigned)x0 < (unsigned)(d.x - 1) && (unsigned)y0 < (unsigned)(d.y - 1) &&
              (unsigned)z0 < (unsigned)(d.z - 1)))
            return 0;
    } else {
        x0 = min(max(x0, 0), d.x - 1);
        y0 = min(max(y0, 0), d.y - 1);
        z0 = min(max(z0, 0), d.z - 1);
    }
    return __ldg(dist + ((uint32_t)(z0 >> OCC_SHIFT) * nby + (uint32_t)(y0 >> OCC_SHIFT)) * nbx + (x0 >> OCC_SHIFT));
}

template <int C, typename S, int BM, bool LIN, int L>
__device__ __forceinline__ void raymarch_fwd_tile(const S* __restrict__ in, Dims din, int filter, int blend_mode,
                                                  float* __restrict__ out, const RaymarchArgs::Store& st,
                                                  const PairTable& tab, int tile) {
    RayPix r;
    r.tile = tile;
    const bool live = ray_pixel(tab, r);  // every lane stays to the warp's clip reduction
    const int p = r.p, x = r.x, y = r.y, W = r.W, H = r.H, D = r.D;
    const CamX& cam = tab.cam[p];
    const S* g = in + (size_t)tab.in_batch[p] * slice_cells<L>(din) * C;
    const float3 dinv = make_float3(1.f / (float)W, 1.f / (float)H, 1.f / (float)D);
    const float zmax = (float)max(D - 1, 1);
    const float3 nearp = idx_to_os(cam, make_float3(x + 0.5f, y + 0.5f, 0.5f), dinv);
    const float3 farp = idx_to_os(cam, make_float3(x + 0.5f, y + 0.5f, zmax + 0.5f), dinv);
    const float3 step = make_float3((farp.x - nearp.x) / zmax, (farp.y - nearp.y) / zmax, (farp.z - nearp.z) / zmax);
    Vec<C> acc = vzero<C>();
    int i0 = 0, i1 = D - 1, w0 = 0, w1 = D - 1;
    // Storing samples (LINEAR): every lane stays in the loop to the warp's
    // last step, for the per-step ballot of the lanes that stored one.
    const bool storing = LIN && st.samples != nullptr;
    // MIN/MAX samples outside are +-FLOAT_MAX, and BEER_LAMBERT_EXCLUSIVE
    // multiplies a zero sample by exp(-density sum), which overflows for
    // sums below -88: neither is clipped.
    if (BM == BM_BORDER && (LIN || filter == F_NEAREST) && (C == 1 || blend_mode != BL_BEER_LAMBERT_EXCLUSIVE)) {
        const bool hit = live && ray_clip(nearp, step, D, din, i0, i1);
        warp_clip_range(hit, D, i0, i1, w0, w1);  // i0 > i1 where !hit
        if (!storing) {
            if (!live) return;
            if (!hit) {
                store<C>(out, tab.pix0[p] + (int64_t)y * W + x, acc);
                return;
            }
        }
    } else if (!live) {
        if (!storing) return;
        i0 = D;
        i1 = -1;
    }
    const uint8_t* dist = storing ? st.dist + (size_t)tab.in_batch[p] * st.nbx * st.nby * st.nbz : nullptr;
    const unsigned lane = (threadIdx.y * RM_BX + threadIdx.x) & 31u;
    // Empty-space skipping: where every sample of a warp step is zero, the
    // warp steps over the samples its lanes' distance maps prove zero too.  A
    // lane at q in a block at distance d reaches only blocks within d - 1 of
    // it (all empty) while it moves at most 4d - 6 voxels along each axis
    // (floor and the block shift add 1 and 3; 0.01 of slack covers the
    // rounding of the positions, which ray_sample computes directly from the
    // step index, so the samples processed are the same).  Zero samples leave
    // the blend unchanged exactly where the ray is clipped: the same
    // condition.  Lanes past their range do not limit the skip; lanes before
    // it limit it by their current position.
    const bool skipping = storing && BM == BM_BORDER && (C == 1 || blend_mode != BL_BEER_LAMBERT_EXCLUSIVE);
    const float smax = fmaxf(fabsf(step.x), fmaxf(fabsf(step.y), fabsf(step.z)));
    const float inv_smax = smax > 1e-6f ? 1.f / smax : 0.f;
    // the warp's current pool chunk [cur, end) (uniform across the warp);
    // full: a chunk request went past the pool's end
    uint32_t cur = 0, end = 0;
    bool full = false;
    for (int i = w0; i <= w1;) {
        bool nonzero = false;
        int dcur = 0;  // this lane's empty-space distance at step i
        Vec<C> smp = vzero<C>();
        if (i >= i0 && i <= i1) {
            const float3 pos = ray_sample(nearp, step, i);
            if constexpr (LIN) {
                const float qx = pos.x - 0.5f, qy = pos.y - 0.5f, qz = pos.z - 0.5f;
                if (storing) dcur = sample_distance<BM>(din, qx, qy, qz, dist, st.nbx, st.nby);
                const bool empty = dcur != 0;
                if (!empty) smp = fetch_linear<C, S, BM, L>(g, din, qx, qy, qz);
                nonzero = storing && !empty;
            } else {
                smp = fetch<C, S, BM, true>(filter, g, din, pos.x - 0.5f, pos.y - 0.5f, pos.z - 0.5f);
            }
            acc = blend<C>(blend_mode, acc, smp);
        } else if (skipping && live && i < i0) {
            const float3 pos = ray_sample(nearp, step, i);
            dcur = sample_distance<BM>(din, pos.x - 0.5f, pos.y - 0.5f, pos.z - 0.5f, dist, st.nbx, st.nby);
        }
        int adv = 1;
        if (storing) {
            const unsigned word = __ballot_sync(0xffffffffu, nonzero);
            if (skipping && word == 0u) {
                unsigned m = 0xffffffffu;
                if (live && i <= i1) {
                    const float lim = 4.f * (float)dcur - 6.01f;
                    m = lim > 0.f ? (unsigned)fminf(lim * inv_smax, 1e6f) : 0u;
                }
                m = __reduce_min_sync(0xffffffffu, m);
                adv = 1 + (int)min(m, (unsigned)(w1 - i));
            }
            uint32_t first = STORE_OVERFLOW;
            if (word != 0u && !full) {
                const uint32_t n = (uint32_t)__popc(word);
                if (end - cur < n) {
                    unsigned long long base = 0;
                    if (lane == 0) base = atomicAdd(st.count, (unsigned long long)STORE_CHUNK);
                    base = __shfl_sync(0xffffffffu, base, 0);
                    if (base + STORE_CHUNK <= (unsigned long long)st.capacity) {
                        cur = (uint32_t)base;
                        end = cur + STORE_CHUNK;
                    } else {
                        full = true;
                    }
                }
                if (!full) {
                    first = cur;
                    cur += n;
                }
            }
            if (nonzero && first != STORE_OVERFLOW)
                store_stream<C>(st.samples, (int64_t)(first + lane_rank(word, lane)), smp);
            if (lane == 0 && word != 0u) {  // the words start zeroed
                const int64_t w = sample_word_index(tab, r.tile, p, D, i);
                st.words[w] = word;
                st.first[w] = first;
            }
        }
        i += adv;
    }
    if (!live) return;
    store<C>(out, tab.pix0[p] + (int64_t)y * W + x, acc);
}

// The raymarch kernels walk the pixel tiles of their launch: one block per
// tile, or (a persistent grid, the launch-configuration knob
// GFT_KNOB_RAYMARCH_BLOCKS_PER_SM) a fixed number of blocks per SM taking
// tiles blockIdx.x, blockIdx.x + gridDim.x, ...  Every thread of a block walks
// the same tiles, so the warp-collective steps of a tile see all 32 lanes.
template <int C, typename S, int BM, bool LIN, int L>
__global__ void __launch_bounds__(RM_BX* RM_BY)
    k_raymarch_fwd(const S* __restrict__ in, Dims din, int filter, int blend_mode, float* __restrict__ out,
                   const RaymarchArgs::Store st, const __grid_constant__ PairTable tab) {
    const int tiles = tab.tile0[tab.n];
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x)
        raymarch_fwd_tile<C, S, BM, LIN, L>(in, din, filter, blend_mode, out, st, tab, tile);
}

// Ray set-up shared by the adjoint kernels: near point, far point and step,
// computed as the forward computes them (the adjoint visits the forward's
// samples i = D-1 .. 0 at ray_sample(nearp, step, i)).
__device__ __forceinline__ void ray_far_step(const CamX& cam, int x, int y, int W, int H, int D, float3& farp,
                                             float3& step, float3& nearp) {
    const float3 dinv = make_float3(1.f / (float)W, 1.f / (float)H, 1.f / (float)D);
    const float zmax = (float)max(D - 1, 1);
    nearp = idx_to_os(cam, make_float3(x + 0.5f, y + 0.5f, 0.5f), dinv);
    farp = idx_to_os(cam, make_float3(x + 0.5f, y + 0.5f, zmax + 0.5f), dinv);
    step = make_float3((farp.x - nearp.x) / zmax, (farp.y - nearp.y) / zmax, (farp.z - nearp.z) / zmax);
}


// --- adjoint scatters ----------------------------------------------------------
// Each sample's cell gradient reaches its eight corners as vector reductions
// (red.global.add.v4/v2.f32) in L2.  The lanes of a warp sample one depth per
// step (warp_clip_range), so neighbouring lanes often share a cell, and samples
// with the same base cell floor(p) share all eight corners: along each 8-lane
// pixel row, a run of lanes with the same base cell hands its members'
// fractions and values to the run's first lane (one shuffle round per member),
// which sums the eight corner contributions and issues one reduction per
// corner -- about half the reductions of one per lane and corner at the
// 5-view 480x270x192 workload (rows of 0.36-0.53 voxels per pixel).  Measured
// on GB300 there: weight pass 0.66 -> 0.59 ms, exact adjoint 1.17 -> 1.04 ms,
// normalised adjoint 1.29 -> 1.27 ms (its 32 accumulators, 8 corners x 4
// channels, take 80 registers; loading the reciprocal weights before the
// shuffle rounds was slower).  Alternatives measured earlier that did
// not pay: summing 2x1 / 1x2 / 2x2 neighbouring rays per thread in registers,
// and per-block shared-memory accumulation boxes flushed with coalesced
// reductions (the shared float atomics and round barriers cost more than the
// L2 sectors they save).
//
// Trilinear corner weights, corner k = (k & 1, k >> 1 & 1, k >> 2 & 1).
__device__ __forceinline__ void corner_weights(float fx, float fy, float fz, float w[8]) {
    const float ax[2] = {1.f - fx, fx}, ay[2] = {1.f - fy, fy};
    float wxy[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) wxy[j] = ax[j & 1] * ay[j >> 1];
#pragma unroll
    for (int k = 0; k < 8; ++k) w[k] = wxy[k & 3] * ((k & 4) ? fz : 1.f - fz);
}

// Bit k set where corner k's weight is non-zero, for fractions in [0, 1).
__device__ __forceinline__ unsigned zero_weight_mask(float fx, float fy, float fz) {
    return 0xffu & (fx != 0.f ? 0xffu : 0x55u) & (fy != 0.f ? 0xffu : 0x33u) & (fz != 0.f ? 0xffu : 0x0fu);
}

// One step of the warp's samples.  All 32 lanes call it; act = this lane has a
// sample.  MODE 0 (exact adjoint): BORDER drops the sample outside the
// forward's half-cell window.  MODE 1 (reference-normalised) and MODE 2 (weight
// sums): BORDER drops it unless -1 < p < dims, the reference's window; MODE 1
// scales each corner's sum by the reciprocal of the camera's weight sum there
// (the per-camera normalise-then-sum applied per contribution, so all cameras
// accumulate into one gradient) and skips corners with no weight.  Zero-weight
// contributions are skipped; the ceil corner is floor + 1 (the reference's
// ceil(p) equals floor(p) only where the ceil weight is 0).
// DET (deterministic adjoint): the corner sums go, scaled by the
// power of two iscale and rounded to integers, into int64 accumulators
// (MODE 2: one per brick cell of the pair; MODE 0/1: C per cell of the batch
// slice) instead of the float reductions; integer addition is associative, so
// the sums do not depend on the order in which the warps add them.
// MODE 3 (per-camera sums, the reference normalisation in one pass): the
// corner sums of the values go into the pair's own gradient, unscaled, and
// the corner sums of the weights into the pair's weight sums (wsum), from the
// same merge rounds; the caller divides per voxel afterwards.
template <int C, int BM, int MODE, int L, bool DET = false>
__device__ __forceinline__ void scatter_step(float* __restrict__ grad, const float* __restrict__ cnt, Dims d,
                                             bool act, float px, float py, float pz, Vec<C> val,
                                             unsigned long long* __restrict__ iacc = nullptr, float iscale = 0.f,
                                             float* __restrict__ wsum = nullptr) {
    static_assert(MODE != 3 || !DET, "per-camera sums: float path only");
    const unsigned lane = (threadIdx.y * RM_BX + threadIdx.x) & 31u;  // blockDim.x == RM_BX
    if constexpr (BM == BM_BORDER) {
        if constexpr (MODE != 0)
            act = act && px > -1.f && px < (float)d.x && py > -1.f && py < (float)d.y && pz > -1.f && pz < (float)d.z;
        else
            act = act && border_inside(px, py, pz, d);
    }
    const float flx = floorf(px), fly = floorf(py), flz = floorf(pz);
    const int x0 = (int)flx, y0 = (int)fly, z0 = (int)flz;
    const float wx = px - flx, wy = py - fly, wz = pz - flz;
    const int ux = __shfl_up_sync(0xffffffffu, x0, 1), uy = __shfl_up_sync(0xffffffffu, y0, 1),
              uz = __shfl_up_sync(0xffffffffu, z0, 1);
    const unsigned acts = __ballot_sync(0xffffffffu, act);
    const bool same = act && (lane & (RM_BX - 1)) != 0 && ((acts >> ((lane - 1) & 31u)) & 1u) && ux == x0 &&
                      uy == y0 && uz == z0;
    const unsigned follow = __ballot_sync(0xffffffffu, same);
    const bool head = act && !same;
    // members after the head: the 'same' lanes directly following it (a run
    // never crosses a row, whose first lane is never 'same'), at most 7
    const int n = head ? __ffs(~(unsigned)((unsigned long long)follow >> (lane + 1))) - 1 : 0;
    const int rounds = __reduce_max_sync(0xffffffffu, n);
    // Corner weights as products of per-axis factors (1 - f, f); f lies in
    // [0, 1), so a weight is zero exactly where it takes an f that is 0.  A
    // zero weight adds +0 to a finite sum; corners that no member reaches with
    // a non-zero weight are not reduced (nz).  (MODE 2: the value is 1.)
    float acc[8][C];
    float accw[8];  // MODE 3: the weights' corner sums
    // (MODE 2 adds weights, which are finite: a zero one adds +0 and needs no
    // mask)
    unsigned nz = MODE == 2 ? 0xffu : zero_weight_mask(wx, wy, wz);
    {
        float w[8];
        corner_weights(wx, wy, wz, w);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
#pragma unroll
            for (int c = 0; c < C; ++c) acc[k][c] = MODE == 2 ? w[k] : w[k] * val.v[c];
            if constexpr (MODE == 3) accw[k] = w[k];
        }
    }
    if constexpr (MODE == 2) {
        // Weight sums: the head pulls each member's three fractions (not its
        // eight weights: shuffles are the scarcer issue slots) and adds the
        // member's corner weights.  Corners no member weights receive +0,
        // which leaves the sums unchanged (the adjoint skips them).
        for (int r = 1; r <= rounds; ++r) {
            const float mx = __shfl_down_sync(0xffffffffu, wx, r), my = __shfl_down_sync(0xffffffffu, wy, r),
                        mz = __shfl_down_sync(0xffffffffu, wz, r);
            if (r <= n) {
                float w[8];
                corner_weights(mx, my, mz, w);
#pragma unroll
                for (int k = 0; k < 8; ++k) acc[k][0] += w[k];
            }
        }
    } else {
        for (int r = 1; r <= rounds; ++r) {
            const float mx = __shfl_down_sync(0xffffffffu, wx, r), my = __shfl_down_sync(0xffffffffu, wy, r),
                        mz = __shfl_down_sync(0xffffffffu, wz, r);
            float mv[C];
#pragma unroll
            for (int c = 0; c < C; ++c) mv[c] = __shfl_down_sync(0xffffffffu, val.v[c], r);
            if (r <= n) {
                nz |= zero_weight_mask(mx, my, mz);
                float w[8];
                corner_weights(mx, my, mz, w);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
#pragma unroll
                    for (int c = 0; c < C; ++c) acc[k][c] = fmaf(w[k], mv[c], acc[k][c]);
                    if constexpr (MODE == 3) accw[k] += w[k];
                }
            }
        }
    }
    if (!head) return;
    if constexpr (BM == BM_BORDER) {
        // BORDER: the corners are base + (0|1) per axis without a remap.  In
        // the bricks the +1 neighbour along x is the next cell of the brick
        // (even x0) or cell 0 of the next brick, 7 cells on (odd x0); along y
        // 2 cells or a brick row minus 2, along z 4 cells or a brick slab
        // minus 4.  In 32-bit arithmetic this holds for the base -1 too (its
        // index wraps below 0 and its neighbour lands on cell 0).  Corners
        // outside the grid (base -1, or base + 1 = dims) are left out through
        // a mask of the eight corners.
        const uint32_t bx = (uint32_t)(d.x + 1) / 2, bxy = bx * ((uint32_t)(d.y + 1) / 2);
        const uint32_t bbase = (uint32_t)(x0 >> 1) * 8u + (uint32_t)(x0 & 1) + (uint32_t)(y0 >> 1) * bx * 8u +
                               ((uint32_t)(y0 & 1) << 1) + (uint32_t)(z0 >> 1) * bxy * 8u + ((uint32_t)(z0 & 1) << 2);
        const uint32_t box = (x0 & 1) ? 7u : 1u, boy = (y0 & 1) ? bx * 8u - 2u : 2u,
                       boz = (z0 & 1) ? bxy * 8u - 4u : 4u;
        uint32_t cbase = bbase, cox = box, coy = boy, coz = boz;
        if constexpr (L == LAYOUT_FLAT) {
            cbase = (uint32_t)x0 + (uint32_t)y0 * (uint32_t)d.x + (uint32_t)z0 * (uint32_t)d.x * (uint32_t)d.y;
            cox = 1u;
            coy = (uint32_t)d.x;
            coz = (uint32_t)d.x * (uint32_t)d.y;
        }
        unsigned mask = nz;
        if (x0 < 0) mask &= 0xaau;
        if (x0 + 1 >= d.x) mask &= 0x55u;
        if (y0 < 0) mask &= 0xccu;
        if (y0 + 1 >= d.y) mask &= 0x33u;
        if (z0 < 0) mask &= 0xf0u;
        if (z0 + 1 >= d.z) mask &= 0x0fu;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int sx = k & 1, sy = (k >> 1) & 1, sz = (k >> 2) & 1;
            if (!((mask >> k) & 1u)) continue;
            const uint32_t bi = bbase + (sx ? box : 0u) + (sy ? boy : 0u) + (sz ? boz : 0u);
            const uint32_t ci = L == LAYOUT_FLAT ? cbase + (sx ? cox : 0u) + (sy ? coy : 0u) + (sz ? coz : 0u) : bi;
            Vec<C> a;
#pragma unroll
            for (int c = 0; c < C; ++c) a.v[c] = acc[k][c];
            if constexpr (DET) {
                if constexpr (MODE == 2) {
                    atomicAdd(iacc + bi, (unsigned long long)__float2ll_rn(a.v[0] * iscale));
                } else {
                    float inv = 1.f;
                    if constexpr (MODE == 1) inv = __ldg(cnt + bi);
                    if (inv > 0.f) {
#pragma unroll
                        for (int c = 0; c < C; ++c)
                            atomicAdd(iacc + (uint64_t)ci * C + c,
                                      (unsigned long long)__float2ll_rn(a.v[c] * inv * iscale));
                    }
                }
                continue;
            }
            if constexpr (MODE == 1) {
                const float inv = __ldg(cnt + bi);
                if (inv > 0.f) atomic_add<C>(grad, ci, vscale(a, inv));
            } else if constexpr (MODE == 2) {
                atomic_add<C>(grad, bi, a);
            } else if constexpr (MODE == 3) {
                atomic_add<C>(grad, ci, a);
                atomicAdd(wsum + bi, accw[k]);
            } else {
                atomic_add<C>(grad, ci, a);
            }
        }
        return;
    }
    int xs[2] = {x0, x0 + 1}, ys[2] = {y0, y0 + 1}, zs[2] = {z0, z0 + 1};
    bool vx[2] = {true, true}, vy[2] = {true, true}, vz[2] = {true, true};
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        if constexpr (BM == BM_BORDER) {
            vx[i] = xs[i] > -1 && xs[i] < d.x;
            vy[i] = ys[i] > -1 && ys[i] < d.y;
            vz[i] = zs[i] > -1 && zs[i] < d.z;
        } else {
            xs[i] = remap<BM>(xs[i], d.x);
            ys[i] = remap<BM>(ys[i], d.y);
            zs[i] = remap<BM>(zs[i], d.z);
        }
    }
    // cell indices as sums of per-axis terms (brick_index, flat3), in 32 bits:
    // the callers limit a grid slice to 2^32 cells (terms of invalid corners
    // wrap but are not used)
    const uint32_t bx = (uint32_t)(d.x + 1) / 2, bxy = bx * ((uint32_t)(d.y + 1) / 2);
    uint32_t bt[3][2], ct[3][2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        bt[0][i] = (uint32_t)(xs[i] >> 1) * 8u + (uint32_t)(xs[i] & 1);
        bt[1][i] = (uint32_t)(ys[i] >> 1) * bx * 8u + ((uint32_t)(ys[i] & 1) << 1);
        bt[2][i] = (uint32_t)(zs[i] >> 1) * bxy * 8u + ((uint32_t)(zs[i] & 1) << 2);
        if constexpr (L == LAYOUT_FLAT) {
            ct[0][i] = (uint32_t)xs[i];
            ct[1][i] = (uint32_t)ys[i] * (uint32_t)d.x;
            ct[2][i] = (uint32_t)zs[i] * (uint32_t)d.x * (uint32_t)d.y;
        }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int sx = k & 1, sy = (k >> 1) & 1, sz = (k >> 2) & 1;
        if (!((nz >> k) & 1u) || !(vx[sx] && vy[sy] && vz[sz])) continue;
        const uint32_t bi = bt[0][sx] + bt[1][sy] + bt[2][sz];
        const uint32_t ci = L == LAYOUT_FLAT ? ct[0][sx] + ct[1][sy] + ct[2][sz] : bi;
        Vec<C> a;
#pragma unroll
        for (int c = 0; c < C; ++c) a.v[c] = acc[k][c];
        if constexpr (DET) {
            if constexpr (MODE == 2) {
                atomicAdd(iacc + bi, (unsigned long long)__float2ll_rn(a.v[0] * iscale));
            } else {
                float inv = 1.f;
                if constexpr (MODE == 1) inv = __ldg(cnt + bi);
                if (inv > 0.f) {
#pragma unroll
                    for (int c = 0; c < C; ++c)
                        atomicAdd(iacc + (uint64_t)ci * C + c, (unsigned long long)__float2ll_rn(a.v[c] * inv * iscale));
                }
            }
            continue;
        }
        if constexpr (MODE == 1) {
            const float inv = __ldg(cnt + bi);
            if (inv > 0.f) atomic_add<C>(grad, ci, vscale(a, inv));
        } else if constexpr (MODE == 2) {
            atomic_add<C>(grad, bi, a);
        } else if constexpr (MODE == 3) {
            atomic_add<C>(grad, ci, a);
            atomicAdd(wsum + bi, accw[k]);
        } else {
            atomic_add<C>(grad, ci, a);
        }
    }
}

// Back to front from the far end point over the (clipped) samples of one ray.
// MODE 2, the reference normalisation's first pass: per (batch, camera) pair
// the per-voxel sum of the trilinear weights of all its samples (the float
// sampleCounter of raymarch_grid.cu.cc:446-456) in the brick layout
// (brick_index); geometry only, C == 1, no gathers.  MODE 0 / 1, the adjoint:
// re-sample (LINEAR only, as the reference gradient op), step the blend
// adjoint and scatter the cell gradient into the batch gradient; MODE 1
// normalises by the pass-1 sums, which equals the reference's per-camera
// normalise-then-sum (kNormalize3DGradients, raymarch_grid.cu.cc:319-341 and
// :519-568) without per-camera buffers.
//
// Clipping (BORDER): a zero sample's adjoint step leaves the state unchanged
// for ADDITIVE, ALPHA_ADDITIVE and C == 1, and for the two BEER_LAMBERT modes
// when the density of the accumulated output is >= 0 (always the case for a
// forward output; a negative one is first clamped by max(., 0), so such rays
// march in full).  ALPHA changes its bookkeeping on every step and marches in
// full.  (Non-finite adjoints are not propagated through skipped samples.)
// Every lane stays in the loop to its warp's last step (scatter_step is
// warp-collective); lanes without a sample at a step pass act = false.
//
// PROJ (C == 4): each sample's 4-channel adjoint is projected onto two
// channels, (pj.a . g, pj.b . g), before its corner reduction, and the
// gradient holds those two per cell (DET: two integer sums per cell).  A
// caller whose next adjoint is linear in the four channels with coefficients
// of the form (per-voxel factor) x (constant) -- the light composition --
// needs only the two sums, and the reductions move half the bytes.
template <int C, typename S, int BM, int MODE, int L, bool DET, bool PROJ>
__device__ __forceinline__ void raymarch_scatter_tile(const S* __restrict__ in, Dims din, int blend_mode,
                                                      const float* __restrict__ out, const float* __restrict__ dout,
                                                      float* __restrict__ grad, const float* __restrict__ cnt,
                                                      unsigned long long* __restrict__ iacc, float iscale,
                                                      const RaymarchArgs::Store& st, const PairTable& tab, int tile,
                                                      const ChanProj& pj) {
    static_assert(!PROJ || (C == 4 && MODE != 2 && !(DET && MODE == 3)), "projection: 4-channel adjoint only");
    static_assert(MODE != 3 || PROJ, "per-camera sums: projected adjoint only");
    constexpr int CA = PROJ ? 2 : C;  // channels of the accumulated gradient
    RayPix r;
    r.tile = tile;
    const bool live = ray_pixel(tab, r);
    const int p = r.p, x = r.x, y = r.y, W = r.W, H = r.H, D = r.D;
    unsigned long long* idst =
        !DET        ? nullptr
        : MODE == 2 ? iacc + (size_t)(tab.pair_base + p) * brick_cells(din)
                        : iacc + (size_t)tab.in_batch[p] * slice_cells<L>(din) * CA;
    float3 farp, step, nearp;
    ray_far_step(tab.cam[p], x, y, W, H, D, farp, step, nearp);
    // With a sample store: the forward's own clip range (front-to-back steps
    // [s_lo, s_hi], computed from the same near point and step as there); its
    // samples outside are zero (BORDER), inside it stored the non-zero ones.
    const bool use_store = MODE != 2 && st.samples != nullptr;
    int s_lo = 0, s_hi = D - 1;
    if (use_store && BM == BM_BORDER)
        if (!ray_clip(nearp, step, D, din, s_lo, s_hi)) {
            s_lo = D;
            s_hi = -1;
        }
    const S* g = in + (size_t)tab.in_batch[p] * slice_cells<L>(din) * C;
    float* dst = MODE == 2   ? grad + (size_t)(tab.pair_base + p) * brick_cells(din)
                 : MODE == 3 ? grad + (size_t)(tab.pair_base + p) * slice_cells<L>(din) * CA
                             : grad + (size_t)tab.in_batch[p] * slice_cells<L>(din) * CA;
    const float* count = MODE == 1 ? cnt + (size_t)(tab.pair_base + p) * brick_cells(din) : nullptr;
    // MODE 3: the pair's weight sums (the workspace, written by this pass)
    float* wdst = MODE == 3 ? const_cast<float*>(cnt) + (size_t)(tab.pair_base + p) * brick_cells(din) : nullptr;
    Vec<C> acc = vzero<C>(), go = vzero<C>();
    if (MODE != 2 && live) {
        const int64_t pix = tab.pix0[p] + (int64_t)y * W + x;
        acc = loadf<C>(out, pix);
        go = loadf<C>(dout, pix);
    }
    // the adjoint visits the forward's samples back to front: step k is
    // sample i = D - 1 - k
    int k_lo = 0, k_hi = D - 1, w_lo = 0, w_hi = D - 1;
    if constexpr (BM == BM_BORDER) {
        const bool clip = MODE == 2 || C == 1 || blend_mode == BL_ADDITIVE || blend_mode == BL_ALPHA_ADDITIVE ||
                          ((blend_mode == BL_BEER_LAMBERT || blend_mode == BL_BEER_LAMBERT_EXCLUSIVE) &&
                           acc.v[C - 1] >= 0.f);
        int i_lo = 0, i_hi = D - 1;
        const bool hit = live && (!clip || ray_clip(nearp, step, D, din, i_lo, i_hi));
        k_lo = D - 1 - i_hi;
        k_hi = D - 1 - i_lo;
        warp_clip_range(hit, D, k_lo, k_hi, w_lo, w_hi);
    } else if (!live) {
        k_lo = D;
        k_hi = -1;
    }
    // Not unrolled: the step body is large, and unrolled copies stalled on
    // instruction fetch (unroll 2 / 4: 13 % / 36 % slower normalised pass at
    // 480x270x192; capping registers at 64 or 72 spilled and was slower too).
    // Stored samples: step k reads the forward's step i = D - 1 - k: zero
    // outside the forward's range or where the warp's ballot word for that
    // step has this lane's bit clear, else the stored sample (re-sampled where
    // the forward found the pool full).  (Words are only
    // read for steps inside the lane's own forward range, which the forward's
    // warp wrote; a warp's words of consecutive steps share a cache line.)
    const unsigned lane = (threadIdx.y * RM_BX + threadIdx.x) & 31u;
#pragma unroll 1
    for (int k = w_lo; k <= w_hi; ++k) {
        const bool on = k >= k_lo && k <= k_hi;
        const float3 pos = ray_sample(nearp, step, D - 1 - k);
        const float px = pos.x - 0.5f, py = pos.y - 0.5f, pz = pos.z - 0.5f;
        Vec<C> val = vfill<C>(1.f);
        if (MODE != 2 && on) {
            Vec<C> smp = vzero<C>();
            bool resample = !use_store;
            if (use_store) {
                const int i = D - 1 - k;
                if (i >= s_lo && i <= s_hi) {
                    const int64_t w = sample_word_index(tab, r.tile, p, D, i);
                    const uint32_t word = __ldg(st.words + w);
                    if ((word >> lane) & 1u) {
                        const uint32_t first = __ldg(st.first + w);
                        if (first != STORE_OVERFLOW)
                            smp = load_stream<C>(st.samples, (int64_t)(first + lane_rank(word, lane)));
                        else
                            resample = true;  // the pool was full: not stored
                    }
                }
            }
            if (resample) smp = fetch_linear<C, S, BM, L>(g, din, px, py, pz);
            val = blend_grad<C>(blend_mode, MODE == 0, go, smp, acc);
        }
        if constexpr (PROJ) {
            Vec<2> pv;
            pv.v[0] = pj.a[0] * val.v[0] + pj.a[1] * val.v[1] + pj.a[2] * val.v[2] + pj.a[3] * val.v[3];
            pv.v[1] = pj.b[0] * val.v[0] + pj.b[1] * val.v[1] + pj.b[2] * val.v[2] + pj.b[3] * val.v[3];
            scatter_step<2, BM, MODE, L, DET>(dst, count, din, on, px, py, pz, pv, idst, iscale, wdst);
        } else {
            scatter_step<C, BM, MODE, L, DET>(dst, count, din, on, px, py, pz, val, idst, iscale);
        }
    }
}

// At least 6 resident blocks per SM: the tile loop would otherwise take 90
// registers (5 blocks); with the bound it stays at the 80 of one tile per
// block, without spills.
template <int C, typename S, int BM, int MODE, int L, bool DET = false, bool PROJ = false>
__global__ void __launch_bounds__(RM_BX* RM_BY, 6)
    k_raymarch_scatter(const S* __restrict__ in, Dims din, int blend_mode, const float* __restrict__ out,
                       const float* __restrict__ dout, float* __restrict__ grad, const float* __restrict__ cnt,
                       unsigned long long* __restrict__ iacc, const float* __restrict__ iscale_ptr, float wscale,
                       const RaymarchArgs::Store st, const __grid_constant__ PairTable tab, const ChanProj pj) {
    // integer accumulation: MODE 2 with the host's weight scale, the adjoint
    // with the scale its bound kernel wrote
    const float iscale = !DET ? 0.f : MODE == 2 ? wscale : *iscale_ptr;
    const int tiles = tab.tile0[tab.n];
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x)
        raymarch_scatter_tile<C, S, BM, MODE, L, DET, PROJ>(in, din, blend_mode, out, dout, grad, cnt, iacc, iscale,
                                                             st, tab, tile, pj);
}

template <int C, typename S, int BM>
static void fwd_dispatch_lin(bool lin, dim3 grid, dim3 block, cudaStream_t s, const void* in, const RaymarchArgs& a,
                             float* out, const PairTable& t) {
    // the brick layout is produced for the LINEAR render path only
    if (a.layout == LAYOUT_BRICK)
        k_raymarch_fwd<C, S, BM, true, LAYOUT_BRICK><<<grid, block, 0, s>>>((const S*)in, a.din, a.filter, a.blend,
                                                                           out, a.store, t);
    else if (lin)
        k_raymarch_fwd<C, S, BM, true, LAYOUT_FLAT><<<grid, block, 0, s>>>((const S*)in, a.din, a.filter, a.blend,
                                                                          out, a.store, t);
    else
        k_raymarch_fwd<C, S, BM, false, LAYOUT_FLAT><<<grid, block, 0, s>>>((const S*)in, a.din, a.filter, a.blend,
                                                                           out, RaymarchArgs::Store{}, t);
}

template <int C, typename S>
static void fwd_dispatch_bm(dim3 grid, dim3 block, cudaStream_t s, const RaymarchArgs& a, float* out,
                            const PairTable& t) {
    const bool lin = a.filter == F_LINEAR;
    switch (a.boundary) {
        case BM_BORDER: fwd_dispatch_lin<C, S, BM_BORDER>(lin, grid, block, s, a.input, a, out, t); break;
        case BM_CLAMP: fwd_dispatch_lin<C, S, BM_CLAMP>(lin, grid, block, s, a.input, a, out, t); break;
        default: fwd_dispatch_lin<C, S, BM_WRAP>(lin, grid, block, s, a.input, a, out, t); break;
    }
}

bool launch_raymarch_fwd(const RaymarchArgs& a, const std::vector<Pair>& pairs, float* out, cudaStream_t s) {
    const dim3 block(RM_BX, RM_BY, 1);
    int64_t cells = 0;
    for (PairTable& t : make_tables(pairs)) {
        const dim3 grid(raymarch_blocks((int)set_ray_tiles(t, &cells)));
        if (a.dtype == 0) {
            if (a.C == 4) fwd_dispatch_bm<4, float>(grid, block, s, a, out, t);
            else if (a.C == 2) fwd_dispatch_bm<2, float>(grid, block, s, a, out, t);
            else fwd_dispatch_bm<1, float>(grid, block, s, a, out, t);
        } else {
            if (a.C == 4) fwd_dispatch_bm<4, __nv_bfloat16>(grid, block, s, a, out, t);
            else if (a.C == 2) fwd_dispatch_bm<2, __nv_bfloat16>(grid, block, s, a, out, t);
            else fwd_dispatch_bm<1, __nv_bfloat16>(grid, block, s, a, out, t);
        }
        if (!launched(1, "raymarch forward launch")) return false;
    }
    return true;
}

template <int C, typename S, int BM, int L>
static void bwd_dispatch_l(bool exact, dim3 grid, dim3 block, cudaStream_t s, const RaymarchArgs& a, const float* out,
                           const float* dout, float* grad, const float* cnt, const PairTable& t) {
    const ChanProj pj = a.proj;
    if constexpr (C == 4 && L == LAYOUT_BRICK) {
        if (a.project && a.camera_sums) {  // reference normalisation by per-camera sums
            k_raymarch_scatter<C, S, BM, 3, L, false, true><<<grid, block, 0, s>>>(
                (const S*)a.input, a.din, a.blend, out, dout, grad, cnt, nullptr, nullptr, 0.f, a.store, t, pj);
            return;
        }
        if (a.project && a.det) {
            if (exact)
                k_raymarch_scatter<C, S, BM, 0, L, true, true><<<grid, block, 0, s>>>(
                    (const S*)a.input, a.din, a.blend, out, dout, grad, cnt, a.det_acc, a.det_scale, 0.f, a.store, t,
                    pj);
            else
                k_raymarch_scatter<C, S, BM, 1, L, true, true><<<grid, block, 0, s>>>(
                    (const S*)a.input, a.din, a.blend, out, dout, grad, cnt, a.det_acc, a.det_scale, 0.f, a.store, t,
                    pj);
            return;
        }
        if (a.project) {
            if (exact)
                k_raymarch_scatter<C, S, BM, 0, L, false, true><<<grid, block, 0, s>>>(
                    (const S*)a.input, a.din, a.blend, out, dout, grad, cnt, nullptr, nullptr, 0.f, a.store, t, pj);
            else
                k_raymarch_scatter<C, S, BM, 1, L, false, true><<<grid, block, 0, s>>>(
                    (const S*)a.input, a.din, a.blend, out, dout, grad, cnt, nullptr, nullptr, 0.f, a.store, t, pj);
            return;
        }
    }
    if (a.det) {
        if (exact)
            k_raymarch_scatter<C, S, BM, 0, L, true><<<grid, block, 0, s>>>(
                (const S*)a.input, a.din, a.blend, out, dout, grad, cnt, a.det_acc, a.det_scale, 0.f, a.store, t, pj);
        else
            k_raymarch_scatter<C, S, BM, 1, L, true><<<grid, block, 0, s>>>(
                (const S*)a.input, a.din, a.blend, out, dout, grad, cnt, a.det_acc, a.det_scale, 0.f, a.store, t, pj);
    } else if (exact) {
        k_raymarch_scatter<C, S, BM, 0, L><<<grid, block, 0, s>>>((const S*)a.input, a.din, a.blend, out, dout, grad,
                                                                     cnt, nullptr, nullptr, 0.f, a.store, t, pj);
    } else {
        k_raymarch_scatter<C, S, BM, 1, L><<<grid, block, 0, s>>>((const S*)a.input, a.din, a.blend, out, dout, grad,
                                                                     cnt, nullptr, nullptr, 0.f, a.store, t, pj);
    }
}

template <int C, typename S, int BM>
static void bwd_dispatch(bool exact, dim3 grid, dim3 block, cudaStream_t s, const RaymarchArgs& a, const float* out,
                         const float* dout, float* grad, const float* cnt, const PairTable& t) {
    if (a.layout == LAYOUT_BRICK)
        bwd_dispatch_l<C, S, BM, LAYOUT_BRICK>(exact, grid, block, s, a, out, dout, grad, cnt, t);
    else
        bwd_dispatch_l<C, S, BM, LAYOUT_FLAT>(exact, grid, block, s, a, out, dout, grad, cnt, t);
}

template <int C, typename S>
static void bwd_dispatch_bm(bool exact, dim3 grid, dim3 block, cudaStream_t s, const RaymarchArgs& a,
                            const float* out, const float* dout, float* grad, const float* cnt, const PairTable& t) {
    switch (a.boundary) {
        case BM_BORDER: bwd_dispatch<C, S, BM_BORDER>(exact, grid, block, s, a, out, dout, grad, cnt, t); break;
        case BM_CLAMP: bwd_dispatch<C, S, BM_CLAMP>(exact, grid, block, s, a, out, dout, grad, cnt, t); break;
        default: bwd_dispatch<C, S, BM_WRAP>(exact, grid, block, s, a, out, dout, grad, cnt, t); break;
    }
}

template <int BM>
static void weights_dispatch(dim3 grid, dim3 block, cudaStream_t s, const RaymarchArgs& a, float* cnt,
                             unsigned long long* wacc, float wscale, const PairTable& t) {
    if (wacc != nullptr)
        k_raymarch_scatter<1, float, BM, 2, LAYOUT_FLAT, true><<<grid, block, 0, s>>>(
            nullptr, a.din, a.blend, nullptr, nullptr, cnt, nullptr, wacc, nullptr, wscale, RaymarchArgs::Store{}, t,
            ChanProj{});
    else
        k_raymarch_scatter<1, float, BM, 2, LAYOUT_FLAT><<<grid, block, 0, s>>>(
            nullptr, a.din, a.blend, nullptr, nullptr, cnt, nullptr, nullptr, nullptr, 0.f, RaymarchArgs::Store{}, t,
            ChanProj{});
}

// Weight sums -> their reciprocals (0 where no sample reached the voxel), 16
// bytes per access: the workspace is 16-byte aligned (checked at the C ABI)
// and holds brick_cells (a multiple of 8) floats per pair; n4 = floats / 4.
__device__ __forceinline__ float inv_or_zero(float v) { return v > 0.f ? 1.f / v : 0.f; }
__global__ void k_invert_weights(float4* __restrict__ w, int64_t n4) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
        float4 v = w[i];
        v.x = inv_or_zero(v.x);
        v.y = inv_or_zero(v.y);
        v.z = inv_or_zero(v.z);
        v.w = inv_or_zero(v.w);
        w[i] = v;
    }
}

// ---- deterministic adjoint (GFT_GRAD_DETERMINISTIC) ---------------------------------
// Every float reduction of the adjoint becomes an exact int64 sum of
// fixed-point contributions, so the gradient is the same bit for bit on every
// run.  The weight sums use a fixed point of scale 2^(61 - ceil(log2 of the
// largest sample count of a pair)): a voxel's weight sum never exceeds the
// number of samples, so no sum overflows.  The adjoint's scale comes from a
// bound on every voxel's partial sums, computed on the GPU from maxima (which
// do not depend on the order of evaluation): each sample's blend adjoint is at
// most B = max|dy| (ADDITIVE, or one channel) or, for BEER_LAMBERT with C > 1,
// max|dy| (1 + (C-1) D max|x|) (the density channel sums the later samples'
// light times the light adjoint, attenuated by exp(-density) <= 1); a voxel's
// reference-normalised gradient is a sum over cameras of weighted means of
// them (at most pairs * B) and its exact gradient at most B times its summed
// trilinear weights (at most pairs * the largest weight sum).  The scale is
// 2^(61 - ceil(log2 bound)), so no partial sum exceeds 2^61.
static int64_t det_weights_offset(int64_t cells, size_t pairs) {
    return (int64_t)align256u(sizeof(float) * cells * pairs);
}
size_t raymarch_det_bytes(int N, int C, Dims din, size_t pairs) {
    const int64_t cells = brick_cells(din);  // >= voxels: covers both layouts
    return (size_t)det_weights_offset(cells, pairs) + align256u(sizeof(unsigned long long) * cells * pairs) +
           align256u(sizeof(unsigned long long) * cells * (size_t)N * C) + 256;
}

// largest sample count of a pair -> fixed-point scale of the weight sums
static float det_weight_scale(const std::vector<Pair>& pairs, const RaymarchArgs& a) {
    double most = 1.0;
    for (const Pair& p : pairs) {
        const double n = (double)(p.W > 0 ? p.W : a.W) * (p.H > 0 ? p.H : a.H) * (p.D > 0 ? p.D : a.D);
        most = std::max(most, n);
    }
    const int e = (int)std::ceil(std::log2(most + 1.0));
    return std::ldexp(1.0f, 61 - e);
}

__global__ void k_det_invert_weights(const unsigned long long* __restrict__ wacc, float wscale, float* __restrict__ w,
                                     int64_t n, unsigned long long* __restrict__ wmax) {
    unsigned long long m = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long q = wacc[i];
        w[i] = q > 0 ? (float)((double)wscale / (double)q) : 0.f;
        m = q > m ? q : m;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_down_sync(0xffffffffu, m, o);
        m = t > m ? t : m;
    }
    if ((threadIdx.x & 31u) == 0 && m > 0) atomicMax(wmax, m);
}

// max |v| over n floats -> atomicMax on the bits (non-negative floats order like
// their bits; NaN compares above every finite value)
__device__ __forceinline__ void warp_absmax_to(unsigned int* out, float m) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31u) == 0) atomicMax(out, __float_as_uint(m));
}
__global__ void k_det_absmax(const float* __restrict__ v, int64_t n, unsigned int* __restrict__ out) {
    float m = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float x = fabsf(v[i]);
        m = (x > m || x != x) ? x : m;
    }
    warp_absmax_to(out, m);
}
// the input grid's voxels (not the brick padding), all channels
template <int C, typename S, int L>
__global__ void k_det_absmax_grid(const S* __restrict__ in, Dims d, int N, unsigned int* __restrict__ out) {
    float m = 0.f;
    const int64_t nv = voxels(d) * N;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = i / voxels(d);
        int x, y, z;
        unflat32((uint32_t)(i - b * voxels(d)), d, x, y, z);
        const Vec<C> a = Load<C, S>::at(in + (size_t)b * slice_cells<L>(d) * C, cell_index<L>(x, y, z, d));
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const float x2 = fabsf(a.v[c]);
            m = (x2 > m || x2 != x2) ? x2 : m;
        }
    }
    warp_absmax_to(out, m);
}
// bounds: [0] max|dy| bits, [1] max|x| bits; wmax: the largest integer weight
// sum (EXACT); scale <- 2^(61 - ceil(log2 bound)), NaN for a non-finite bound
// pfac: the accumulated values are projections sum_c p_c v_c of the channels
// (1 when they are the channels), at most pfac = max sum_c |p_c| times the
// channels' bound.
__global__ void k_det_scale(const unsigned int* __restrict__ bounds, const unsigned long long* __restrict__ wmax,
                            float wscale, int C, int D, int blend, int pairs, bool exact, float pfac,
                            float* __restrict__ scale) {
    const double dy = (double)__uint_as_float(bounds[0]), x = (double)__uint_as_float(bounds[1]);
    double b = dy;
    if (C > 1 && blend == BL_BEER_LAMBERT) b = dy * (1.0 + (double)(C - 1) * D * x);
    b *= (double)pfac;
    double f = (double)pairs;
    if (exact) f *= (double)(*wmax) / (double)wscale;
    const double t = b * f;
    float sc;
    if (!(t < 1e300)) {
        sc = __int_as_float(0x7fc00000);  // non-finite inputs: the gradient becomes NaN
    } else if (t <= 0.0) {
        sc = 1.f;
    } else {
        const int e = max(-60, (int)ceil(log2(t)));
        sc = ldexpf(1.f, 61 - e);
    }
    *scale = sc;
}
__global__ void k_det_convert(const unsigned long long* __restrict__ acc, const float* __restrict__ scale,
                              float* __restrict__ grad, int64_t n) {
    const double inv = 1.0 / (double)(*scale);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        grad[i] = (float)((double)(long long)acc[i] * inv);
}

static unsigned grid_stride_blocks(int64_t n) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8));
}

struct DetLayout {
    unsigned long long* wacc;
    unsigned long long* gacc;
    unsigned int* bounds;           // [0] max|dy| bits, [1] max|x| bits
    unsigned long long* wmax;       // largest weight sum
    float* scale;                   // the adjoint's fixed-point scale
};
static DetLayout det_layout(float* ws, const RaymarchArgs& a, size_t pairs) {
    const int64_t cells = brick_cells(a.din);
    char* base = reinterpret_cast<char*>(ws);
    DetLayout L;
    L.wacc = reinterpret_cast<unsigned long long*>(base + det_weights_offset(cells, pairs));
    char* g = reinterpret_cast<char*>(L.wacc) + align256u(sizeof(unsigned long long) * cells * pairs);
    L.gacc = reinterpret_cast<unsigned long long*>(g);
    char* t = g + align256u(sizeof(unsigned long long) * cells * (size_t)a.N * a.C);
    L.bounds = reinterpret_cast<unsigned int*>(t);
    L.wmax = reinterpret_cast<unsigned long long*>(t + 16);
    L.scale = reinterpret_cast<float*>(t + 32);
    return L;
}

// Pass 1 of the reference-normalised adjoint: per-pair weight sums into
// ws_cnt, inverted to reciprocals (deterministic: exact integer sums first,
// and the largest sum into the layout's wmax).
static bool raymarch_weights_impl(const RaymarchArgs& a, const std::vector<Pair>& pairs, float* ws_cnt, bool det,
                                  cudaStream_t s) {
    const int64_t cells = brick_cells(a.din);
    const int64_t n = cells * (int64_t)pairs.size();
    DetLayout L{};
    float wscale = 0.f;
    if (det) {
        L = det_layout(ws_cnt, a, pairs.size());
        wscale = det_weight_scale(pairs, a);
        if (!cuda_ok(cudaMemsetAsync(L.wacc, 0, sizeof(unsigned long long) * n, s), "zero weights") ||
            !cuda_ok(cudaMemsetAsync(L.wmax, 0, sizeof(unsigned long long), s), "zero weight max"))
            return false;
    } else if (!cuda_ok(cudaMemsetAsync(ws_cnt, 0, sizeof(float) * n, s), "zero weights")) {
        return false;
    }
    const dim3 block(RM_BX, RM_BY, 1);
    for (PairTable& t : make_tables(pairs)) {
        const dim3 grid(weights_blocks((int)set_ray_tiles(t)));
        switch (a.boundary) {
            case BM_BORDER: weights_dispatch<BM_BORDER>(grid, block, s, a, ws_cnt, L.wacc, wscale, t); break;
            case BM_CLAMP: weights_dispatch<BM_CLAMP>(grid, block, s, a, ws_cnt, L.wacc, wscale, t); break;
            default: weights_dispatch<BM_WRAP>(grid, block, s, a, ws_cnt, L.wacc, wscale, t); break;
        }
        if (!launched(1, "raymarch weight launch")) return false;
    }
    if (det) {
        k_det_invert_weights<<<grid_stride_blocks(n), 256, 0, s>>>(L.wacc, wscale, ws_cnt, n, L.wmax);
        return launched(1, "raymarch weight inversion launch");
    }
    const int64_t want = (n / 4 + 255) / 256;
    k_invert_weights<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sm_count() * 8)), 256, 0, s>>>(
        reinterpret_cast<float4*>(ws_cnt), n / 4);
    return launched(1, "raymarch weight inversion launch");
}

bool launch_raymarch_weights_det(const RaymarchArgs& a, const std::vector<Pair>& pairs, float* ws_cnt,
                                cudaStream_t s) {
    return raymarch_weights_impl(a, pairs, ws_cnt, true, s);
}

bool launch_raymarch_weights(const RaymarchArgs& a, const std::vector<Pair>& pairs, float* ws_cnt, cudaStream_t s) {
    return raymarch_weights_impl(a, pairs, ws_cnt, false, s);
}

template <int C, typename S, int L>
static void det_absmax_grid(const RaymarchArgs& a, unsigned int* out, cudaStream_t s) {
    k_det_absmax_grid<C, S, L><<<grid_stride_blocks(voxels(a.din) * a.N), 256, 0, s>>>((const S*)a.input, a.din, a.N,
                                                                                      out);
}

// ---- weight pass beside the scatter (GFT_KNOB_WEIGHTS_PIPELINE) ---------------------
// The reference-normalised adjoint needs each camera's weight sums before its
// scatter.  The weight pass is bound by instruction issue, the scatter by its
// L2 reductions, so they share the SMs well: the weight sums of camera k + 1
// are computed on a side stream while camera k scatters.  The side stream and
// its events belong to the library (one set per device); the side stream
// forks from and joins the caller's stream through events, which a CUDA-graph
// capture records as dependencies.
constexpr int PIPE_MAX_PAIRS = 64;
namespace {
struct SideStream {
    cudaStream_t st = nullptr;
    cudaEvent_t ev[PIPE_MAX_PAIRS + 1] = {};
};
std::mutex g_side_mu;
SideStream g_side[64];
}  // namespace

static SideStream* side_stream() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(g_side_mu);
    SideStream& ss = g_side[dev];
    if (ss.st == nullptr) {
        cudaStream_t st = nullptr;
        if (!cuda_ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "side stream")) return nullptr;
        for (int i = 0; i <= PIPE_MAX_PAIRS; ++i)
            if (!cuda_ok(cudaEventCreateWithFlags(&ss.ev[i], cudaEventDisableTiming), "side stream event"))
                return nullptr;
        ss.st = st;
    }
    return &ss;
}

bool prepare_side_stream() { return side_stream() != nullptr; }

// Pair k of a table as a one-pair table: same camera, image, output pixels
// and sample-store offset, its tiles numbered from 0.
static PairTable single_pair(const PairTable& t, int k) {
    PairTable u;
    std::memset(&u, 0, sizeof(u));
    u.cam[0] = t.cam[k];
    u.in_batch[0] = t.in_batch[k];
    u.out_slot[0] = t.out_slot[k];
    u.rw[0] = t.rw[k];
    u.rh[0] = t.rh[k];
    u.rd[0] = t.rd[k];
    u.pix0[0] = t.pix0[k];
    u.smp0[0] = t.smp0[k];
    u.tile0[0] = 0;
    u.tile0[1] = t.tile0[k + 1] - t.tile0[k];
    u.pair_base = t.pair_base + k;
    u.n = 1;
    return u;
}

static bool raymarch_bwd_pipelined(const RaymarchArgs& a, const std::vector<Pair>& pairs, const float* out,
                                   const float* dout, float* grad, float* ws_cnt, SideStream& ss, cudaStream_t s) {
    const int64_t cells = brick_cells(a.din);
    const dim3 block(RM_BX, RM_BY, 1);
    std::vector<PairTable> singles;
    int64_t smp_cells = 0;
    for (PairTable& t : make_tables(pairs)) {
        set_ray_tiles(t, &smp_cells);
        for (int k = 0; k < t.n; ++k) singles.push_back(single_pair(t, k));
    }
    if (!cuda_ok(cudaEventRecord(ss.ev[0], s), "fork") || !cuda_ok(cudaStreamWaitEvent(ss.st, ss.ev[0], 0), "fork") ||
        !cuda_ok(cudaMemsetAsync(ws_cnt, 0, sizeof(float) * cells * pairs.size(), ss.st), "zero weights"))
        return false;
    for (size_t k = 0; k < singles.size(); ++k) {
        const PairTable& u = singles[k];
        const dim3 grid(weights_blocks(u.tile0[1]));
        switch (a.boundary) {
            case BM_BORDER: weights_dispatch<BM_BORDER>(grid, block, ss.st, a, ws_cnt, nullptr, 0.f, u); break;
            case BM_CLAMP: weights_dispatch<BM_CLAMP>(grid, block, ss.st, a, ws_cnt, nullptr, 0.f, u); break;
            default: weights_dispatch<BM_WRAP>(grid, block, ss.st, a, ws_cnt, nullptr, 0.f, u); break;
        }
        const int64_t n4 = cells / 4;  // cells is a multiple of 8
        const int64_t want = (n4 + 255) / 256;
        k_invert_weights<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sm_count() * 8)), 256, 0,
                           ss.st>>>(reinterpret_cast<float4*>(ws_cnt + (size_t)u.pair_base * cells), n4);
        if (!launched(2, "raymarch weight launch") || !cuda_ok(cudaEventRecord(ss.ev[1 + k], ss.st), "weights event"))
            return false;
    }
    for (size_t k = 0; k < singles.size(); ++k) {
        const PairTable& u = singles[k];
        if (!cuda_ok(cudaStreamWaitEvent(s, ss.ev[1 + k], 0), "join")) return false;
        const dim3 grid(raymarch_blocks(u.tile0[1]));
        if (a.dtype == 0) {
            if (a.C == 4) bwd_dispatch_bm<4, float>(false, grid, block, s, a, out, dout, grad, ws_cnt, u);
            else if (a.C == 2) bwd_dispatch_bm<2, float>(false, grid, block, s, a, out, dout, grad, ws_cnt, u);
            else bwd_dispatch_bm<1, float>(false, grid, block, s, a, out, dout, grad, ws_cnt, u);
        } else {
            if (a.C == 4) bwd_dispatch_bm<4, __nv_bfloat16>(false, grid, block, s, a, out, dout, grad, ws_cnt, u);
            else if (a.C == 2) bwd_dispatch_bm<2, __nv_bfloat16>(false, grid, block, s, a, out, dout, grad, ws_cnt, u);
            else bwd_dispatch_bm<1, __nv_bfloat16>(false, grid, block, s, a, out, dout, grad, ws_cnt, u);
        }
        if (!launched(1, "raymarch backward launch")) return false;
    }
    return true;
}

bool launch_raymarch_bwd(const RaymarchArgs& a_in, const std::vector<Pair>& pairs, const float* out,
                         const float* dout, bool exact, bool weights_ready, float* grad, float* ws_cnt,
                         cudaStream_t s) {
    RaymarchArgs a = a_in;
    const int64_t cells = a.layout == LAYOUT_BRICK ? brick_cells(a.din) : voxels(a.din);
    const int64_t n = cells * (a.project ? 2 : a.C) * a.N;
    if (a.camera_sums) {
        // per pair: the projected value sums and the weight sums, both
        // accumulated from zero by one pass
        const size_t pn = (size_t)cells * 2 * pairs.size(), wn = (size_t)brick_cells(a.din) * pairs.size();
        if (!cuda_ok(cudaMemsetAsync(grad, 0, sizeof(float) * pn, s), "zero gradient") ||
            !cuda_ok(cudaMemsetAsync(ws_cnt, 0, sizeof(float) * wn, s), "zero weight sums"))
            return false;
        const dim3 block(RM_BX, RM_BY, 1);
        int64_t smp_cells = 0;
        for (PairTable& t : make_tables(pairs)) {
            const dim3 grid(raymarch_blocks((int)set_ray_tiles(t, &smp_cells)));
            if (a.dtype == 0) bwd_dispatch_bm<4, float>(false, grid, block, s, a, out, dout, grad, ws_cnt, t);
            else bwd_dispatch_bm<4, __nv_bfloat16>(false, grid, block, s, a, out, dout, grad, ws_cnt, t);
            if (!launched(1, "raymarch backward launch")) return false;
        }
        return true;
    }
    if (!a.det) {
        if (!cuda_ok(cudaMemsetAsync(grad, 0, sizeof(float) * n, s), "zero gradient")) return false;
        if (!exact && !weights_ready && knob_value(GFT_KNOB_WEIGHTS_PIPELINE) == 1 &&
            pairs.size() <= (size_t)PIPE_MAX_PAIRS) {
            SideStream* ss = side_stream();
            if (ss == nullptr) return false;
            return raymarch_bwd_pipelined(a, pairs, out, dout, grad, ws_cnt, *ss, s);
        }
        if (!exact && !weights_ready && !launch_raymarch_weights(a, pairs, ws_cnt, s)) return false;
    } else {
        // integer sums into gacc, then converted into grad
        const DetLayout L = det_layout(ws_cnt, a, pairs.size());
        if (!cuda_ok(cudaMemsetAsync(L.gacc, 0, sizeof(unsigned long long) * n, s), "zero gradient") ||
            !cuda_ok(cudaMemsetAsync(L.bounds, 0, 8, s), "zero bounds"))
            return false;
        // (with the weights ready: integer sums, reciprocals and their largest
        // sum from gft_raymarch_grid_transform_grad_weights_mode)
        if (!weights_ready && !raymarch_weights_impl(a, pairs, ws_cnt, true, s)) return false;
        int64_t pix = 0;
        int dmax = a.D;
        for (const Pair& p : pairs) {
            pix += (int64_t)(p.W > 0 ? p.W : a.W) * (p.H > 0 ? p.H : a.H);
            dmax = std::max(dmax, p.D);
        }
        k_det_absmax<<<grid_stride_blocks(pix * a.C), 256, 0, s>>>(dout, pix * a.C, L.bounds);
        const bool brick = a.layout == LAYOUT_BRICK;
        if (a.dtype == 0) {
            if (a.C == 4) brick ? det_absmax_grid<4, float, LAYOUT_BRICK>(a, L.bounds + 1, s) : det_absmax_grid<4, float, LAYOUT_FLAT>(a, L.bounds + 1, s);
            else if (a.C == 2) brick ? det_absmax_grid<2, float, LAYOUT_BRICK>(a, L.bounds + 1, s) : det_absmax_grid<2, float, LAYOUT_FLAT>(a, L.bounds + 1, s);
            else brick ? det_absmax_grid<1, float, LAYOUT_BRICK>(a, L.bounds + 1, s) : det_absmax_grid<1, float, LAYOUT_FLAT>(a, L.bounds + 1, s);
        } else {
            if (a.C == 4) brick ? det_absmax_grid<4, __nv_bfloat16, LAYOUT_BRICK>(a, L.bounds + 1, s) : det_absmax_grid<4, __nv_bfloat16, LAYOUT_FLAT>(a, L.bounds + 1, s);
            else if (a.C == 2) brick ? det_absmax_grid<2, __nv_bfloat16, LAYOUT_BRICK>(a, L.bounds + 1, s) : det_absmax_grid<2, __nv_bfloat16, LAYOUT_FLAT>(a, L.bounds + 1, s);
            else brick ? det_absmax_grid<1, __nv_bfloat16, LAYOUT_BRICK>(a, L.bounds + 1, s) : det_absmax_grid<1, __nv_bfloat16, LAYOUT_FLAT>(a, L.bounds + 1, s);
        }
        float pfac = 1.f;
        if (a.project) {
            float sa = 0.f, sb = 0.f;
            for (int c = 0; c < 4; ++c) {
                sa += std::fabs(a.proj.a[c]);
                sb += std::fabs(a.proj.b[c]);
            }
            pfac = std::max(sa, sb);
        }
        k_det_scale<<<1, 1, 0, s>>>(L.bounds, L.wmax, det_weight_scale(pairs, a), a.C, dmax, a.blend, (int)pairs.size(),
                                    exact, pfac, L.scale);
        if (!launched(3, "deterministic bound launch")) return false;
        a.det_acc = L.gacc;
        a.det_scale = L.scale;
    }
    const dim3 block(RM_BX, RM_BY, 1);
    int64_t smp_cells = 0;
    for (PairTable& t : make_tables(pairs)) {
        const dim3 grid(raymarch_blocks((int)set_ray_tiles(t, &smp_cells)));
        if (a.dtype == 0) {
            if (a.C == 4) bwd_dispatch_bm<4, float>(exact, grid, block, s, a, out, dout, grad, ws_cnt, t);
            else if (a.C == 2) bwd_dispatch_bm<2, float>(exact, grid, block, s, a, out, dout, grad, ws_cnt, t);
            else bwd_dispatch_bm<1, float>(exact, grid, block, s, a, out, dout, grad, ws_cnt, t);
        } else {
            if (a.C == 4) bwd_dispatch_bm<4, __nv_bfloat16>(exact, grid, block, s, a, out, dout, grad, ws_cnt, t);
            else if (a.C == 2) bwd_dispatch_bm<2, __nv_bfloat16>(exact, grid, block, s, a, out, dout, grad, ws_cnt, t);
            else bwd_dispatch_bm<1, __nv_bfloat16>(exact, grid, block, s, a, out, dout, grad, ws_cnt, t);
        }
        if (!launched(1, "raymarch backward launch")) return false;
    }
    if (a.det) {
        k_det_convert<<<grid_stride_blocks(n), 256, 0, s>>>(a.det_acc, a.det_scale, grad, n);
        return launched(1, "deterministic gradient conversion launch");
    }
    return true;
}

}  // namespace gft
