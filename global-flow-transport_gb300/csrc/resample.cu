// Resampling ops: mip pyramid, SampleGridTransform (+ scatter adjoint),
// SampleGridLut (+ adjoint) and LodTransform.
//
// Semantics: resample_grid.cu.cc (kGenerateMip3D :46-72, kSample3D :240-252,
// kSampleGrid3DLuT :465-484, kScatter3DGradients :841-861,
// kScatterLuT3DGradients :1051-1081, kComputeLoD3D :1288-1300) and the
// sampler of sampling.hpp.  All cameras of a batch slice run in one launch;
// per-camera transforms travel in the launch parameters.
#include <algorithm>

#include <cmath>

#include "gft_internal.h"

namespace gft {

constexpr int RS_THREADS = 256;

// ---- mips --------------------------------------------------------------------
// Level m+1 = 2x2x2 mean of level m, dims >> 1, averaging z pairs, then y, then
// x as kGenerateMip3D does.
template <int C, typename S>
__global__ void k_mip_level(const S* __restrict__ src, Dims ds, float* __restrict__ dst, Dims dd) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= voxels(dd)) return;
    int x, y, z;
    unflat32(t, dd, x, y, z);
    Vec<C> c[2];
#pragma unroll
    for (int dx = 0; dx < 2; ++dx) {
        const int sx = 2 * x + dx;
        const Vec<C> a = vscale(vadd(Load<C, S>::at(src, flat3(sx, 2 * y, 2 * z, ds)),
                                     Load<C, S>::at(src, flat3(sx, 2 * y, 2 * z + 1, ds))), 0.5f);
        const Vec<C> b = vscale(vadd(Load<C, S>::at(src, flat3(sx, 2 * y + 1, 2 * z, ds)),
                                     Load<C, S>::at(src, flat3(sx, 2 * y + 1, 2 * z + 1, ds))), 0.5f);
        c[dx] = vscale(vadd(a, b), 0.5f);
    }
    store<C>(dst, t, vscale(vadd(c[0], c[1]), 0.5f));
}

// The 2x2x2 mean of kGenerateMip3D in its operation order (z pairs, then y,
// then x); at(dx, dy, dz) reads a child.
template <int C, typename F>
__device__ __forceinline__ Vec<C> mip_mean(F at) {
    Vec<C> c[2];
#pragma unroll
    for (int dx = 0; dx < 2; ++dx) {
        const Vec<C> a = vscale(vadd(at(dx, 0, 0), at(dx, 0, 1)), 0.5f);
        const Vec<C> b = vscale(vadd(at(dx, 1, 0), at(dx, 1, 1)), 0.5f);
        c[dx] = vscale(vadd(a, b), 0.5f);
    }
    return vscale(vadd(c[0], c[1]), 0.5f);
}

// Levels 1 to `levels` (<= 3) in one launch: a block of 64 threads computes a
// 4x4x4 tile of level 1 (from an 8x8x8 region of level 0), then from that tile
// in shared memory the 2x2x2 level-2 cells and the level-3 cell above it; a
// parent exists exactly where its children do (dims >> 1 per level).
template <int C, typename S>
__global__ void __launch_bounds__(64)
    k_mip_pyramid(const S* __restrict__ src, Dims d0, float* __restrict__ l1, Dims d1, float* __restrict__ l2, Dims d2,
                  float* __restrict__ l3, Dims d3, int levels) {
    __shared__ float s1[64 * C];
    __shared__ float s2[8 * C];
    const unsigned tx = (d1.x + 3) / 4, ty = (d1.y + 3) / 4;
    unsigned b = blockIdx.x;
    const int bx = (int)(b % tx);
    b /= tx;
    const int by = (int)(b % ty), bz = (int)(b / ty);
    const int t = threadIdx.x, lx = t & 3, ly = (t >> 2) & 3, lz = t >> 4;
    const int x = bx * 4 + lx, y = by * 4 + ly, z = bz * 4 + lz;
    Vec<C> v = vzero<C>();
    if (x < d1.x && y < d1.y && z < d1.z) {
        v = mip_mean<C>([&](int dx, int dy, int dz) {
            return Load<C, S>::at(src, flat3(2 * x + dx, 2 * y + dy, 2 * z + dz, d0));
        });
        store<C>(l1, flat3(x, y, z, d1), v);
    }
    if (levels < 2) return;  // uniform over the launch
#pragma unroll
    for (int c = 0; c < C; ++c) s1[t * C + c] = v.v[c];
    __syncthreads();
    if (t < 8) {
        const int cx = t & 1, cy = (t >> 1) & 1, cz = t >> 2;
        const int x2 = bx * 2 + cx, y2 = by * 2 + cy, z2 = bz * 2 + cz;
        Vec<C> v2 = vzero<C>();
        if (x2 < d2.x && y2 < d2.y && z2 < d2.z) {
            v2 = mip_mean<C>([&](int dx, int dy, int dz) {
                Vec<C> r;
                const int k = ((2 * cz + dz) * 4 + 2 * cy + dy) * 4 + 2 * cx + dx;
#pragma unroll
                for (int c = 0; c < C; ++c) r.v[c] = s1[k * C + c];
                return r;
            });
            store<C>(l2, flat3(x2, y2, z2, d2), v2);
        }
#pragma unroll
        for (int c = 0; c < C; ++c) s2[t * C + c] = v2.v[c];
    }
    if (levels < 3) return;
    __syncthreads();
    if (t == 0 && bx < d3.x && by < d3.y && bz < d3.z) {
        const Vec<C> v3 = mip_mean<C>([&](int dx, int dy, int dz) {
            Vec<C> r;
            const int k = (dz * 2 + dy) * 2 + dx;
#pragma unroll
            for (int c = 0; c < C; ++c) r.v[c] = s2[k * C + c];
            return r;
        });
        store<C>(l3, flat3(bx, by, bz, d3), v3);
    }
}

int usable_mip_levels(Dims d, int num_mips) {
    int L = num_mips < 0 ? 0 : num_mips;
    if (L > MAX_MIPS) L = MAX_MIPS;
    for (int m = 1; m <= L; ++m) {
        if ((int64_t)(d.x >> m) * (d.y >> m) * (d.z >> m) <= 0) return m - 1;
    }
    return L;
}

size_t mip_workspace_floats(Dims d, int levels, int C) {
    size_t n = 0;
    for (int m = 1; m <= levels; ++m) {
        const size_t v = (size_t)(d.x >> m) * (d.y >> m) * (d.z >> m) * C;
        n += (v + 63) & ~size_t(63);  // 256 B aligned levels
    }
    return n;
}

template <int C>
static void mip_launch(const void* src, int dtype, Dims ds, float* dst, Dims dd, cudaStream_t s) {
    const int64_t n = voxels(dd);
    const unsigned blocks = (unsigned)((n + RS_THREADS - 1) / RS_THREADS);
    if (dtype == 0)
        k_mip_level<C, float><<<blocks, RS_THREADS, 0, s>>>((const float*)src, ds, dst, dd);
    else
        k_mip_level<C, __nv_bfloat16><<<blocks, RS_THREADS, 0, s>>>((const __nv_bfloat16*)src, ds, dst, dd);
}

// The per-cell kernels index one grid slice with 32-bit arithmetic.
static bool slice_ok(int64_t cells) {
    if (cells < MAX_SLICE_CELLS) return true;
    set_error("a grid slice has 2^32 or more cells");
    return false;
}

bool launch_build_mips(const void* input, int dtype, int C, Dims d, int levels, float* ws, cudaStream_t s,
                       MipSet* set) {
    if (!slice_ok(voxels(d))) return false;
    set->levels = levels;
    set->lvl[0] = (const float*)input;  // reinterpreted by the sampler according to dtype
    set->dims[0] = d;
    float* p = ws;
    for (int m = 1; m <= levels; ++m) {  // level pointers and dims
        const Dims dm{d.x >> m, d.y >> m, d.z >> m};
        set->lvl[m] = p;
        set->dims[m] = dm;
        const size_t v = (size_t)voxels(dm) * C;
        p += (v + 63) & ~size_t(63);
    }
    // levels 1-3 in one launch, further levels one launch each
    const int first = std::min(levels, 3);
    if (first > 0) {
        const Dims d1 = set->dims[1], d2 = set->dims[std::min(first, 2)], d3 = set->dims[first];
        const int64_t blocks = (int64_t)((d1.x + 3) / 4) * ((d1.y + 3) / 4) * ((d1.z + 3) / 4);
        float* l1 = const_cast<float*>(set->lvl[1]);
        float* l2 = const_cast<float*>(set->lvl[std::min(first, 2)]);
        float* l3 = const_cast<float*>(set->lvl[first]);
        if (dtype == 0) {
            if (C == 4) k_mip_pyramid<4, float><<<(unsigned)blocks, 64, 0, s>>>((const float*)input, d, l1, d1, l2, d2, l3, d3, first);
            else if (C == 2) k_mip_pyramid<2, float><<<(unsigned)blocks, 64, 0, s>>>((const float*)input, d, l1, d1, l2, d2, l3, d3, first);
            else k_mip_pyramid<1, float><<<(unsigned)blocks, 64, 0, s>>>((const float*)input, d, l1, d1, l2, d2, l3, d3, first);
        } else {
            const __nv_bfloat16* in = (const __nv_bfloat16*)input;
            if (C == 4) k_mip_pyramid<4, __nv_bfloat16><<<(unsigned)blocks, 64, 0, s>>>(in, d, l1, d1, l2, d2, l3, d3, first);
            else if (C == 2) k_mip_pyramid<2, __nv_bfloat16><<<(unsigned)blocks, 64, 0, s>>>(in, d, l1, d1, l2, d2, l3, d3, first);
            else k_mip_pyramid<1, __nv_bfloat16><<<(unsigned)blocks, 64, 0, s>>>(in, d, l1, d1, l2, d2, l3, d3, first);
        }
        if (!launched(1, "mip pyramid launch")) return false;
    }
    for (int m = 4; m <= levels; ++m) {
        const Dims dm{d.x >> m, d.y >> m, d.z >> m};
        float* dst = const_cast<float*>(set->lvl[m]);
        if (C == 4) mip_launch<4>(set->lvl[m - 1], 0, set->dims[m - 1], dst, dm, s);
        else if (C == 2) mip_launch<2>(set->lvl[m - 1], 0, set->dims[m - 1], dst, dm, s);
        else mip_launch<1>(set->lvl[m - 1], 0, set->dims[m - 1], dst, dm, s);
        if (!launched(1, "mip generation launch")) return false;
    }
    return true;
}

// ---- occupancy of a sampled grid -------------------------------------------------
// A transform-mode sample at level-0 position p reads, at mip level m, the
// level-m cells around p * 2^-m, i.e. level-0 voxels within 1.5 * 2^m of p;
// with the floor of the folded position (a few ulp from the exact one) and
// up to L levels, within 1.5 * 2^L + 3 voxels of floor(p).  Under CLAMP a
// position beyond the grid reads the clamped border cells of level m, at most
// 2^(m+1) - 2 voxels from the clamped floor position (level dims = dims >> m).
// So every voxel read lies within R = max(1.5 * 2^L + 3, 2^(L+1)) voxels of
// the clamped floor(p).  A block's grown flag ORs the raw flags of the blocks
// within ceil(R / 8) blocks, so 0 means that every sample with its clamped
// floor position in the block reads zeros at every level: exactly zero.
__host__ __device__ inline int occupancy_radius_blocks(int levels) {
    const int R = max((3 << levels) / 2 + 3, 2 << levels);
    return (R + (1 << OCC_BLOCK_SHIFT) - 1) >> OCC_BLOCK_SHIFT;
}
static Dims occ_block_dims(Dims d) {
    const int b = 1 << OCC_BLOCK_SHIFT;
    return Dims{(d.x + b - 1) / b, (d.y + b - 1) / b, (d.z + b - 1) / b};
}
size_t occupancy_bytes(Dims d) { return 2 * (((size_t)voxels(occ_block_dims(d)) + 255) & ~size_t(255)); }

// Raw flags: one thread per 8-voxel x-run of a block row (coalesced reads,
// one flag store per run with a non-zero voxel).
template <int C, typename S>
__global__ void k_occupancy_raw(const S* __restrict__ g, Dims d, uint8_t* __restrict__ raw, Dims od) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t runs = (uint32_t)od.x * d.y * d.z;
    if (t >= runs) return;
    const int bx = (int)(t % (uint32_t)od.x);
    const uint32_t r = t / (uint32_t)od.x;  // z * H + y
    const int y = (int)(r % (uint32_t)d.y), z = (int)(r / (uint32_t)d.y);
    const int x0 = bx << OCC_BLOCK_SHIFT, x1 = min(x0 + (1 << OCC_BLOCK_SHIFT), d.x);
    bool nonzero = false;
    for (int x = x0; x < x1; ++x) {
        const Vec<C> a = Load<C, S>::at(g, (int64_t)r * d.x + x);
#pragma unroll
        for (int c = 0; c < C; ++c) nonzero = nonzero || a.v[c] != 0.f;  // NaN counts as non-zero
    }
    if (nonzero) raw[((size_t)(z >> OCC_BLOCK_SHIFT) * od.y + (y >> OCC_BLOCK_SHIFT)) * od.x + bx] = 1;
}

// Grown flags: one thread per block ORs the raw flags within rb blocks (RB: rb
// known at compile time, the loads of a row independent; 0: any rb).
template <int RB>
__global__ void __launch_bounds__(64) k_occupancy_grow(const uint8_t* __restrict__ raw, Dims od, int rb,
                                                       uint8_t* __restrict__ grown) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= voxels(od)) return;
    int x, y, z;
    unflat32(v, od, x, y, z);
    const int r = RB > 0 ? RB : rb;
    unsigned any = 0;
    for (int k = max(z - r, 0); k <= min(z + r, od.z - 1); ++k)
        for (int j = max(y - r, 0); j <= min(y + r, od.y - 1); ++j) {
            const uint8_t* row = raw + ((size_t)k * od.y + j) * od.x;
            if constexpr (RB > 0) {
#pragma unroll
                for (int o = -RB; o <= RB; ++o) {
                    const int i = x + o;
                    if (i >= 0 && i < od.x) any |= __ldg(row + i);
                }
            } else {
                for (int i = max(x - r, 0); i <= min(x + r, od.x - 1); ++i) any |= __ldg(row + i);
            }
        }
    grown[v] = any != 0;
}

template <int C, typename S>
static void occ_raw_launch(const void* input, Dims d, uint8_t* raw, Dims od, cudaStream_t s) {
    const int64_t runs = (int64_t)od.x * d.y * d.z;
    k_occupancy_raw<C, S><<<(unsigned)((runs + 255) / 256), 256, 0, s>>>((const S*)input, d, raw, od);
}

bool launch_occupancy(const void* input, int dtype, int C, Dims d, int levels, uint8_t* raw, uint8_t* grown,
                      cudaStream_t s, MipSet* set) {
    const Dims od = occ_block_dims(d);
    const int64_t nb = voxels(od);
    if (!cuda_ok(cudaMemsetAsync(raw, 0, (size_t)nb, s), "zero occupancy")) return false;
    if (dtype == 0) {
        if (C == 4) occ_raw_launch<4, float>(input, d, raw, od, s);
        else if (C == 2) occ_raw_launch<2, float>(input, d, raw, od, s);
        else occ_raw_launch<1, float>(input, d, raw, od, s);
    } else {
        if (C == 4) occ_raw_launch<4, __nv_bfloat16>(input, d, raw, od, s);
        else if (C == 2) occ_raw_launch<2, __nv_bfloat16>(input, d, raw, od, s);
        else occ_raw_launch<1, __nv_bfloat16>(input, d, raw, od, s);
    }
    const int rb = occupancy_radius_blocks(levels);
    const unsigned gb = (unsigned)((nb + 63) / 64);
    if (rb == 1) k_occupancy_grow<1><<<gb, 64, 0, s>>>(raw, od, rb, grown);
    else if (rb == 2) k_occupancy_grow<2><<<gb, 64, 0, s>>>(raw, od, rb, grown);
    else k_occupancy_grow<0><<<gb, 64, 0, s>>>(raw, od, rb, grown);
    if (!launched(2, "occupancy launch")) return false;
    set->occ = grown;
    set->occ_dims = od;
    return true;
}

// Sampler2::sample3D / Sampling::sample3D with mips (sampling.hpp:551-620, 690-712).
// Level 0 is read with the storage type S, coarser levels are fp32.
template <int C, typename S, int BM>
__device__ __forceinline__ Vec<C> read_level(int filter, const MipSet& ms, int m, float3 p, float cco) {
    const float inv = __int_as_float((127 - m) << 23);  // 2^-m: the product rounds exactly as p / 2^m
    const float px = p.x * inv - cco, py = p.y * inv - cco, pz = p.z * inv - cco;
    if (m == 0) return fetch<C, S, BM, false>(filter, reinterpret_cast<const S*>(ms.lvl[0]), ms.dims[0], px, py, pz);
    return fetch<C, float, BM, false>(filter, ms.lvl[m], ms.dims[m], px, py, pz);
}

template <int C, typename S, int BM>
__device__ __forceinline__ Vec<C> sample_mip(int filter, int mip_mode, const MipSet& ms, float4 pos, float bias,
                                             float cco) {
    const float3 p = make_float3(pos.x, pos.y, pos.z);
    if (mip_mode == MIP_NONE) return read_level<C, S, BM>(filter, ms, 0, p, cco);
    const int L = ms.levels;
    const float lod = fminf(fmaxf(pos.w + bias, 0.f), (float)L);
    const int lf = min((int)(lod + (mip_mode == MIP_NEAREST ? 0.5f : 0.f)), L);
    Vec<C> data = read_level<C, S, BM>(filter, ms, lf, p, cco);
    if (mip_mode == MIP_LINEAR) {
        const int lc = min((int)ceilf(lod), L);
        if (lc > lf) data = vlerp(data, read_level<C, S, BM>(filter, ms, lc, p, cco), lod - floorf(lod));
    }
    return data;
}

// ---- SampleGridTransform -------------------------------------------------------
constexpr int CM_LINDEPTH = 0, CM_LINDEPTH_REVERSE = 1, CM_TRANSFORM = 3, CM_TRANSFORM_REVERSE = 4;

__device__ __forceinline__ float3 map_pos(const CamX& c, int cm, float3 idx, float3 din, float3 dout_inv) {
    switch (cm) {
        case CM_LINDEPTH: return idx_to_os_lindepth(c, idx, dout_inv);
        case CM_TRANSFORM: return idx_to_os(c, idx, dout_inv);
        case CM_LINDEPTH_REVERSE: return os_to_idx_lindepth(c, idx, din);
        default: return os_to_idx(c, idx, din);
    }
}

// samplePos3D<CM, MIP> (sampling.hpp:58-136): position and LOD from forward
// differences; forward modes use Jacobian rows, reverse modes its columns.
// The position follows the reference's operation sequence.  For the LOD the
// neighbours idx + e_x, e_y, e_z differ from idx by a constant step in the
// folded homogeneous coordinates (for the linear-depth z, by a step of NDC z
// alone), so each costs a column add and a reciprocal instead of a transform;
// the differences are taken between folded positions.
//
// outside_zero: the caller's samples are zero at every mip level outside
// 0 <= p < din (LINEAR under BORDER with a half-cell centre offset: level m
// reads p * 2^-m, exactly, inside [0, (din >> m) * 2^m)), so there the LOD,
// which cannot change the result, is not computed.
template <int CM>
__device__ __forceinline__ bool skip_lod(float3 p, float3 din, bool outside_zero) {
    return outside_zero && !(p.x >= 0.f && p.x < din.x && p.y >= 0.f && p.y < din.y && p.z >= 0.f && p.z < din.z);
}

// Homogeneous divide for the LOD's finite differences (and the folded
// position of the outside test): the fast reciprocal intrinsic, whose error of
// a few ulp is far below the differences taken.
__device__ __forceinline__ float3 dehom_lod(float4 h) {
    const float iw = __fdividef(1.f, h.w);
    return make_float3(h.x * iw, h.y * iw, h.z * iw);
}

// With an occupancy map (forward modes): a sample whose clamped floor
// position lies in an empty grown block reads only zeros at every level and is
// returned with w = -1 (exactly zero, no position, LOD or fetch needed).
template <int CM>
__device__ __forceinline__ float4 sample_pos_cm(const CamX& c, float3 idx, float3 din, float3 dout_inv, bool lod,
                                                bool outside_zero = false, const uint8_t* occ = nullptr,
                                                Dims od = Dims{0, 0, 0}) {
    float3 p, f, ex, ey, ez;
    if constexpr (CM == CM_TRANSFORM || CM == CM_LINDEPTH) {
        float4 ndc = idx_to_ndc(idx, dout_inv);
        if (CM == CM_LINDEPTH) ndc.z = lindepth_ndc_z(c, idx.z, dout_inv.z);
        const float4 h = mul(c.q, ndc);
        f = dehom_lod(h);
        if (outside_zero) {
            // The folded position differs from the exact one by rounding only:
            // half a cell (plus 1e-3 relative) outside the domain, the exact one
            // is outside too and every level samples zero, so it is not needed.
            const float m = 0.5f + 1e-3f * fmaxf(fabsf(f.x), fmaxf(fabsf(f.y), fabsf(f.z)));
            if (f.x <= -m || f.x >= din.x + m || f.y <= -m || f.y >= din.y + m || f.z <= -m || f.z >= din.z + m)
                return make_float4(f.x, f.y, f.z, 0.f);
        }
        if (occ != nullptr && fabsf(f.x) <= 3.0e9f && fabsf(f.y) <= 3.0e9f && fabsf(f.z) <= 3.0e9f) {
            const int bx = min(max((int)floorf(f.x), 0), (int)din.x - 1) >> OCC_BLOCK_SHIFT;
            const int by = min(max((int)floorf(f.y), 0), (int)din.y - 1) >> OCC_BLOCK_SHIFT;
            const int bz = min(max((int)floorf(f.z), 0), (int)din.z - 1) >> OCC_BLOCK_SHIFT;
            if (__ldg(occ + ((size_t)bz * od.y + by) * od.x + bx) == 0) return make_float4(f.x, f.y, f.z, -1.f);
        }
        p = CM == CM_TRANSFORM ? idx_to_os(c, idx, dout_inv) : idx_to_os_lindepth(c, idx, dout_inv);
        if (!lod || skip_lod<CM>(p, din, outside_zero)) return make_float4(p.x, p.y, p.z, 0.f);
        const float dz = CM == CM_TRANSFORM ? 2.f * dout_inv.z : lindepth_ndc_z(c, idx.z + 1.f, dout_inv.z) - ndc.z;
        ex = dehom_lod(add_col<0>(h, c.q, 2.f * dout_inv.x));
        ey = dehom_lod(add_col<1>(h, c.q, 2.f * dout_inv.y));
        ez = dehom_lod(add_col<2>(h, c.q, dz));
    } else {
        constexpr bool LIN = CM == CM_LINDEPTH_REVERSE;
        p = LIN ? os_to_idx_lindepth(c, idx, din) : os_to_idx(c, idx, din);
        if (!lod || skip_lod<CM>(p, din, outside_zero)) return make_float4(p.x, p.y, p.z, 0.f);
        const float4 h = mul(c.r, make_float4(idx.x, idx.y, idx.z, 1.f));
        f = ndc_to_idx<LIN>(c, dehom_lod(h), din);
        ex = ndc_to_idx<LIN>(c, dehom_lod(add_col<0>(h, c.r, 1.f)), din);
        ey = ndc_to_idx<LIN>(c, dehom_lod(add_col<1>(h, c.r, 1.f)), din);
        ez = ndc_to_idx<LIN>(c, dehom_lod(add_col<2>(h, c.r, 1.f)), din);
    }
    const float3 dx = make_float3(f.x - ex.x, f.y - ex.y, f.z - ex.z);
    const float3 dy = make_float3(f.x - ey.x, f.y - ey.y, f.z - ey.z);
    const float3 dz = make_float3(f.x - ez.x, f.y - ez.y, f.z - ez.z);
    // lod = log2 of the largest per-axis step length = half the log2 of the
    // largest squared length (no square roots); the fast log2 intrinsic
    float qx, qy, qz;
    if constexpr (CM == CM_LINDEPTH || CM == CM_TRANSFORM) {
        qx = dx.x * dx.x + dy.x * dy.x + dz.x * dz.x;
        qy = dx.y * dx.y + dy.y * dy.y + dz.y * dz.y;
        qz = dx.z * dx.z + dy.z * dy.z + dz.z * dz.z;
    } else {
        qx = dx.x * dx.x + dx.y * dx.y + dx.z * dx.z;
        qy = dy.x * dy.x + dy.y * dy.y + dy.z * dy.z;
        qz = dz.x * dz.x + dz.y * dz.y + dz.z * dz.z;
    }
    const float qm = fmaxf(qx, fmaxf(qy, qz));
    return make_float4(p.x, p.y, p.z, fmaxf(0.f, 0.5f * __log2f(qm)));
}

__device__ __forceinline__ float4 sample_pos(const CamX& c, int cm, float3 idx, float3 din, float3 dout_inv,
                                             bool lod, bool outside_zero = false) {
    switch (cm) {
        case CM_LINDEPTH: return sample_pos_cm<CM_LINDEPTH>(c, idx, din, dout_inv, lod, outside_zero);
        case CM_TRANSFORM: return sample_pos_cm<CM_TRANSFORM>(c, idx, din, dout_inv, lod, outside_zero);
        case CM_LINDEPTH_REVERSE: return sample_pos_cm<CM_LINDEPTH_REVERSE>(c, idx, din, dout_inv, lod, outside_zero);
        default: return sample_pos_cm<CM_TRANSFORM_REVERSE>(c, idx, din, dout_inv, lod, outside_zero);
    }
}

// One kernel per coordinate mode (the transform and its LOD are inlined for
// that mode only).  The transform sampler reads nothing under WRAP, as the
// reference's (zeros for any coordinate mode).
// lod: the sample's LOD is computed (mip modes, unless the host proved it
// zero for every sample of the launch, reverse_lod_zero).
template <int C, typename S, int BM, int CM>
__global__ void __launch_bounds__(RS_THREADS)
    k_sample_transform(Dims dout, int filter, int mip_mode, bool lod, float bias, float cco, const MipSet ms,
                       float* __restrict__ out, const __grid_constant__ PairTable tab) {
    const int64_t nv = voxels(dout);
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const int p = blockIdx.y;
    Vec<C> r = vzero<C>();
    if constexpr (BM == BM_BORDER || BM == BM_CLAMP) {
        int x, y, z;
        unflat32(v, dout, x, y, z);
        const float3 din = make_float3((float)ms.dims[0].x, (float)ms.dims[0].y, (float)ms.dims[0].z);
        const float3 dinv = make_float3(1.f / (float)dout.x, 1.f / (float)dout.y, 1.f / (float)dout.z);
        const float4 pos = sample_pos_cm<CM>(tab.cam[p], make_float3(x + 0.5f, y + 0.5f, z + 0.5f), din, dinv,
                                             lod,
                                             BM == BM_BORDER && filter == F_LINEAR && cco == 0.5f, ms.occ,
                                             ms.occ_dims);
        if ((filter == F_LINEAR || filter == F_NEAREST) && !(pos.w < 0.f))
            r = sample_mip<C, S, BM>(filter, mip_mode, ms, pos, bias, cco);
    }
    store<C>(out, (int64_t)tab.out_slot[p] * nv + v, r);
}

// The reverse modes (volume -> frustum grid) sample the frustum grid at
// each volume voxel with the LOD of one voxel step measured in frustum cells
// (the largest squared step length qm; LOD = max(0, log2(qm) / 2)).  Each
// component of the map is scale * N / D + const with N and D affine in the
// voxel position, so its derivative along axis k is scale * (N_k D - N D_k)
// / D^2, whose numerator is affine: over a box its magnitude is at most the
// largest |numerator| at the box's corners over the smallest D^2 there (D
// keeping one sign).  The positions of the voxels and of their steps,
// [0.5, n + 0.5] per axis, are cut into 8^3 boxes; a step along k is at most
// the largest of these bounds per component.  If the squared length so
// bounded stays below 0.98 (the rest absorbs the float rounding of the
// kernel's differences) for every axis and pair, every sample's LOD is 0
// and the kernel need not compute it: the result is the same.
static bool reverse_lod_zero(const CamX& c, int cm, Dims vol, Dims frus) {
    if (cm != CM_LINDEPTH_REVERSE && cm != CM_TRANSFORM_REVERSE) return false;
    const float4 rows[4] = {c.r.r0, c.r.r1, c.r.r2, c.r.r3};
    double X[4], Y[4], Z[4], Wc[4];
    double* dst[4] = {X, Y, Z, Wc};
    for (int i = 0; i < 4; ++i) {
        dst[i][0] = rows[i].x, dst[i][1] = rows[i].y, dst[i][2] = rows[i].z, dst[i][3] = rows[i].w;
    }
    struct Comp {
        double scale, n[4], d[4];
    } comp[3];
    comp[0].scale = 0.5 * frus.x;
    comp[1].scale = 0.5 * frus.y;
    for (int j = 0; j < 4; ++j) {
        comp[0].n[j] = X[j], comp[0].d[j] = Wc[j];
        comp[1].n[j] = Y[j], comp[1].d[j] = Wc[j];
    }
    if (cm == CM_LINDEPTH_REVERSE) {
        // idx.z = -(z + near) / (far - near) * dims.z with z = -p23 w / (clip_z + p22 w)
        const double range = (double)c.far_ - (double)c.near_;
        if (!(std::fabs(range) > 0.0)) return false;
        comp[2].scale = (double)frus.z / std::fabs(range);
        for (int j = 0; j < 4; ++j) {
            comp[2].n[j] = (double)c.p23 * Wc[j];
            comp[2].d[j] = Z[j] + (double)c.p22 * Wc[j];
        }
    } else {
        comp[2].scale = 0.5 * frus.z;
        for (int j = 0; j < 4; ++j) comp[2].n[j] = Z[j], comp[2].d[j] = Wc[j];
    }
    constexpr int S = 8;
    const double n3[3] = {(double)vol.x, (double)vol.y, (double)vol.z};
    double bound[3][3] = {};  // [axis][component]
    for (int bz = 0; bz < S; ++bz)
        for (int by = 0; by < S; ++by)
            for (int bx = 0; bx < S; ++bx) {
                const int bi[3] = {bx, by, bz};
                double lo[3], hi[3];
                for (int a = 0; a < 3; ++a) {
                    lo[a] = 0.5 + n3[a] * bi[a] / S;
                    hi[a] = 0.5 + n3[a] * (bi[a] + 1) / S;
                }
                for (int i = 0; i < 3; ++i) {
                    const Comp& f = comp[i];
                    double nv[8], dv[8], dmin = INFINITY;
                    int sign = 0;
                    for (int corner = 0; corner < 8; ++corner) {
                        double n = f.n[3], d = f.d[3];
                        for (int a = 0; a < 3; ++a) {
                            const double v = (corner >> a) & 1 ? hi[a] : lo[a];
                            n += f.n[a] * v;
                            d += f.d[a] * v;
                        }
                        const int sd = d > 0.0 ? 1 : (d < 0.0 ? -1 : 0);
                        if (sd == 0 || (sign != 0 && sd != sign)) return false;
                        sign = sd;
                        nv[corner] = n;
                        dv[corner] = d;
                        dmin = std::min(dmin, std::fabs(d));
                    }
                    for (int k = 0; k < 3; ++k) {
                        double num = 0.0;
                        for (int corner = 0; corner < 8; ++corner)
                            num = std::max(num, std::fabs(f.n[k] * dv[corner] - nv[corner] * f.d[k]));
                        bound[k][i] = std::max(bound[k][i], f.scale * num / (dmin * dmin));
                    }
                }
            }
    double qm = 0.0;
    for (int k = 0; k < 3; ++k)
        qm = std::max(qm, bound[k][0] * bound[k][0] + bound[k][1] * bound[k][1] + bound[k][2] * bound[k][2]);
    return qm < 0.98;
}

template <int C, typename S, int BM>
static void st_fwd_cm(int cm, dim3 blocks, int T, cudaStream_t s, const SampleArgs& a, const MipSet& ms, float* out,
                      const PairTable& t) {
    bool lod = a.mip_mode != MIP_NONE;
    if (lod) {
        bool zero = true;
        for (int k = 0; k < t.n && zero; ++k) zero = reverse_lod_zero(t.cam[k], cm, a.dout, a.din);
        lod = !zero;
    }
#define GFT_ST(CMV)                                                                                             \
    k_sample_transform<C, S, BM, CMV><<<blocks, T, 0, s>>>(a.dout, a.filter, a.mip_mode, lod, a.mip_bias, a.cco, \
                                                           ms, out, t)
    switch (cm) {
        case CM_LINDEPTH: GFT_ST(CM_LINDEPTH); break;
        case CM_TRANSFORM: GFT_ST(CM_TRANSFORM); break;
        case CM_LINDEPTH_REVERSE: GFT_ST(CM_LINDEPTH_REVERSE); break;
        default: GFT_ST(CM_TRANSFORM_REVERSE); break;
    }
#undef GFT_ST
}

template <int C, typename S>
static void st_fwd(int bm, dim3 blocks, int T, cudaStream_t s, const SampleArgs& a, const MipSet& ms, float* out,
                   const PairTable& t) {
    switch (bm) {
        case BM_BORDER: st_fwd_cm<C, S, BM_BORDER>(a.coord_mode, blocks, T, s, a, ms, out, t); break;
        case BM_CLAMP: st_fwd_cm<C, S, BM_CLAMP>(a.coord_mode, blocks, T, s, a, ms, out, t); break;
        default:
            k_sample_transform<C, S, BM_WRAP, CM_LINDEPTH><<<blocks, T, 0, s>>>(a.dout, a.filter, a.mip_mode,
                                                                                a.mip_mode != MIP_NONE, a.mip_bias,
                                                                                a.cco, ms, out, t);
            break;
    }
}

bool launch_sample_transform_fwd(const SampleArgs& a, const std::vector<Pair>& pairs, const MipSet* mips,
                                 float* out, cudaStream_t s) {
    const int64_t nv = voxels(a.dout);
    if (!slice_ok(nv)) return false;
    for (int b = 0; b < a.N; ++b) {
        std::vector<Pair> pb;
        for (const Pair& p : pairs)
            if (p.in_batch == b) pb.push_back(p);
        const int T = knob_value(GFT_KNOB_RESAMPLE_THREADS);  // <= RS_THREADS, the launch bounds
        for (const PairTable& t : make_tables(pb)) {
            const dim3 blocks((unsigned)((nv + T - 1) / T), t.n);
            if (a.dtype == 0) {
                if (a.C == 4) st_fwd<4, float>(a.boundary, blocks, T, s, a, mips[b], out, t);
                else if (a.C == 2) st_fwd<2, float>(a.boundary, blocks, T, s, a, mips[b], out, t);
                else st_fwd<1, float>(a.boundary, blocks, T, s, a, mips[b], out, t);
            } else {
                if (a.C == 4) st_fwd<4, __nv_bfloat16>(a.boundary, blocks, T, s, a, mips[b], out, t);
                else if (a.C == 2) st_fwd<2, __nv_bfloat16>(a.boundary, blocks, T, s, a, mips[b], out, t);
                else st_fwd<1, __nv_bfloat16>(a.boundary, blocks, T, s, a, mips[b], out, t);
            }
            if (!launched(1, "sample transform launch")) return false;
        }
    }
    return true;
}

// Scatter adjoint (kScatter3DGradients): trilinear scatter of dy at the
// sampling position, +1 per reached corner on the uint32 counter.
template <int C, int BM, int COUNT>
__global__ void __launch_bounds__(RS_THREADS)
    k_sample_transform_bwd(Dims din, Dims dout, int cm, float cco, const float* __restrict__ dy,
                           float* __restrict__ grad, unsigned int* __restrict__ count,
                           const __grid_constant__ PairTable tab) {
    const int64_t nv = voxels(dout);
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const int p = blockIdx.y;
    int x, y, z;
    unflat32(v, dout, x, y, z);
    const float3 dinf = make_float3((float)din.x, (float)din.y, (float)din.z);
    const float3 dinv = make_float3(1.f / (float)dout.x, 1.f / (float)dout.y, 1.f / (float)dout.z);
    const float4 pos = sample_pos(tab.cam[p], cm, make_float3(x + 0.5f, y + 0.5f, z + 0.5f), dinf, dinv, false);
    const Vec<C> g = loadf<C>(dy, (int64_t)tab.out_slot[p] * nv + v);
    scatter_linear<C, BM, COUNT>(grad, count, din, pos.x - cco, pos.y - cco, pos.z - cco, g);
}

// grad /= count where count > 0; the counter is reset (kNormalize3DGradients<T,true>).
template <int C>
__global__ void k_normalize_count(float* __restrict__ grad, unsigned int* __restrict__ count, int64_t nv) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nv) return;
    const unsigned int n = count[t];
    if (n > 0) {
        const float w = 1.0f / (float)n;
        store<C>(grad, t, vscale(loadf<C>(grad, t), w));
        count[t] = 0;
    }
}

template <int C>
static void normalize_launch(float* grad, unsigned int* count, int64_t nv, cudaStream_t s) {
    k_normalize_count<C><<<(unsigned)((nv + RS_THREADS - 1) / RS_THREADS), RS_THREADS, 0, s>>>(grad, count, nv);
}
static void normalize_any(int C, float* grad, unsigned int* count, int64_t nv, cudaStream_t s) {
    if (C == 4) normalize_launch<4>(grad, count, nv, s);
    else if (C == 2) normalize_launch<2>(grad, count, nv, s);
    else normalize_launch<1>(grad, count, nv, s);
}

template <int C, int COUNT>
static void stb_launch(int bm, dim3 blocks, cudaStream_t s, Dims din, Dims dout, int cm, float cco,
                       const float* dy, float* grad, unsigned int* count, const PairTable& t) {
    switch (bm) {
        case BM_BORDER:
            k_sample_transform_bwd<C, BM_BORDER, COUNT><<<blocks, RS_THREADS, 0, s>>>(din, dout, cm, cco, dy, grad, count, t);
            break;
        case BM_CLAMP:
            k_sample_transform_bwd<C, BM_CLAMP, COUNT><<<blocks, RS_THREADS, 0, s>>>(din, dout, cm, cco, dy, grad, count, t);
            break;
        default:
            k_sample_transform_bwd<C, BM_WRAP, COUNT><<<blocks, RS_THREADS, 0, s>>>(din, dout, cm, cco, dy, grad, count, t);
            break;
    }
}

bool launch_sample_transform_bwd(int N, int C, Dims din, Dims dout, int boundary, int coord_mode, float cco,
                                 const std::vector<Pair>& pairs, const float* dy, bool exact, float* grad,
                                 unsigned int* count, cudaStream_t s) {
    const int64_t nvi = voxels(din), nvo = voxels(dout);
    if (!slice_ok(nvo)) return false;
    if (!cuda_ok(cudaMemsetAsync(grad, 0, sizeof(float) * nvi * C * N, s), "zero gradient")) return false;
    if (!exact && !cuda_ok(cudaMemsetAsync(count, 0, sizeof(unsigned int) * nvi, s), "zero counter")) return false;
    for (int b = 0; b < N; ++b) {
        std::vector<Pair> pb;
        for (const Pair& p : pairs)
            if (p.in_batch == b) pb.push_back(p);
        float* gb = grad + (size_t)b * nvi * C;
        for (const PairTable& t : make_tables(pb)) {
            const dim3 blocks((unsigned)((nvo + RS_THREADS - 1) / RS_THREADS), t.n);
            if (exact) {
                if (C == 4) stb_launch<4, 0>(boundary, blocks, s, din, dout, coord_mode, cco, dy, gb, count, t);
                else if (C == 2) stb_launch<2, 0>(boundary, blocks, s, din, dout, coord_mode, cco, dy, gb, count, t);
                else stb_launch<1, 0>(boundary, blocks, s, din, dout, coord_mode, cco, dy, gb, count, t);
            } else {
                if (C == 4) stb_launch<4, 1>(boundary, blocks, s, din, dout, coord_mode, cco, dy, gb, count, t);
                else if (C == 2) stb_launch<2, 1>(boundary, blocks, s, din, dout, coord_mode, cco, dy, gb, count, t);
                else stb_launch<1, 1>(boundary, blocks, s, din, dout, coord_mode, cco, dy, gb, count, t);
            }
            if (!launched(1, "sample transform gradient launch")) return false;
        }
        if (!exact) {
            normalize_any(C, gb, count, nvi, s);
            if (!launched(1, "normalize launch")) return false;
        }
    }
    return true;
}

// ---- SampleGridLut -------------------------------------------------------------
struct LutK {
    Dims dout;
    int n_cam;      // cameras handled by this launch
    int cam0;       // first lookup index (separate) or the batch index
    int slot0;      // first output slot
    int filter, mip_mode;
    float bias, cco;
    int relative, normalized;
};

__device__ __forceinline__ float4 lut_pos(const float* __restrict__ lut, int cam, int64_t v, int x, int y, int z,
                                          const LutK& k) {
    float4 p = __ldg(reinterpret_cast<const float4*>(lut) + (int64_t)cam * voxels(k.dout) + v);
    if (k.normalized) {
        p.x *= (float)k.dout.x;
        p.y *= (float)k.dout.y;
        p.z *= (float)k.dout.z;
    }
    if (k.relative) {
        p.x += (float)x;
        p.y += (float)y;
        p.z += (float)z;
    }
    return p;
}

template <int C, typename S, int BM>
__global__ void __launch_bounds__(RS_THREADS)
    k_lut_fwd(const float* __restrict__ lut, const LutK k, const MipSet ms, float* __restrict__ out) {
    const int64_t nv = voxels(k.dout);
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const int c = blockIdx.y;
    int x, y, z;
    unflat32(v, k.dout, x, y, z);
    const float4 pos = lut_pos(lut, k.cam0 + c, v, x, y, z, k);
    const Vec<C> r = sample_mip<C, S, BM>(k.filter, k.mip_mode, ms, pos, k.bias, k.cco);
    store<C>(out, (int64_t)(k.slot0 + c) * nv + v, r);
}

template <int C, typename S>
static void lut_fwd_launch(int bm, dim3 blocks, cudaStream_t s, const float* lut, const LutK& k,
                           const MipSet& ms, float* out) {
    switch (bm) {
        case BM_BORDER: k_lut_fwd<C, S, BM_BORDER><<<blocks, RS_THREADS, 0, s>>>(lut, k, ms, out); break;
        case BM_CLAMP: k_lut_fwd<C, S, BM_CLAMP><<<blocks, RS_THREADS, 0, s>>>(lut, k, ms, out); break;
        default: k_lut_fwd<C, S, BM_WRAP><<<blocks, RS_THREADS, 0, s>>>(lut, k, ms, out); break;
    }
}

static LutK make_lutk(const LutArgs& a, int b) {
    LutK k;
    k.dout = a.dout;
    k.n_cam = a.separate ? a.n_lut : 1;
    k.cam0 = a.separate ? 0 : b;
    k.slot0 = a.separate ? b * a.n_lut : b;
    k.filter = a.filter;
    k.mip_mode = a.mip_mode;
    k.bias = a.mip_bias;
    k.cco = a.cco;
    k.relative = a.relative;
    k.normalized = a.normalized;
    return k;
}

bool launch_lut_fwd(const LutArgs& a, const float* lut, const MipSet* mips, float* out, cudaStream_t s) {
    const int64_t nv = voxels(a.dout);
    if (!slice_ok(nv)) return false;
    for (int b = 0; b < a.N; ++b) {
        const LutK k = make_lutk(a, b);
        const dim3 blocks((unsigned)((nv + RS_THREADS - 1) / RS_THREADS), k.n_cam);
        if (a.dtype == 0) {
            if (a.C == 4) lut_fwd_launch<4, float>(a.boundary, blocks, s, lut, k, mips[b], out);
            else if (a.C == 2) lut_fwd_launch<2, float>(a.boundary, blocks, s, lut, k, mips[b], out);
            else lut_fwd_launch<1, float>(a.boundary, blocks, s, lut, k, mips[b], out);
        } else {
            if (a.C == 4) lut_fwd_launch<4, __nv_bfloat16>(a.boundary, blocks, s, lut, k, mips[b], out);
            else if (a.C == 2) lut_fwd_launch<2, __nv_bfloat16>(a.boundary, blocks, s, lut, k, mips[b], out);
            else lut_fwd_launch<1, __nv_bfloat16>(a.boundary, blocks, s, lut, k, mips[b], out);
        }
        if (!launched(1, "sample lut launch")) return false;
    }
    return true;
}

// kScatterLuT3DGradients: lookup gradient (LINEAR only, written) and trilinear
// input-gradient scatter for every filter mode.
template <int C, int BM, int COUNT>
__global__ void __launch_bounds__(RS_THREADS)
    k_lut_bwd(const float* __restrict__ in, Dims din, const float* __restrict__ lut, const LutK k,
              const float* __restrict__ dy, float* __restrict__ grad, float* __restrict__ lut_grad,
              unsigned int* __restrict__ count) {
    const int64_t nv = voxels(k.dout);
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const int c = blockIdx.y;
    int x, y, z;
    unflat32(v, k.dout, x, y, z);
    const float4 pos = lut_pos(lut, k.cam0 + c, v, x, y, z, k);
    const float px = pos.x - k.cco, py = pos.y - k.cco, pz = pos.z - k.cco;
    const Vec<C> g = loadf<C>(dy, (int64_t)(k.slot0 + c) * nv + v);
    if (k.filter == F_LINEAR) {
        Vec<C> ddx, ddy, ddz;
        fetch_grad<C, BM>(in, din, px, py, pz, ddx, ddy, ddz);
        float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
        for (int i = 0; i < C; ++i) {
            sx += g.v[i] * ddx.v[i];
            sy += g.v[i] * ddy.v[i];
            sz += g.v[i] * ddz.v[i];
        }
        reinterpret_cast<float4*>(lut_grad)[(int64_t)(k.cam0 + c) * nv + v] = make_float4(sx, sy, sz, 0.f);
    }
    scatter_linear<C, BM, COUNT>(grad, count, din, px, py, pz, g);
}

template <int C, int COUNT>
static void lut_bwd_launch(int bm, dim3 blocks, cudaStream_t s, const float* in, Dims din, const float* lut,
                           const LutK& k, const float* dy, float* grad, float* lut_grad, unsigned int* count) {
    switch (bm) {
        case BM_BORDER:
            k_lut_bwd<C, BM_BORDER, COUNT><<<blocks, RS_THREADS, 0, s>>>(in, din, lut, k, dy, grad, lut_grad, count);
            break;
        case BM_CLAMP:
            k_lut_bwd<C, BM_CLAMP, COUNT><<<blocks, RS_THREADS, 0, s>>>(in, din, lut, k, dy, grad, lut_grad, count);
            break;
        default:
            k_lut_bwd<C, BM_WRAP, COUNT><<<blocks, RS_THREADS, 0, s>>>(in, din, lut, k, dy, grad, lut_grad, count);
            break;
    }
}

bool launch_lut_bwd(const LutArgs& a, const float* input, const float* lut, const float* dy, bool exact,
                    float* grad, float* lut_grad, unsigned int* count, cudaStream_t s) {
    const int64_t nvi = voxels(a.din), nvo = voxels(a.dout);
    if (!slice_ok(nvo)) return false;
    if (!cuda_ok(cudaMemsetAsync(grad, 0, sizeof(float) * nvi * a.C * a.N, s), "zero gradient")) return false;
    if (!cuda_ok(cudaMemsetAsync(lut_grad, 0, sizeof(float) * 4 * nvo * a.n_lut, s), "zero lookup gradient"))
        return false;
    if (!exact && !cuda_ok(cudaMemsetAsync(count, 0, sizeof(unsigned int) * nvi, s), "zero counter")) return false;
    for (int b = 0; b < a.N; ++b) {
        const LutK k = make_lutk(a, b);
        const float* inb = input + (size_t)b * nvi * a.C;
        float* gb = grad + (size_t)b * nvi * a.C;
        const dim3 blocks((unsigned)((nvo + RS_THREADS - 1) / RS_THREADS), k.n_cam);
        if (exact) {
            if (a.C == 4) lut_bwd_launch<4, 0>(a.boundary, blocks, s, inb, a.din, lut, k, dy, gb, lut_grad, count);
            else if (a.C == 2) lut_bwd_launch<2, 0>(a.boundary, blocks, s, inb, a.din, lut, k, dy, gb, lut_grad, count);
            else lut_bwd_launch<1, 0>(a.boundary, blocks, s, inb, a.din, lut, k, dy, gb, lut_grad, count);
        } else {
            if (a.C == 4) lut_bwd_launch<4, 1>(a.boundary, blocks, s, inb, a.din, lut, k, dy, gb, lut_grad, count);
            else if (a.C == 2) lut_bwd_launch<2, 1>(a.boundary, blocks, s, inb, a.din, lut, k, dy, gb, lut_grad, count);
            else lut_bwd_launch<1, 1>(a.boundary, blocks, s, inb, a.din, lut, k, dy, gb, lut_grad, count);
        }
        if (!launched(1, "sample lut gradient launch")) return false;
        if (!exact) {
            normalize_any(a.C, gb, count, nvi, s);
            if (!launched(1, "normalize launch")) return false;
        }
    }
    return true;
}

// ---- LodTransform ----------------------------------------------------------------
// calcLoD (sampling.hpp:18-56): central differences, rows of the Jacobian.
__global__ void __launch_bounds__(RS_THREADS)
    k_lod_transform(Dims din, Dims dout, int cm, float* __restrict__ out, const __grid_constant__ PairTable tab) {
    const int64_t nv = voxels(dout);
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const int p = blockIdx.y;
    int x, y, z;
    unflat32(v, dout, x, y, z);
    const float3 dinf = make_float3((float)din.x, (float)din.y, (float)din.z);
    const float3 dinv = make_float3(1.f / (float)dout.x, 1.f / (float)dout.y, 1.f / (float)dout.z);
    const CamX& c = tab.cam[p];
    const float3 idx = make_float3(x + 0.5f, y + 0.5f, z + 0.5f);
    const float3 pos = map_pos(c, cm, idx, dinf, dinv);
    float3 d[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float3 e = make_float3(a == 0 ? 1.f : 0.f, a == 1 ? 1.f : 0.f, a == 2 ? 1.f : 0.f);
        const float3 m = map_pos(c, cm, make_float3(idx.x - e.x, idx.y - e.y, idx.z - e.z), dinf, dinv);
        const float3 q = map_pos(c, cm, make_float3(idx.x + e.x, idx.y + e.y, idx.z + e.z), dinf, dinv);
        d[a] = make_float3((m.x - q.x) * 0.5f, (m.y - q.y) * 0.5f, (m.z - q.z) * 0.5f);
    }
    const float px = sqrtf(d[0].x * d[0].x + d[1].x * d[1].x + d[2].x * d[2].x);
    const float py = sqrtf(d[0].y * d[0].y + d[1].y * d[1].y + d[2].y * d[2].y);
    const float pz = sqrtf(d[0].z * d[0].z + d[1].z * d[1].z + d[2].z * d[2].z);
    const float lod = fmaxf(0.f, log2f(fmaxf(px, fmaxf(py, pz))));
    reinterpret_cast<float4*>(out)[(int64_t)tab.out_slot[p] * nv + v] = make_float4(pos.x, pos.y, pos.z, lod);
}

bool launch_lod_transform(Dims din, Dims dout, const std::vector<Pair>& pairs, bool inverse, float* out,
                          cudaStream_t s) {
    const int64_t nv = voxels(dout);
    if (!slice_ok(nv)) return false;
    for (const PairTable& t : make_tables(pairs)) {
        const dim3 blocks((unsigned)((nv + RS_THREADS - 1) / RS_THREADS), t.n);
        k_lod_transform<<<blocks, RS_THREADS, 0, s>>>(din, dout, inverse ? CM_LINDEPTH_REVERSE : CM_LINDEPTH, out, t);
        if (!launched(1, "lod transform launch")) return false;
    }
    return true;
}

}  // namespace gft
