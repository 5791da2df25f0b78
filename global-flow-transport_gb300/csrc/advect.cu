// Fused advection of a density grid by a staggered velocity grid
// (VelocityGrid.warp, data_structures.py:870-905) and its adjoint.
//
// The reference builds lut = -dt * centered(v) with TF ops and calls
// SampleGridLut up to four times (forward, back, MIN, MAX) plus TF elementwise
// ops.  Here the staggered -> centred average is folded into the lookup and
// MacCormack runs in two passes: (1) the semi-Lagrangian value, (2) the back
// lookup of (1), the correction and the MC_SMOOTH clamp, with the MIN/MAX of
// the forward footprint taken from the same 8 gathers as the forward value.
#include <algorithm>
#include <mutex>
#include <string>

#include "../../include/gft.h"
#include "gft_internal.h"

namespace gft {

constexpr int AD_THREADS = 256;  // the largest block (launch bounds); GFT_KNOB_ADVECT_THREADS picks the size
static int adv_threads() { return knob_value(GFT_KNOB_ADVECT_THREADS); }
constexpr int CLAMP_NONE = 0, CLAMP_MC_SMOOTH = 1, CLAMP_NEGATIVE = 2;

// lut = -dt * centred velocity at voxel (x, y, z) (centered, data_structures.py:819-833)
__device__ __forceinline__ float3 lut_at(const float* __restrict__ vx, const float* __restrict__ vy,
                                         const float* __restrict__ vz, Dims d, int x, int y, int z, float dt) {
    // 32-bit indices: the launchers keep the staggered components of a slice
    // below 2^32 values together (advect_size_ok)
    const uint32_t ux = (uint32_t)x, uy = (uint32_t)y, uz = (uint32_t)z, dx = (uint32_t)d.x, dy = (uint32_t)d.y;
    const uint32_t ix = (uz * dy + uy) * (dx + 1u) + ux;
    const uint32_t iy = (uz * (dy + 1u) + uy) * dx + ux;
    const uint32_t iz = (uz * dy + uy) * dx + ux;
    const float cx = (__ldg(vx + ix + 1u) + __ldg(vx + ix)) * 0.5f;
    const float cy = (__ldg(vy + iy + dx) + __ldg(vy + iy)) * 0.5f;
    const float cz = (__ldg(vz + iz + dx * dy) + __ldg(vz + iz)) * 0.5f;
    return make_float3(cx * (-dt), cy * (-dt), cz * (-dt));
}

// Slices below 2^32 cells (checked by the launchers): 32-bit division.
__device__ __forceinline__ void unflat(int64_t v, Dims d, int& x, int& y, int& z) {
    unflat32((uint32_t)v, d, x, y, z);
}

// Trilinear value plus the MIN/MAX of the lookup op (read3DMin/Max) from one
// set of 8 corner reads.
template <int C, typename S, int BM>
__device__ __forceinline__ void fetch_linear_minmax(const S* __restrict__ g, Dims d, float px, float py, float pz,
                                                    Vec<C>& val, Vec<C>& mn, Vec<C>& mx) {
    if constexpr (BM == BM_BORDER) {
        if (!border_inside(px, py, pz, d)) {
            val = mn = mx = vzero<C>();
            return;
        }
    }
    const Corners c = corners<BM>(px, py, pz, d);
    const bool ok[8] = {c.vx0 && c.vy0 && c.vz0, c.vx1 && c.vy0 && c.vz0, c.vx0 && c.vy1 && c.vz0,
                        c.vx1 && c.vy1 && c.vz0, c.vx0 && c.vy0 && c.vz1, c.vx1 && c.vy0 && c.vz1,
                        c.vx0 && c.vy1 && c.vz1, c.vx1 && c.vy1 && c.vz1};
    const int xs[8] = {c.x0, c.x1, c.x0, c.x1, c.x0, c.x1, c.x0, c.x1};
    const int ys[8] = {c.y0, c.y0, c.y1, c.y1, c.y0, c.y0, c.y1, c.y1};
    const int zs[8] = {c.z0, c.z0, c.z0, c.z0, c.z1, c.z1, c.z1, c.z1};
    Vec<C> v[8];
    bool all_ok = true;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = read_corner<C, S, BM>(g, d, xs[k], ys[k], zs[k], ok[k]);
        all_ok = all_ok && ok[k];
    }
    const Vec<C> v0 = vlerp(vlerp(v[0], v[1], c.wx), vlerp(v[2], v[3], c.wx), c.wy);
    const Vec<C> v1 = vlerp(vlerp(v[4], v[5], c.wx), vlerp(v[6], v[7], c.wx), c.wy);
    val = vlerp(v0, v1, c.wz);
    mn = vfill<C>(all_ok ? REF_FLOAT_MAX : 0.f);
    mx = vfill<C>(all_ok ? -REF_FLOAT_MAX : 0.f);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        if (BM != BM_BORDER || ok[k]) {
            mn = vmin(mn, v[k]);
            mx = vmax(mx, v[k]);
        }
    }
}

template <int C>
__device__ __forceinline__ Vec<C> vmax0(Vec<C> a) {
#pragma unroll
    for (int i = 0; i < C; ++i) a.v[i] = fmaxf(a.v[i], 0.f);
    return a;
}

// Pass 1 / semi-Lagrangian: out = d(x + lut(x))
template <int C, typename S, int BM>
__global__ void __launch_bounds__(AD_THREADS)
    k_adv_sl(const S* __restrict__ d, Dims dm, const float* __restrict__ vx, const float* __restrict__ vy,
             const float* __restrict__ vz, float dt, bool negative, float* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= voxels(dm)) return;
    int x, y, z;
    unflat(t, dm, x, y, z);
    const float3 l = lut_at(vx, vy, vz, dm, x, y, z, dt);
    Vec<C> r = fetch_linear<C, S, BM>(d, dm, l.x + (float)x, l.y + (float)y, l.z + (float)z);
    if (negative) r = vmax0(r);
    store<C>(out, t, r);
}

// Pass 2 / MacCormack: corr = fwd + 0.5*(d - fwd(x - lut)), MC_SMOOTH keeps fwd
// where corr leaves [min, max] of the forward footprint.
template <int C, typename S, int BM>
__global__ void __launch_bounds__(AD_THREADS)
    k_adv_mc(const S* __restrict__ d, const float* __restrict__ fwd, Dims dm, const float* __restrict__ vx,
             const float* __restrict__ vy, const float* __restrict__ vz, float dt, int clamp, float* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= voxels(dm)) return;
    int x, y, z;
    unflat(t, dm, x, y, z);
    const float3 l = lut_at(vx, vy, vz, dm, x, y, z, dt);
    Vec<C> f, mn, mx;
    fetch_linear_minmax<C, S, BM>(d, dm, l.x + (float)x, l.y + (float)y, l.z + (float)z, f, mn, mx);
    const Vec<C> back = fetch_linear<C, float, BM>(fwd, dm, -l.x + (float)x, -l.y + (float)y, -l.z + (float)z);
    const Vec<C> dv = Load<C, S>::at(d, t);
    Vec<C> r;
#pragma unroll
    for (int i = 0; i < C; ++i) {
        float corr = f.v[i] + 0.5f * (dv.v[i] - back.v[i]);
        if (clamp == CLAMP_MC_SMOOTH && (corr < mn.v[i] || corr > mx.v[i])) corr = f.v[i];
        if (clamp == CLAMP_NEGATIVE) corr = fmaxf(corr, 0.f);
        r.v[i] = corr;
    }
    store<C>(out, t, r);
}

template <int C, typename S>
static bool adv_fwd_c(const AdvectArgs& a, float* out, float* ws, cudaStream_t s) {
    const int64_t nv = voxels(a.d);
    const int T = adv_threads();
    const unsigned blocks = (unsigned)((nv + T - 1) / T);
    for (int b = 0; b < a.N; ++b) {
        const S* db = reinterpret_cast<const S*>(a.density) + (size_t)b * nv * C;
        float* ob = out + (size_t)b * nv * C;
        if (a.order == 1) {
            const bool neg = a.clamp == CLAMP_NEGATIVE;
            switch (a.boundary) {
                case BM_BORDER: k_adv_sl<C, S, BM_BORDER><<<blocks, T, 0, s>>>(db, a.d, a.vx, a.vy, a.vz, a.dt, neg, ob); break;
                case BM_CLAMP: k_adv_sl<C, S, BM_CLAMP><<<blocks, T, 0, s>>>(db, a.d, a.vx, a.vy, a.vz, a.dt, neg, ob); break;
                default: k_adv_sl<C, S, BM_WRAP><<<blocks, T, 0, s>>>(db, a.d, a.vx, a.vy, a.vz, a.dt, neg, ob); break;
            }
        } else {
            switch (a.boundary) {
                case BM_BORDER:
                    k_adv_sl<C, S, BM_BORDER><<<blocks, T, 0, s>>>(db, a.d, a.vx, a.vy, a.vz, a.dt, false, ws);
                    k_adv_mc<C, S, BM_BORDER><<<blocks, T, 0, s>>>(db, ws, a.d, a.vx, a.vy, a.vz, a.dt, a.clamp, ob);
                    break;
                case BM_CLAMP:
                    k_adv_sl<C, S, BM_CLAMP><<<blocks, T, 0, s>>>(db, a.d, a.vx, a.vy, a.vz, a.dt, false, ws);
                    k_adv_mc<C, S, BM_CLAMP><<<blocks, T, 0, s>>>(db, ws, a.d, a.vx, a.vy, a.vz, a.dt, a.clamp, ob);
                    break;
                default:
                    k_adv_sl<C, S, BM_WRAP><<<blocks, T, 0, s>>>(db, a.d, a.vx, a.vy, a.vz, a.dt, false, ws);
                    k_adv_mc<C, S, BM_WRAP><<<blocks, T, 0, s>>>(db, ws, a.d, a.vx, a.vy, a.vz, a.dt, a.clamp, ob);
                    break;
            }
        }
        if (!launched(a.order == 1 ? 1 : 2, "advect launch")) return false;
    }
    return true;
}

// The advection kernels index a grid slice (and the three staggered
// components together) with 32-bit arithmetic.
static bool advect_size_ok(Dims d) {
    const int64_t n = voxels(d);
    const int64_t stag = n * 3 + (int64_t)d.y * d.z + (int64_t)d.x * d.z + (int64_t)d.x * d.y;
    if (stag < MAX_SLICE_CELLS) return true;
    set_error("advection grid too large for 32-bit cell indexing");
    return false;
}

bool launch_advect_fwd(const AdvectArgs& a, float* out, float* ws, cudaStream_t s) {
    if (!advect_size_ok(a.d)) return false;
    if (a.dtype == 0) {
        if (a.C == 4) return adv_fwd_c<4, float>(a, out, ws, s);
        if (a.C == 2) return adv_fwd_c<2, float>(a, out, ws, s);
        return adv_fwd_c<1, float>(a, out, ws, s);
    }
    if (a.C == 4) return adv_fwd_c<4, __nv_bfloat16>(a, out, ws, s);
    if (a.C == 2) return adv_fwd_c<2, __nv_bfloat16>(a, out, ws, s);
    return adv_fwd_c<1, __nv_bfloat16>(a, out, ws, s);
}

// ---- adjoint ---------------------------------------------------------------------
// Single-channel reference-mode scatters keep each voxel's gradient sum and
// its sample count side by side (float2: sum, count) and add both with one
// vector reduction per corner instead of a float and an integer reduction;
// counts stay far below 2^24, where float counting is exact.
// COUNT: 0 exact (no counts), 1 uint counters, 2 packed (C == 1 only)
template <int C, int COUNT>
constexpr bool packed_count() {
    return C == 1 && COUNT == 2;
}

// Trilinear scatter of an adjoint lookup, neighbouring lanes merged.  The
// lanes of a warp are consecutive voxels along x, and their lookups usually
// land one cell apart: a lane's upper-x corners are then the next lane's
// lower-x corners (x1 = x0' with the same y0, y1, z0, z1 -- compared after the
// boundary remap, so equal coordinates are the same cells).  Such a lane hands
// its four upper-x contributions to the next lane, which adds them to its
// own lower-x ones (with count 2) before reducing: 4 reductions instead of 8
// for the lane that gives.  All 32 lanes call it; act = this lane scatters.
// COUNT 0: exact (BORDER: the fetch window); 1: uint counters, 2: packed
// (sum, count) pairs (C == 1), both with the reference's (-1, dims) window.
// DET (deterministic adjoint; COUNT 0 or 1): the contributions, scaled by the
// power of two iscale and rounded, are added to int64 accumulators (C per
// voxel) instead of buf; integer sums do not depend on the order of the adds.
template <int C, int BM, int COUNT, bool DET = false>
__device__ __forceinline__ void scatter_merged(float* __restrict__ buf, unsigned int* __restrict__ cnt, Dims d,
                                               bool act, float px, float py, float pz, Vec<C> val,
                                               unsigned long long* __restrict__ iacc = nullptr, float iscale = 0.f) {
    constexpr bool PACK = packed_count<C, COUNT>();
    constexpr unsigned FULL = 0xffffffffu;
    if constexpr (BM == BM_BORDER) {
        if constexpr (COUNT == 0)
            act = act && border_inside(px, py, pz, d);
        else
            act = act && px > -1.f && px < (float)d.x && py > -1.f && py < (float)d.y && pz > -1.f && pz < (float)d.z;
    }
    const Corners c = corners<BM>(px, py, pz, d);
    const unsigned lane = threadIdx.x & 31u;  // 1-D blocks of whole warps
    const int ux1 = __shfl_up_sync(FULL, c.x1, 1), uy0 = __shfl_up_sync(FULL, c.y0, 1),
              uy1 = __shfl_up_sync(FULL, c.y1, 1), uz0 = __shfl_up_sync(FULL, c.z0, 1),
              uz1 = __shfl_up_sync(FULL, c.z1, 1);
    const unsigned acts = __ballot_sync(FULL, act);
    // bit lane - 1 of acts (0 for lane 0)
    const bool take = act && (((acts << 1) >> lane) & 1u) && ux1 == c.x0 && uy0 == c.y0 && uy1 == c.y1 &&
                      uz0 == c.z0 && uz1 == c.z1;
    const unsigned takes = __ballot_sync(FULL, take);
    const bool give = ((takes >> 1) >> lane) & 1u;  // bit lane + 1 (0 for lane 31)
    const float cw[3] = {c.wx, c.wy, c.wz};
    Vec<C> v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int sx = k & 1, sy = (k >> 1) & 1, sz = (k >> 2) & 1;
        const float w = (sx ? cw[0] : 1.f - cw[0]) * (sy ? cw[1] : 1.f - cw[1]) * (sz ? cw[2] : 1.f - cw[2]);
        v[k] = vscale(val, w);
    }
#pragma unroll
    for (int k = 1; k < 8; k += 2)
#pragma unroll
        for (int ch = 0; ch < C; ++ch) {
            const float m = __shfl_up_sync(FULL, v[k].v[ch], 1);
            if (take) v[k - 1].v[ch] += m;
        }
    if (!act) return;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int sx = k & 1, sy = (k >> 1) & 1, sz = (k >> 2) & 1;
        const bool ok = (sx ? c.vx1 : c.vx0) && (sy ? c.vy1 : c.vy0) && (sz ? c.vz1 : c.vz0);
        if ((BM == BM_BORDER && !ok) || (sx && give)) continue;
        const int64_t f = flat3(sx ? c.x1 : c.x0, sy ? c.y1 : c.y0, sz ? c.z1 : c.z0, d);
        const bool two = !sx && take;
        if constexpr (DET) {
#pragma unroll
            for (int ch = 0; ch < C; ++ch)
                atomicAdd(iacc + f * C + ch, (unsigned long long)__float2ll_rn(v[k].v[ch] * iscale));
            if constexpr (COUNT == 1) atomicAdd(cnt + f, two ? 2u : 1u);
            continue;
        }
        if constexpr (PACK) {
            atomicAdd(reinterpret_cast<float2*>(buf) + f, make_float2(v[k].v[0], two ? 2.f : 1.f));
        } else {
            atomic_add<C>(buf, f, v[k]);
            if constexpr (COUNT == 1) atomicAdd(cnt + f, two ? 2u : 1u);
        }
    }
}

// ---- deterministic adjoint (GFT_GRAD_DETERMINISTIC) ---------------------------
// The two lookup scatters add fixed-point int64 contributions.  Their scales
// are powers of two from bounds of every voxel's partial sums, computed on the
// GPU from maxima (independent of the evaluation order): the back lookup
// scatters -0.5 g_corr (|.| <= 0.5 max|dy|) with trilinear weights summing to
// one per lookup, so no voxel's sum exceeds 0.5 max|dy| N; the forward lookup
// scatters the fwd adjoint, whose largest magnitude a max pass measures, times
// N.  scale = 2^(61 - ceil(log2 bound)) keeps every partial sum below 2^61.
template <int C>
__device__ __forceinline__ Vec<C> det_load(const unsigned long long* __restrict__ acc, int64_t t, float scale) {
    Vec<C> r;
    const double inv = 1.0 / (double)scale;
#pragma unroll
    for (int c = 0; c < C; ++c) r.v[c] = (float)((double)(long long)acc[t * C + c] * inv);
    return r;
}
__device__ __forceinline__ void adv_warp_absmax(unsigned int* out, float m) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float x = __shfl_down_sync(0xffffffffu, m, o);
        m = (x > m || x != x) ? x : m;  // NaN propagates
    }
    if ((threadIdx.x & 31u) == 0) atomicMax(out, __float_as_uint(m));
}
// max |dy| of one slice
__global__ void k_adv_det_absmax(const float* __restrict__ v, int64_t n, unsigned int* __restrict__ out) {
    float m = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float x = fabsf(v[i]);
        m = (x > m || x != x) ? x : m;
    }
    adv_warp_absmax(out, m);
}
// max |fwd adjoint| = max |gdir + (normalised) back-lookup scatter|
template <int C, int COUNT>
__global__ void k_adv_det_gfmax(const float* __restrict__ gdir, const unsigned long long* __restrict__ iacc,
                                const float* __restrict__ iscale, const unsigned int* __restrict__ cnt, int64_t nv,
                                unsigned int* __restrict__ out) {
    float m = 0.f;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nv; t += (int64_t)gridDim.x * blockDim.x) {
        Vec<C> sc = det_load<C>(iacc, t, *iscale);
        if (COUNT) {
            const unsigned int n = cnt[t];
            if (n > 0) sc = vscale(sc, 1.0f / (float)n);
        }
        const Vec<C> g = loadf<C>(gdir, t);
#pragma unroll
        for (int c = 0; c < C; ++c) {
            const float x = fabsf(g.v[c] + sc.v[c]);
            m = (x > m || x != x) ? x : m;
        }
    }
    adv_warp_absmax(out, m);
}
// scale <- 2^(61 - ceil(log2(factor * max))), NaN for a non-finite bound
__global__ void k_adv_det_scale(const unsigned int* __restrict__ maxbits, double factor, float* __restrict__ scale) {
    const double t = (double)__uint_as_float(*maxbits) * factor;
    float sc;
    if (!(t < 1e300)) {
        sc = __int_as_float(0x7fc00000);
    } else if (t <= 0.0) {
        sc = 1.f;
    } else {
        sc = ldexpf(1.f, 61 - max(-60, (int)ceil(log2(t))));
    }
    *scale = sc;
}

// (sum / count where count > 0) of a packed pair, as the uint-counter form
__device__ __forceinline__ float packed_normalised(const float* __restrict__ buf, int64_t t) {
    const float2 v = reinterpret_cast<const float2*>(buf)[t];
    return v.y > 0.f ? v.x * (1.0f / v.y) : v.x;
}

// Stage B (MacCormack only): route the output gradient through the MC_SMOOTH
// `where` (TF semantics: each branch gets the gradient where selected, none to
// min/max), store the direct density term 0.5*g_corr, scatter the back-lookup
// gradient -0.5*g_corr into the fwd adjoint and accumulate the lookup gradient
// of the back lookup (whose lut is -lut).
// Single channel: at most 51 registers (5 blocks of 256 per SM; 48 used, no
// spills with the 32-bit cell indices) for the latency of the two corner
// gathers.
template <int C, int BM, int COUNT, bool DET = false>
__global__ void __launch_bounds__(AD_THREADS, C == 1 ? 5 : 1)
    k_adv_bwd_back(const float* __restrict__ d, const float* __restrict__ fwd, Dims dm, const float* __restrict__ vx,
                   const float* __restrict__ vy, const float* __restrict__ vz, float dt, int clamp,
                   const float* __restrict__ dy, float* __restrict__ gd, float* __restrict__ gfwd_sc,
                   unsigned int* __restrict__ cnt2, float* __restrict__ gdir, float* __restrict__ glut, bool first,
                   unsigned long long* __restrict__ iacc, const float* __restrict__ iscale) {
    const int64_t nv = voxels(dm), t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = t0 < nv;  // lanes past the end stay for the merged scatter
    const int64_t t = in ? t0 : nv - 1;
    int x, y, z;
    unflat(t, dm, x, y, z);
    const float3 l = lut_at(vx, vy, vz, dm, x, y, z, dt);
    Vec<C> f, mn, mx;
    fetch_linear_minmax<C, float, BM>(d, dm, l.x + (float)x, l.y + (float)y, l.z + (float)z, f, mn, mx);
    const float bx = -l.x + (float)x, by = -l.y + (float)y, bz = -l.z + (float)z;
    Vec<C> back, ddx, ddy, ddz;  // back lookup value and its spatial derivative, one corner set
    fetch_linear_grad<C, BM>(fwd, dm, bx, by, bz, back, ddx, ddy, ddz);
    const Vec<C> dv = loadf<C>(d, t);
    Vec<C> g = loadf<C>(dy, t);
    Vec<C> gcorr, gback;
#pragma unroll
    for (int i = 0; i < C; ++i) {
        const float corr = f.v[i] + 0.5f * (dv.v[i] - back.v[i]);
        bool oob = false;
        if (clamp == CLAMP_MC_SMOOTH) oob = corr < mn.v[i] || corr > mx.v[i];
        if (clamp == CLAMP_NEGATIVE && !(corr >= 0.f)) g.v[i] = 0.f;
        gcorr.v[i] = oob ? 0.f : g.v[i];
        gback.v[i] = -0.5f * gcorr.v[i];
    }
    if (in) {
        store<C>(gd, t, vscale(gcorr, 0.5f));
        if (gdir != nullptr) store<C>(gdir, t, g);  // only the NEGATIVE clamp changes g
    }
    scatter_merged<C, BM, COUNT, DET>(gfwd_sc, cnt2, dm, in, bx, by, bz, gback, iacc, DET ? *iscale : 0.f);
    if (!in) return;
    float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
    for (int i = 0; i < C; ++i) {
        sx += gback.v[i] * ddx.v[i];
        sy += gback.v[i] * ddy.v[i];
        sz += gback.v[i] * ddz.v[i];
    }
    float* gl = glut + t;  // three planes (x, y, z components) of nv floats
    if (first) {           // the slice's first lookup-gradient term: written, not added
        gl[0] = -sx;
        gl[nv] = -sy;
        gl[2 * nv] = -sz;
    } else {
        gl[0] -= sx;
        gl[nv] -= sy;
        gl[2 * nv] -= sz;
    }
}

// Stage C: fwd adjoint = direct term + (normalised) back-lookup scatter; scatter
// it into the density through the forward lookup and accumulate that lookup's
// gradient.  first_order: the fwd adjoint is the output gradient itself.
template <int C, int BM, int COUNT, bool DET = false>
__global__ void __launch_bounds__(AD_THREADS)
    k_adv_bwd_fwd(const float* __restrict__ d, Dims dm, const float* __restrict__ vx, const float* __restrict__ vy,
                  const float* __restrict__ vz, float dt, bool first_order, bool negative,
                  const float* __restrict__ gdir, const float* __restrict__ gfwd_sc,
                  const unsigned int* __restrict__ cnt2, float* __restrict__ gd_sc, unsigned int* __restrict__ cnt3,
                  float* __restrict__ glut, bool first, const unsigned long long* __restrict__ iacc_in,
                  const float* __restrict__ iscale_in, unsigned long long* __restrict__ iacc_out,
                  const float* __restrict__ iscale_out, float* __restrict__ gvx, float* __restrict__ gvy,
                  float* __restrict__ gvz) {
    const int64_t nv = voxels(dm), t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = t0 < nv;  // lanes past the end stay for the merged scatter
    const int64_t t = in ? t0 : nv - 1;
    int x, y, z;
    unflat(t, dm, x, y, z);
    const float3 l = lut_at(vx, vy, vz, dm, x, y, z, dt);
    const float px = l.x + (float)x, py = l.y + (float)y, pz = l.z + (float)z;
    Vec<C> gf = loadf<C>(gdir, t);
    Vec<C> ddx, ddy, ddz;
    if (first_order && negative) {
        Vec<C> f;
        fetch_linear_grad<C, BM>(d, dm, px, py, pz, f, ddx, ddy, ddz);
#pragma unroll
        for (int i = 0; i < C; ++i)
            if (!(f.v[i] >= 0.f)) gf.v[i] = 0.f;
    } else {
        fetch_grad<C, BM>(d, dm, px, py, pz, ddx, ddy, ddz);
    }
    if (!first_order) {
        Vec<C> sc;
        if constexpr (DET) {
            sc = det_load<C>(iacc_in, t, *iscale_in);
            if (COUNT) {
                const unsigned int n = cnt2[t];
                if (n > 0) sc = vscale(sc, 1.0f / (float)n);
            }
        } else if constexpr (packed_count<C, COUNT>()) {
            sc.v[0] = packed_normalised(gfwd_sc, t);
        } else {
            sc = loadf<C>(gfwd_sc, t);
            if (COUNT) {
                const unsigned int n = cnt2[t];
                if (n > 0) sc = vscale(sc, 1.0f / (float)n);
            }
        }
        gf = vadd(gf, sc);
    }
    scatter_merged<C, BM, COUNT, DET>(gd_sc, cnt3, dm, in, px, py, pz, gf, iacc_out, DET ? *iscale_out : 0.f);
    if (!in) return;
    float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
    for (int i = 0; i < C; ++i) {
        sx += gf.v[i] * ddx.v[i];
        sy += gf.v[i] * ddy.v[i];
        sz += gf.v[i] * ddz.v[i];
    }
    float* gl = glut + t;  // three planes (x, y, z components) of nv floats
    if (!first) {
        sx += gl[0];
        sy += gl[nv];
        sz += gl[2 * nv];
    }
    if (gvx != nullptr) {
        // the last slice: the velocity gradient directly.  g_centred = -dt
        // g_lut, and the adjoint of the face average gives each of the cell's
        // two faces per axis half of it.  Every face receives at most two
        // additions into the zeroed gradient, whose sum does not depend on
        // their order.
        const float h = -0.5f * dt;
        const int64_t rx = ((int64_t)z * dm.y + y) * (dm.x + 1) + x;
        const int64_t ry = ((int64_t)z * (dm.y + 1) + y) * dm.x + x;
        const float ax = h * sx, ay = h * sy, az = h * sz;
        atomicAdd(gvx + rx, ax);
        atomicAdd(gvx + rx + 1, ax);
        atomicAdd(gvy + ry, ay);
        atomicAdd(gvy + ry + dm.x, ay);
        atomicAdd(gvz + t, az);
        atomicAdd(gvz + t + (int64_t)dm.x * dm.y, az);
        return;
    }
    gl[0] = sx;  // the slice's lookup-gradient terms, added to the earlier slices'
    gl[nv] = sy;
    gl[2 * nv] = sz;
}

// Stage D: density gradient = direct term + (normalised) forward-lookup scatter.
template <int C, int COUNT, bool DET = false>
__global__ void k_adv_bwd_density(float* __restrict__ gd, const float* __restrict__ gd_sc,
                                  const unsigned int* __restrict__ cnt3, int64_t nv,
                                  const unsigned long long* __restrict__ iacc, const float* __restrict__ iscale) {
    constexpr bool NORM = COUNT != 0;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nv) return;
    Vec<C> sc;
    if constexpr (DET) {
        sc = det_load<C>(iacc, t, *iscale);
        if (NORM) {
            const unsigned int n = cnt3[t];
            if (n > 0) sc = vscale(sc, 1.0f / (float)n);
        }
    } else if constexpr (packed_count<C, COUNT>()) {
        sc.v[0] = packed_normalised(gd_sc, t);
    } else {
        sc = loadf<C>(gd_sc, t);
        if (NORM) {
            const unsigned int n = cnt3[t];
            if (n > 0) sc = vscale(sc, 1.0f / (float)n);
        }
    }
    store<C>(gd, t, vadd(loadf<C>(gd, t), sc));
}

// Velocity gradient of the deterministic adjoint (the float adjoint adds it in
// its last kernel): g_centred = -dt * g_lut, then the adjoint of the face
// average (each face receives half of both adjacent cells).  glut holds the
// lookup gradient as three planes (x, y, z components) of voxels(dm) floats.
__global__ void k_adv_bwd_velocity(const float* __restrict__ glut, Dims dm, float dt, float* __restrict__ gvx,
                                   float* __restrict__ gvy, float* __restrict__ gvz) {
    const float* __restrict__ gx = glut;
    const float* __restrict__ gy = glut + voxels(dm);
    const float* __restrict__ gz = glut + 2 * voxels(dm);
    // nx + ny + nz < 2^32 (checked by the launcher): 32-bit index arithmetic
    const uint32_t nx = (uint32_t)(dm.x + 1) * dm.y * dm.z;
    const uint32_t ny = (uint32_t)dm.x * (dm.y + 1) * dm.z;
    const uint32_t nz = (uint32_t)dm.x * dm.y * (dm.z + 1);
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const float h = -0.5f * dt;
    if (t < nx) {
        const uint32_t r = t / (uint32_t)(dm.x + 1);  // z*H + y
        const int i = (int)(t - r * (uint32_t)(dm.x + 1));
        float a = 0.f;
        if (i > 0) a += gx[r * (uint32_t)dm.x + i - 1];
        if (i < dm.x) a += gx[r * (uint32_t)dm.x + i];
        gvx[t] = h * a;
        return;
    }
    t -= nx;
    if (t < ny) {
        int x, j, z;
        unflat32(t, Dims{dm.x, dm.y + 1, dm.z}, x, j, z);
        float a = 0.f;
        if (j > 0) a += gy[((uint32_t)z * dm.y + j - 1) * dm.x + x];
        if (j < dm.y) a += gy[((uint32_t)z * dm.y + j) * dm.x + x];
        gvy[t] = h * a;
        return;
    }
    t -= ny;
    if (t < nz) {
        const uint32_t plane = (uint32_t)dm.x * dm.y;
        const int64_t k = t / plane;
        const int64_t xy = t - (uint32_t)k * plane;
        float a = 0.f;
        if (k > 0) a += gz[(k - 1) * plane + xy];
        if (k < dm.z) a += gz[k * plane + xy];
        gvz[t] = h * a;
    }
}

// Workspace of the deterministic adjoint: fwd | gdir | glut (3 planes) | two
// counter planes | the two int64 scatter targets | maxima and scales.
struct AdvDetLayout {
    size_t fwd, gdir, glut, cnt2, cnt3, acc2, acc3, small, total;  // byte offsets
};
static AdvDetLayout adv_det_layout(size_t nv, size_t C) {
    AdvDetLayout l;
    const size_t vc = nv * C;
    l.fwd = 0;
    l.gdir = l.fwd + 4 * vc;
    l.glut = l.gdir + 4 * vc;
    l.cnt2 = l.glut + 12 * nv;
    l.cnt3 = l.cnt2 + 4 * nv;
    l.acc2 = (l.cnt3 + 4 * nv + 7) & ~size_t(7);
    l.acc3 = l.acc2 + 8 * vc;
    l.small = l.acc3 + 8 * vc;
    l.total = l.small + 16;
    return l;
}

size_t advect_det_ws_bytes(size_t nv, size_t C) { return adv_det_layout(nv, C).total; }

static unsigned det_reduce_blocks(int64_t n) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8));
}

template <int C, int BM, int COUNT>
static bool adv_bwd_det(const AdvectArgs& a, bool forward_ready, const float* dy, float* gd, float* gvx, float* gvy,
                        float* gvz, float* ws, cudaStream_t s) {
    const int64_t nv = voxels(a.d);
    const int T = adv_threads();
    const unsigned blocks = (unsigned)((nv + T - 1) / T);
    const size_t vc = (size_t)nv * C;
    const AdvDetLayout L = adv_det_layout((size_t)nv, C);
    char* base = reinterpret_cast<char*>(ws);
    float* fwd = reinterpret_cast<float*>(base + L.fwd);
    float* gdir = reinterpret_cast<float*>(base + L.gdir);
    float* glut = reinterpret_cast<float*>(base + L.glut);
    unsigned int* cnt2 = reinterpret_cast<unsigned int*>(base + L.cnt2);
    unsigned int* cnt3 = reinterpret_cast<unsigned int*>(base + L.cnt3);
    unsigned long long* acc2 = reinterpret_cast<unsigned long long*>(base + L.acc2);
    unsigned long long* acc3 = reinterpret_cast<unsigned long long*>(base + L.acc3);
    unsigned int* maxbits = reinterpret_cast<unsigned int*>(base + L.small);
    float* scale = reinterpret_cast<float*>(base + L.small + 8);
    const float* dens = reinterpret_cast<const float*>(a.density);
    const unsigned rb = det_reduce_blocks((int64_t)vc);
    for (int b = 0; b < a.N; ++b) {
        const float* db = dens + (size_t)b * vc;
        const float* dyb = dy + (size_t)b * vc;
        float* gdb = gd + (size_t)b * vc;
        // counters (when used) and both accumulators are contiguous from cnt2
        if (!cuda_ok(cudaMemsetAsync(base + L.cnt2, 0, L.small + 8 - L.cnt2, s), "zero scatter")) return false;
        int n = 0;
        if (a.order == 2) {
            if (!forward_ready)
                k_adv_sl<C, float, BM><<<blocks, T, 0, s>>>(db, a.d, a.vx, a.vy, a.vz, a.dt, false, fwd), ++n;
            // back-lookup scatter of -0.5 g_corr: |sum| <= 0.5 max|dy| * voxels
            k_adv_det_absmax<<<rb, 256, 0, s>>>(dyb, (int64_t)vc, maxbits);
            k_adv_det_scale<<<1, 1, 0, s>>>(maxbits, 0.5 * (double)nv, scale);
            const bool neg = a.clamp == CLAMP_NEGATIVE;
            const float* gd_dir = neg ? gdir : dyb;
            k_adv_bwd_back<C, BM, COUNT, true><<<blocks, T, 0, s>>>(db, fwd, a.d, a.vx, a.vy, a.vz, a.dt, a.clamp,
                                                                    dyb, gdb, nullptr, cnt2, neg ? gdir : nullptr,
                                                                    glut, b == 0, acc2, scale);
            k_adv_det_gfmax<C, COUNT><<<rb, 256, 0, s>>>(gd_dir, acc2, scale, cnt2, nv, maxbits + 1);
            k_adv_det_scale<<<1, 1, 0, s>>>(maxbits + 1, (double)nv, scale + 1);
            k_adv_bwd_fwd<C, BM, COUNT, true><<<blocks, T, 0, s>>>(db, a.d, a.vx, a.vy, a.vz, a.dt, false, false,
                                                                   gd_dir, nullptr, cnt2, nullptr, cnt3, glut, false,
                                                                   acc2, scale, acc3, scale + 1, nullptr, nullptr,
                                                                   nullptr);
            n += 6;
        } else {
            if (!cuda_ok(cudaMemsetAsync(gdb, 0, sizeof(float) * vc, s), "zero gradient")) return false;
            k_adv_det_absmax<<<rb, 256, 0, s>>>(dyb, (int64_t)vc, maxbits + 1);
            k_adv_det_scale<<<1, 1, 0, s>>>(maxbits + 1, (double)nv, scale + 1);
            k_adv_bwd_fwd<C, BM, COUNT, true><<<blocks, T, 0, s>>>(db, a.d, a.vx, a.vy, a.vz, a.dt, true,
                                                                   a.clamp == CLAMP_NEGATIVE, dyb, nullptr, nullptr,
                                                                   nullptr, cnt3, glut, b == 0, nullptr, nullptr,
                                                                   acc3, scale + 1, nullptr, nullptr, nullptr);
            n += 3;
        }
        k_adv_bwd_density<C, COUNT, true><<<blocks, T, 0, s>>>(gdb, nullptr, cnt3, nv, acc3, scale + 1);
        if (!launched(n + 1, "advect gradient launch")) return false;
    }
    const int64_t nstag = (int64_t)(a.d.x + 1) * a.d.y * a.d.z + (int64_t)a.d.x * (a.d.y + 1) * a.d.z +
                          (int64_t)a.d.x * a.d.y * (a.d.z + 1);
    k_adv_bwd_velocity<<<(unsigned)((nstag + T - 1) / T), T, 0, s>>>(glut, a.d, a.dt, gvx, gvy, gvz);
    return launched(1, "velocity gradient launch");
}

template <int C, int BM, int COUNT>
static bool adv_bwd_impl(const AdvectArgs& a, bool forward_ready, const float* dy, float* gd, float* gvx, float* gvy,
                         float* gvz, float* ws, cudaStream_t s) {
    const int64_t nv = voxels(a.d);
    const int T = adv_threads();
    const unsigned blocks = (unsigned)((nv + T - 1) / T);
    const size_t vc = (size_t)nv * C;
    // packed: the two scatter targets hold (sum, count) pairs at even offsets
    // (8-byte aligned with ws), no counters
    constexpr bool PACK = packed_count<C, COUNT>();
    const size_t sc_floats = PACK ? 2 * vc : vc, vc_pad = PACK ? (vc + 1) & ~size_t(1) : vc;
    float* fwd = ws;
    float* gfwd_sc = fwd + vc_pad;
    float* gdir = gfwd_sc + sc_floats;
    float* gd_sc = gdir + vc_pad;
    float* glut = gd_sc + sc_floats;
    unsigned int* cnt2 = PACK ? nullptr : reinterpret_cast<unsigned int*>(glut + (size_t)nv * 3);
    unsigned int* cnt3 = PACK ? nullptr : cnt2 + nv;
    // glut: slice 0's first kernel writes every voxel's lookup gradient, the
    // later kernels and slices add to it (no zeroing pass); the last slice's
    // final kernel adds its terms into the velocity faces instead
    const size_t nfx = (size_t)(a.d.x + 1) * a.d.y * a.d.z, nfy = (size_t)a.d.x * (a.d.y + 1) * a.d.z,
                 nfz = (size_t)a.d.x * a.d.y * (a.d.z + 1);
    if (!cuda_ok(cudaMemsetAsync(gvx, 0, sizeof(float) * nfx, s), "zero velocity gradient") ||
        !cuda_ok(cudaMemsetAsync(gvy, 0, sizeof(float) * nfy, s), "zero velocity gradient") ||
        !cuda_ok(cudaMemsetAsync(gvz, 0, sizeof(float) * nfz, s), "zero velocity gradient"))
        return false;
    const float* dens = reinterpret_cast<const float*>(a.density);
    for (int b = 0; b < a.N; ++b) {
        const bool last = b == a.N - 1;
        const float* db = dens + (size_t)b * vc;
        const float* dyb = dy + (size_t)b * vc;
        float* gdb = gd + (size_t)b * vc;
        if (!cuda_ok(cudaMemsetAsync(gd_sc, 0, sizeof(float) * sc_floats, s), "zero scatter")) return false;
        if (COUNT && !PACK && !cuda_ok(cudaMemsetAsync(cnt3, 0, sizeof(unsigned int) * nv, s), "zero counter"))
            return false;
        if (a.order == 2) {
            if (!cuda_ok(cudaMemsetAsync(gfwd_sc, 0, sizeof(float) * sc_floats, s), "zero scatter")) return false;
            if (COUNT && !PACK && !cuda_ok(cudaMemsetAsync(cnt2, 0, sizeof(unsigned int) * nv, s), "zero counter"))
                return false;
            if (!forward_ready)  // else fwd holds this slice's semi-Lagrangian grid already
                k_adv_sl<C, float, BM><<<blocks, T, 0, s>>>(db, a.d, a.vx, a.vy, a.vz, a.dt, false, fwd);
            // the fwd adjoint's direct term is the output gradient itself
            // unless the NEGATIVE clamp zeroes parts of it
            const bool neg = a.clamp == CLAMP_NEGATIVE;
            k_adv_bwd_back<C, BM, COUNT><<<blocks, T, 0, s>>>(db, fwd, a.d, a.vx, a.vy, a.vz, a.dt, a.clamp,
                                                                      dyb, gdb, gfwd_sc, cnt2, neg ? gdir : nullptr,
                                                                      glut, b == 0, nullptr, nullptr);
            k_adv_bwd_fwd<C, BM, COUNT><<<blocks, T, 0, s>>>(db, a.d, a.vx, a.vy, a.vz, a.dt, false, false,
                                                                     neg ? gdir : dyb, gfwd_sc, cnt2, gd_sc, cnt3,
                                                                     glut, false,
                                                             nullptr, nullptr, nullptr, nullptr,
                                                             last ? gvx : nullptr, gvy, gvz);
        } else {
            if (!cuda_ok(cudaMemsetAsync(gdb, 0, sizeof(float) * vc, s), "zero gradient")) return false;
            k_adv_bwd_fwd<C, BM, COUNT><<<blocks, T, 0, s>>>(db, a.d, a.vx, a.vy, a.vz, a.dt, true,
                                                                     a.clamp == CLAMP_NEGATIVE, dyb, nullptr,
                                                                     nullptr, gd_sc, cnt3, glut, b == 0, nullptr,
                                                             nullptr, nullptr, nullptr, last ? gvx : nullptr, gvy,
                                                             gvz);
        }
        k_adv_bwd_density<C, COUNT><<<blocks, T, 0, s>>>(gdb, gd_sc, cnt3, nv, nullptr, nullptr);
        if (!launched(a.order == 2 ? (forward_ready ? 3 : 4) : 2, "advect gradient launch")) return false;
    }
    return true;
}

template <int C, int BM>
static bool adv_bwd_bm(const AdvectArgs& a, bool exact, bool fr, const float* dy, float* gd, float* gvx, float* gvy,
                       float* gvz, float* ws, cudaStream_t s) {
    if (a.det) {
        if (exact) return adv_bwd_det<C, BM, 0>(a, fr, dy, gd, gvx, gvy, gvz, ws, s);
        return adv_bwd_det<C, BM, 1>(a, fr, dy, gd, gvx, gvy, gvz, ws, s);
    }
    if (exact) return adv_bwd_impl<C, BM, 0>(a, fr, dy, gd, gvx, gvy, gvz, ws, s);
    if constexpr (C == 1) {
        if ((reinterpret_cast<uintptr_t>(ws) & 7u) == 0) return adv_bwd_impl<C, BM, 2>(a, fr, dy, gd, gvx, gvy, gvz, ws, s);
    }
    return adv_bwd_impl<C, BM, 1>(a, fr, dy, gd, gvx, gvy, gvz, ws, s);
}

template <int C>
static bool adv_bwd_c(const AdvectArgs& a, bool exact, bool fr, const float* dy, float* gd, float* gvx, float* gvy,
                      float* gvz, float* ws, cudaStream_t s) {
    switch (a.boundary) {
        case BM_BORDER: return adv_bwd_bm<C, BM_BORDER>(a, exact, fr, dy, gd, gvx, gvy, gvz, ws, s);
        case BM_CLAMP: return adv_bwd_bm<C, BM_CLAMP>(a, exact, fr, dy, gd, gvx, gvy, gvz, ws, s);
        default: return adv_bwd_bm<C, BM_WRAP>(a, exact, fr, dy, gd, gvx, gvy, gvz, ws, s);
    }
}

bool launch_advect_bwd(const AdvectArgs& a, bool exact, bool forward_ready, const float* dy, float* gd, float* gvx,
                       float* gvy, float* gvz, float* ws, cudaStream_t s) {
    if (!advect_size_ok(a.d)) return false;
    if (a.C == 4) return adv_bwd_c<4>(a, exact, forward_ready, dy, gd, gvx, gvy, gvz, ws, s);
    if (a.C == 2) return adv_bwd_c<2>(a, exact, forward_ready, dy, gd, gvx, gvy, gvz, ws, s);
    return adv_bwd_c<1>(a, exact, forward_ready, dy, gd, gvx, gvy, gvz, ws, s);
}

// ---- allocation-free advection ---------------------------------------------------
// gft_advect_noalloc keeps the intermediate semi-Lagrangian grid of MacCormack
// in this fixed device array instead of a caller-provided workspace.  It holds
// NOALLOC_MAX_ELEMENTS floats (16 MiB); every device that loads the library
// keeps it until the process exits.  Host code cannot pass the array's name to a
// kernel (on the host it is only a stand-in symbol), so its device address is
// looked up with cudaGetSymbolAddress.
constexpr size_t NOALLOC_MAX_ELEMENTS = size_t(1) << 22;
static __device__ __align__(256) float g_noalloc_scratch[NOALLOC_MAX_ELEMENTS];

constexpr int NOALLOC_MAX_DEVICES = 64;
static std::mutex g_noalloc_mu;
static float* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of g_noalloc_scratch on the current device.  Outside stream
// capture the address is looked up on every call (cheap), so a context that
// was reset and reloaded the module never sees a stale pointer; the result is
// cached per device for calls made while `s` is being captured, where the
// lookup (which may load the module) is not made.
static bool noalloc_scratch(cudaStream_t s, float** out) {
    int dev = -1;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return false;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        set_error("gft_advect_noalloc: device ordinal out of range");
        return false;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
        (void)cudaGetLastError();  // reset the last-error state the failed query set
        cap = cudaStreamCaptureStatusActive;  // unknown: do not risk an unsafe call
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (cap != cudaStreamCaptureStatusNone) {
        if (g_noalloc_ptr[dev] == nullptr) {
            set_error("gft_advect_noalloc: first call on this device made during stream capture; "
                      "call it once before capturing");
            return false;
        }
        *out = g_noalloc_ptr[dev];
        return true;
    }
    void* p = nullptr;
    if (!cuda_ok(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(noalloc scratch)"))
        return false;
    g_noalloc_ptr[dev] = reinterpret_cast<float*>(p);
    *out = g_noalloc_ptr[dev];
    return true;
}

}  // namespace gft

extern "C" {

size_t gft_advect_noalloc_max_elements(void) { return gft::NOALLOC_MAX_ELEMENTS; }

gft_status gft_advect_noalloc(const void* density, int32_t density_dtype, const int64_t density_shape[5],
                              const float* vel_x, const float* vel_y, const float* vel_z, float dt, int32_t order,
                              int32_t clamp, int32_t boundary, float* output, void* stream) {
    using namespace gft;
    if (density_shape == nullptr) {
        set_error("density shape is NULL");
        return GFT_ERR_INVALID_ARGUMENT;
    }
    for (int i = 0; i < 5; ++i)
        if (density_shape[i] <= 0) {
            set_error("Invalid input shape (NDHWC): all dimensions must be positive");
            return GFT_ERR_INVALID_ARGUMENT;
        }
    if (density_shape[1] > INT32_MAX || density_shape[2] > INT32_MAX || density_shape[3] > INT32_MAX) {
        set_error("grid dimension too large");
        return GFT_ERR_INVALID_ARGUMENT;
    }
    const int64_t C = density_shape[4];
    if (!(C == 1 || C == 2 || C == 4)) {
        set_error("Only 1,2 and 4 Channel supported.");
        return GFT_ERR_UNIMPLEMENTED;
    }
    if ((order != 1 && order != 2) || clamp < 0 || clamp > 2 || boundary < 0 || boundary > 2 ||
        (density_dtype != GFT_DTYPE_F32 && density_dtype != GFT_DTYPE_BF16)) {
        set_error("gft_advect_noalloc: invalid order, clamp, boundary or dtype");
        return GFT_ERR_INVALID_ARGUMENT;
    }
    if (!density || !vel_x || !vel_y || !vel_z || !output) {
        set_error("tensor pointer is NULL");
        return GFT_ERR_INVALID_ARGUMENT;
    }
    // the density and output are accessed as C-element vectors
    const uintptr_t vin = (uintptr_t)C * (density_dtype == GFT_DTYPE_BF16 ? 2 : 4), vout = (uintptr_t)C * 4;
    if (reinterpret_cast<uintptr_t>(density) % vin != 0 || reinterpret_cast<uintptr_t>(output) % vout != 0 ||
        reinterpret_cast<uintptr_t>(vel_x) % 4 != 0 || reinterpret_cast<uintptr_t>(vel_y) % 4 != 0 ||
        reinterpret_cast<uintptr_t>(vel_z) % 4 != 0) {
        set_error("device pointer not aligned to its channel vector");
        return GFT_ERR_INVALID_ARGUMENT;
    }
    const double elems = (double)density_shape[1] * (double)density_shape[2] * (double)density_shape[3] * (double)C;
    if (order == 2 && elems > (double)NOALLOC_MAX_ELEMENTS) {
        set_error("gft_advect_noalloc: D*H*W*C = " + std::to_string((long long)elems) +
                  " exceeds the built-in scratch of " + std::to_string((long long)NOALLOC_MAX_ELEMENTS) +
                  " floats; use gft_advect with a workspace");
        return GFT_ERR_INVALID_ARGUMENT;
    }
    float* scratch = nullptr;
    if (order == 2 && !noalloc_scratch(reinterpret_cast<cudaStream_t>(stream), &scratch)) return GFT_ERR_CUDA;
    AdvectArgs a;
    a.density = density;
    a.dtype = density_dtype;
    a.N = (int)density_shape[0];
    a.C = (int)C;
    a.d = Dims{(int)density_shape[3], (int)density_shape[2], (int)density_shape[1]};
    a.vx = vel_x;
    a.vy = vel_y;
    a.vz = vel_z;
    a.dt = dt;
    a.order = order;
    a.clamp = clamp;
    a.boundary = boundary;
    if (!launch_advect_fwd(a, output, scratch, reinterpret_cast<cudaStream_t>(stream))) return GFT_ERR_CUDA;
    return GFT_OK;
}

}  // extern "C"
