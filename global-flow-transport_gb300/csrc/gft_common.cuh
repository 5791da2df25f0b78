// Device library shared by all kernels: storage loads, grid fetches with the
// reference's boundary semantics, trilinear scatter, frustum transforms and
// the blend functors.  Written for sm_103a; all arithmetic is fp32.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace gft {

// --- enums (values of the reference, sampling_settings_v2.hpp:9-10) --------
constexpr int BM_BORDER = 0, BM_CLAMP = 1, BM_WRAP = 2;
constexpr int F_NEAREST = 0, F_LINEAR = 1, F_MIN = 2, F_MAX = 3;
constexpr int MIP_NONE = 0, MIP_NEAREST = 1, MIP_LINEAR = 2;
constexpr int BL_BEER_LAMBERT = 0, BL_BEER_LAMBERT_EXCLUSIVE = 1, BL_ALPHA = 2, BL_ALPHA_ADDITIVE = 3,
              BL_ADDITIVE = 4;
// FLOAT_MAX of the reference (vectormath.hpp:13) as a float
constexpr float REF_FLOAT_MAX = 3.40282e38f;

struct Dims {
    int x, y, z;  // W, H, D
};

__host__ __device__ inline int64_t voxels(Dims d) { return (int64_t)d.x * d.y * d.z; }
// Cell index in a grid slice, in 32-bit arithmetic: every launcher limits a
// slice to fewer than 2^32 cells (MAX_SLICE_CELLS), so a cell inside the
// slice gets its exact index (coordinates outside wrap and must not be read).
__device__ __forceinline__ int64_t flat3(int x, int y, int z, Dims d) {
    return (int64_t)(((uint32_t)z * (uint32_t)d.y + (uint32_t)y) * (uint32_t)d.x + (uint32_t)x);
}

// Cell (x, y, z) of a flat index v < 2^32 of a grid of dims d: two 32-bit
// divisions (the per-cell kernels run one grid slice per blockIdx.y).
__device__ __forceinline__ void unflat32(uint32_t v, Dims d, int& x, int& y, int& z) {
    const uint32_t q = v / (uint32_t)d.x;
    x = (int)(v - q * (uint32_t)d.x);
    const uint32_t zz = q / (uint32_t)d.y;
    y = (int)(q - zz * (uint32_t)d.y);
    z = (int)zz;
}
// Brick layout of the per-camera weight sums of the reference-normalised
// raymarch gradient: 2x2x2 voxels per 32-byte sector, bricks in x, y, z order.
// A warp's reduction to one corner of 32 neighbouring rays' samples then
// touches about half as many sectors as with rows of voxels.
__host__ __device__ inline int64_t brick_cells(Dims d) {
    return (int64_t)((d.x + 1) / 2) * ((d.y + 1) / 2) * ((d.z + 1) / 2) * 8;
}
// (32-bit arithmetic, as flat3: brick_cells of a slice stays below 2^32.)
__device__ __forceinline__ int64_t brick_index(int x, int y, int z, Dims d) {
    const uint32_t b = ((uint32_t)(z >> 1) * (uint32_t)((d.y + 1) / 2) + (uint32_t)(y >> 1)) *
                           (uint32_t)((d.x + 1) / 2) + (uint32_t)(x >> 1);
    return (int64_t)(b * 8u + (uint32_t)((z & 1) << 2 | (y & 1) << 1 | (x & 1)));
}

// Cell layouts of a grid slice: rows (NDHWC) or 2x2x2-voxel bricks
// (brick_index; one 128-byte line per brick for C == 4 fp32).
constexpr int LAYOUT_FLAT = 0, LAYOUT_BRICK = 1;
template <int L>
__device__ __forceinline__ int64_t cell_index(int x, int y, int z, Dims d) {
    if constexpr (L == LAYOUT_BRICK) return brick_index(x, y, z, d);
    return flat3(x, y, z, d);
}
template <int L>
__host__ __device__ inline int64_t slice_cells(Dims d) {
    if constexpr (L == LAYOUT_BRICK) return brick_cells(d);
    return voxels(d);
}

// Grid slices up to this many cells run as one launch dimension.
constexpr int64_t MAX_SLICE_CELLS = int64_t(1) << 32;

// --- small fixed-size channel vectors ----------------------------------------
template <int C>
struct Vec {
    float v[C];
};

template <int C>
__device__ __forceinline__ Vec<C> vzero() {
    Vec<C> r;
#pragma unroll
    for (int i = 0; i < C; ++i) r.v[i] = 0.f;
    return r;
}
template <int C>
__device__ __forceinline__ Vec<C> vfill(float a) {
    Vec<C> r;
#pragma unroll
    for (int i = 0; i < C; ++i) r.v[i] = a;
    return r;
}
template <int C>
__device__ __forceinline__ Vec<C> vadd(Vec<C> a, Vec<C> b) {
#pragma unroll
    for (int i = 0; i < C; ++i) a.v[i] += b.v[i];
    return a;
}
template <int C>
__device__ __forceinline__ Vec<C> vscale(Vec<C> a, float s) {
#pragma unroll
    for (int i = 0; i < C; ++i) a.v[i] *= s;
    return a;
}
// lerp(a, b, t) = a + t*(b - a), the reference's lerp (helper_math.h / vectormath.hpp:255)
template <int C>
__device__ __forceinline__ Vec<C> vlerp(Vec<C> a, Vec<C> b, float t) {
#pragma unroll
    for (int i = 0; i < C; ++i) a.v[i] = a.v[i] + t * (b.v[i] - a.v[i]);
    return a;
}
template <int C>
__device__ __forceinline__ Vec<C> vmin(Vec<C> a, Vec<C> b) {
#pragma unroll
    for (int i = 0; i < C; ++i) a.v[i] = fminf(a.v[i], b.v[i]);
    return a;
}
template <int C>
__device__ __forceinline__ Vec<C> vmax(Vec<C> a, Vec<C> b) {
#pragma unroll
    for (int i = 0; i < C; ++i) a.v[i] = fmaxf(a.v[i], b.v[i]);
    return a;
}

// --- storage loads / stores ---------------------------------------------------
__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xffff0000u); }

template <int C, typename S>
struct Load;

template <>
struct Load<4, float> {
    static __device__ __forceinline__ Vec<4> at(const float* p, int64_t i) {
        float4 f = __ldg(reinterpret_cast<const float4*>(p) + i);
        return Vec<4>{{f.x, f.y, f.z, f.w}};
    }
};
template <>
struct Load<2, float> {
    static __device__ __forceinline__ Vec<2> at(const float* p, int64_t i) {
        float2 f = __ldg(reinterpret_cast<const float2*>(p) + i);
        return Vec<2>{{f.x, f.y}};
    }
};
template <>
struct Load<1, float> {
    static __device__ __forceinline__ Vec<1> at(const float* p, int64_t i) { return Vec<1>{{__ldg(p + i)}}; }
};
template <>
struct Load<4, __nv_bfloat16> {
    static __device__ __forceinline__ Vec<4> at(const __nv_bfloat16* p, int64_t i) {
        uint2 w = __ldg(reinterpret_cast<const uint2*>(p) + i);
        return Vec<4>{{bf16_lo(w.x), bf16_hi(w.x), bf16_lo(w.y), bf16_hi(w.y)}};
    }
};
template <>
struct Load<2, __nv_bfloat16> {
    static __device__ __forceinline__ Vec<2> at(const __nv_bfloat16* p, int64_t i) {
        uint32_t w = __ldg(reinterpret_cast<const unsigned int*>(p) + i);
        return Vec<2>{{bf16_lo(w), bf16_hi(w)}};
    }
};
template <>
struct Load<1, __nv_bfloat16> {
    static __device__ __forceinline__ Vec<1> at(const __nv_bfloat16* p, int64_t i) {
        uint32_t w = __ldg(reinterpret_cast<const unsigned short*>(p) + i);
        return Vec<1>{{__uint_as_float(w << 16)}};
    }
};

template <int C>
__device__ __forceinline__ void store(float* p, int64_t i, Vec<C> a) {
    if constexpr (C == 4) {
        reinterpret_cast<float4*>(p)[i] = make_float4(a.v[0], a.v[1], a.v[2], a.v[3]);
    } else if constexpr (C == 2) {
        reinterpret_cast<float2*>(p)[i] = make_float2(a.v[0], a.v[1]);
    } else {
        p[i] = a.v[0];
    }
}
template <int C>
__device__ __forceinline__ Vec<C> loadf(const float* p, int64_t i) {
    return Load<C, float>::at(p, i);
}
// Streaming (evict-first) store and load of data written once and read once
// (st.global.cs / ld.global.cs), so that it does not push reused data out of L2.
template <int C>
__device__ __forceinline__ void store_stream(float* p, int64_t i, Vec<C> a) {
    if constexpr (C == 4) {
        __stcs(reinterpret_cast<float4*>(p) + i, make_float4(a.v[0], a.v[1], a.v[2], a.v[3]));
    } else if constexpr (C == 2) {
        __stcs(reinterpret_cast<float2*>(p) + i, make_float2(a.v[0], a.v[1]));
    } else {
        __stcs(p + i, a.v[0]);
    }
}
template <int C>
__device__ __forceinline__ Vec<C> load_stream(const float* p, int64_t i) {
    if constexpr (C == 4) {
        const float4 f = __ldcs(reinterpret_cast<const float4*>(p) + i);
        return Vec<4>{{f.x, f.y, f.z, f.w}};
    } else if constexpr (C == 2) {
        const float2 f = __ldcs(reinterpret_cast<const float2*>(p) + i);
        return Vec<2>{{f.x, f.y}};
    } else {
        return Vec<1>{{__ldcs(p + i)}};
    }
}

// Atomic add of a channel vector; C == 4 and C == 2 use the sm_90+ vector
// reductions (one red.global.v4/v2.f32 per voxel instead of C scalar ones).
template <int C>
__device__ __forceinline__ void atomic_add(float* p, int64_t i, Vec<C> a) {
    if constexpr (C == 4) {
        atomicAdd(reinterpret_cast<float4*>(p) + i, make_float4(a.v[0], a.v[1], a.v[2], a.v[3]));
    } else if constexpr (C == 2) {
        atomicAdd(reinterpret_cast<float2*>(p) + i, make_float2(a.v[0], a.v[1]));
    } else {
        atomicAdd(p + i, a.v[0]);
    }
}

// --- boundary handling --------------------------------------------------------
__device__ __forceinline__ int pmod(int v, int m) {
    int r = v % m;
    return r < 0 ? r + m : r;
}
template <int BM>
__device__ __forceinline__ int remap(int i, int n) {
    if constexpr (BM == BM_CLAMP) return min(max(i, 0), n - 1);
    if constexpr (BM == BM_WRAP) return pmod(i, n);
    return i;
}

// Corner set of a trilinear footprint (sampling_v2.hpp:38-123): floor and ceil
// indices per axis after the boundary remap, ceil weights fract(p), validity
// (BORDER only; -1 < i < n).
struct Corners {
    int x0, x1, y0, y1, z0, z1;
    float wx, wy, wz;
    bool vx0, vx1, vy0, vy1, vz0, vz1;
};

template <int BM>
__device__ __forceinline__ Corners corners(float px, float py, float pz, Dims d) {
    Corners c;
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    c.wx = px - fx;
    c.wy = py - fy;
    c.wz = pz - fz;
    c.x0 = (int)fx;
    c.y0 = (int)fy;
    c.z0 = (int)fz;
    c.x1 = (int)ceilf(px);
    c.y1 = (int)ceilf(py);
    c.z1 = (int)ceilf(pz);
    if constexpr (BM == BM_BORDER) {
        c.vx0 = c.x0 > -1 && c.x0 < d.x;
        c.vx1 = c.x1 > -1 && c.x1 < d.x;
        c.vy0 = c.y0 > -1 && c.y0 < d.y;
        c.vy1 = c.y1 > -1 && c.y1 < d.y;
        c.vz0 = c.z0 > -1 && c.z0 < d.z;
        c.vz1 = c.z1 > -1 && c.z1 < d.z;
    } else {
        c.x0 = remap<BM>(c.x0, d.x);
        c.x1 = remap<BM>(c.x1, d.x);
        c.y0 = remap<BM>(c.y0, d.y);
        c.y1 = remap<BM>(c.y1, d.y);
        c.z0 = remap<BM>(c.z0, d.z);
        c.z1 = remap<BM>(c.z1, d.z);
        c.vx0 = c.vx1 = c.vy0 = c.vy1 = c.vz0 = c.vz1 = true;
    }
    return c;
}

// BORDER early-out of the fetches: 0 <= p + 0.5 < dims (sampling_v2.hpp:49-51)
__device__ __forceinline__ bool border_inside(float px, float py, float pz, Dims d) {
    const float ax = px + 0.5f, ay = py + 0.5f, az = pz + 0.5f;
    return ax >= 0.f && ax < (float)d.x && ay >= 0.f && ay < (float)d.y && az >= 0.f && az < (float)d.z;
}

template <int C, typename S, int BM, int L = LAYOUT_FLAT>
__device__ __forceinline__ Vec<C> read_corner(const S* g, Dims d, int x, int y, int z, bool ok) {
    if constexpr (BM == BM_BORDER) {
        if (!ok) return vzero<C>();
    }
    return Load<C, S>::at(g, cell_index<L>(x, y, z, d));
}

// Trilinear fetch (read3DInterpolated): p has cell centres at integers; L is
// the cell layout of g.
template <int C, typename S, int BM, int L = LAYOUT_FLAT>
__device__ __forceinline__ Vec<C> fetch_linear(const S* __restrict__ g, Dims d, float px, float py, float pz) {
    if constexpr (BM == BM_BORDER) {
        if (!border_inside(px, py, pz, d)) return vzero<C>();
    }
    {
        // Interior fast path: all eight corners inside the grid, so no boundary
        // remap or validity applies; one base index and constant strides.  The
        // ceil corner is taken as floor + 1: the two differ only where the
        // fraction is 0, where that corner's lerp weight is 0 and
        // a + 0 * (b - a) == a.
        const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
        const int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
        if ((unsigned)x0 < (unsigned)(d.x - 1) && (unsigned)y0 < (unsigned)(d.y - 1) &&
            (unsigned)z0 < (unsigned)(d.z - 1)) {
            const float wx = px - fx, wy = py - fy, wz = pz - fz;
            // 32-bit cell indices: every caller limits a grid slice to 2^32 cells
            uint32_t i000, i100, i010, i110, i001, i101, i011, i111;
            if constexpr (L == LAYOUT_BRICK) {
                // brick index = x term + y term + z term (brick_index)
                const uint32_t bx = (uint32_t)(d.x + 1) / 2, bxy = bx * ((uint32_t)(d.y + 1) / 2);
                const uint32_t x1 = x0 + 1, y1 = y0 + 1, z1 = z0 + 1;
                const uint32_t tx0 = (uint32_t)(x0 >> 1) * 8u + (x0 & 1), tx1 = (x1 >> 1) * 8u + (x1 & 1);
                const uint32_t ty0 = (uint32_t)(y0 >> 1) * bx * 8u + ((y0 & 1) << 1);
                const uint32_t ty1 = (y1 >> 1) * bx * 8u + ((y1 & 1) << 1);
                const uint32_t tz0 = (uint32_t)(z0 >> 1) * bxy * 8u + ((z0 & 1) << 2);
                const uint32_t tz1 = (z1 >> 1) * bxy * 8u + ((z1 & 1) << 2);
                i000 = tz0 + ty0 + tx0;
                i100 = tz0 + ty0 + tx1;
                i010 = tz0 + ty1 + tx0;
                i110 = tz0 + ty1 + tx1;
                i001 = tz1 + ty0 + tx0;
                i101 = tz1 + ty0 + tx1;
                i011 = tz1 + ty1 + tx0;
                i111 = tz1 + ty1 + tx1;
            } else {
                const uint32_t sy = d.x, sz = (uint32_t)d.x * d.y;
                i000 = ((uint32_t)z0 * d.y + y0) * d.x + x0;
                i100 = i000 + 1;
                i010 = i000 + sy;
                i110 = i000 + sy + 1;
                i001 = i000 + sz;
                i101 = i000 + sz + 1;
                i011 = i000 + sz + sy;
                i111 = i000 + sz + sy + 1;
            }
            const Vec<C> fff = Load<C, S>::at(g, i000), cff = Load<C, S>::at(g, i100);
            const Vec<C> fcf = Load<C, S>::at(g, i010), ccf = Load<C, S>::at(g, i110);
            const Vec<C> ffc = Load<C, S>::at(g, i001), cfc = Load<C, S>::at(g, i101);
            const Vec<C> fcc = Load<C, S>::at(g, i011), ccc = Load<C, S>::at(g, i111);
            const Vec<C> v0 = vlerp(vlerp(fff, cff, wx), vlerp(fcf, ccf, wx), wy);
            const Vec<C> v1 = vlerp(vlerp(ffc, cfc, wx), vlerp(fcc, ccc, wx), wy);
            return vlerp(v0, v1, wz);
        }
    }
    const Corners c = corners<BM>(px, py, pz, d);
    const Vec<C> fff = read_corner<C, S, BM, L>(g, d, c.x0, c.y0, c.z0, c.vx0 && c.vy0 && c.vz0);
    const Vec<C> cff = read_corner<C, S, BM, L>(g, d, c.x1, c.y0, c.z0, c.vx1 && c.vy0 && c.vz0);
    const Vec<C> fcf = read_corner<C, S, BM, L>(g, d, c.x0, c.y1, c.z0, c.vx0 && c.vy1 && c.vz0);
    const Vec<C> ccf = read_corner<C, S, BM, L>(g, d, c.x1, c.y1, c.z0, c.vx1 && c.vy1 && c.vz0);
    const Vec<C> ffc = read_corner<C, S, BM, L>(g, d, c.x0, c.y0, c.z1, c.vx0 && c.vy0 && c.vz1);
    const Vec<C> cfc = read_corner<C, S, BM, L>(g, d, c.x1, c.y0, c.z1, c.vx1 && c.vy0 && c.vz1);
    const Vec<C> fcc = read_corner<C, S, BM, L>(g, d, c.x0, c.y1, c.z1, c.vx0 && c.vy1 && c.vz1);
    const Vec<C> ccc = read_corner<C, S, BM, L>(g, d, c.x1, c.y1, c.z1, c.vx1 && c.vy1 && c.vz1);
    const Vec<C> v0 = vlerp(vlerp(fff, cff, c.wx), vlerp(fcf, ccf, c.wx), c.wy);
    const Vec<C> v1 = vlerp(vlerp(ffc, cfc, c.wx), vlerp(fcc, ccc, c.wx), c.wy);
    return vlerp(v0, v1, c.wz);
}

// Nearest fetch (read3DNearest): idx = int(p + 0.5), truncating toward zero.
template <int C, typename S, int BM>
__device__ __forceinline__ Vec<C> fetch_nearest(const S* __restrict__ g, Dims d, float px, float py, float pz) {
    int ix = (int)(px + 0.5f), iy = (int)(py + 0.5f), iz = (int)(pz + 0.5f);
    if constexpr (BM == BM_BORDER) {
        if (!(ix >= 0 && ix < d.x && iy >= 0 && iy < d.y && iz >= 0 && iz < d.z)) return vzero<C>();
    } else {
        ix = remap<BM>(ix, d.x);
        iy = remap<BM>(iy, d.y);
        iz = remap<BM>(iz, d.z);
    }
    return Load<C, S>::at(g, flat3(ix, iy, iz, d));
}

// MIN/MAX over the 8 corners.  RAYMARCH=true: read3DInterpolatedWithExtrema
// (sampling_v2.hpp:149-256): running extremum from +-FLOAT_MAX, updated per
// valid corner (order fff, cff, fcf, ccf, ffc, cfc, fcc, ccc) as
// m = m + t*(v - m) with t = (v < m) resp. (m < v); the first update cancels
// against FLOAT_MAX to 0 exactly as in the reference; the start value outside
// the BORDER domain.  RAYMARCH=false: read3DMin/Max (sampling.hpp:372-491),
// 0 outside, and a start of 0 when any corner is invalid.
template <int C, typename S, int BM, bool IS_MAX, bool RAYMARCH>
__device__ __forceinline__ Vec<C> fetch_extremum(const S* __restrict__ g, Dims d, float px, float py, float pz) {
    const float start = IS_MAX ? -REF_FLOAT_MAX : REF_FLOAT_MAX;
    if constexpr (BM == BM_BORDER) {
        if (!border_inside(px, py, pz, d)) return vfill<C>(RAYMARCH ? start : 0.f);
    }
    const Corners c = corners<BM>(px, py, pz, d);
    const bool ok[8] = {c.vx0 && c.vy0 && c.vz0, c.vx1 && c.vy0 && c.vz0, c.vx0 && c.vy1 && c.vz0,
                        c.vx1 && c.vy1 && c.vz0, c.vx0 && c.vy0 && c.vz1, c.vx1 && c.vy0 && c.vz1,
                        c.vx0 && c.vy1 && c.vz1, c.vx1 && c.vy1 && c.vz1};
    const int xs[8] = {c.x0, c.x1, c.x0, c.x1, c.x0, c.x1, c.x0, c.x1};
    const int ys[8] = {c.y0, c.y0, c.y1, c.y1, c.y0, c.y0, c.y1, c.y1};
    const int zs[8] = {c.z0, c.z0, c.z0, c.z0, c.z1, c.z1, c.z1, c.z1};
    bool all_ok = true;
#pragma unroll
    for (int k = 0; k < 8; ++k) all_ok = all_ok && ok[k];
    Vec<C> acc = vfill<C>((!RAYMARCH && !all_ok) ? 0.f : start);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        if (ok[k]) {
            const Vec<C> v = Load<C, S>::at(g, flat3(xs[k], ys[k], zs[k], d));
            if constexpr (RAYMARCH) {
#pragma unroll
                for (int i = 0; i < C; ++i) {
                    const float t = (IS_MAX ? (acc.v[i] < v.v[i]) : (v.v[i] < acc.v[i])) ? 1.f : 0.f;
                    acc.v[i] = acc.v[i] + t * (v.v[i] - acc.v[i]);
                }
            } else {
                acc = IS_MAX ? vmax(acc, v) : vmin(acc, v);
            }
        }
    }
    return acc;
}

template <int C, typename S, int BM, bool RAYMARCH>
__device__ __forceinline__ Vec<C> fetch(int filter, const S* __restrict__ g, Dims d, float px, float py, float pz) {
    switch (filter) {
        case F_LINEAR: return fetch_linear<C, S, BM>(g, d, px, py, pz);
        case F_NEAREST: return fetch_nearest<C, S, BM>(g, d, px, py, pz);
        case F_MIN: return fetch_extremum<C, S, BM, false, RAYMARCH>(g, d, px, py, pz);
        case F_MAX: return fetch_extremum<C, S, BM, true, RAYMARCH>(g, d, px, py, pz);
        default: return vzero<C>();
    }
}

// Spatial derivative of the trilinear fetch (read3DGrad, sampling.hpp:257-352).
template <int C, int BM>
__device__ __forceinline__ void fetch_grad(const float* __restrict__ g, Dims d, float px, float py, float pz,
                                           Vec<C>& dx, Vec<C>& dy, Vec<C>& dz) {
    if constexpr (BM == BM_BORDER) {
        if (!border_inside(px, py, pz, d)) {
            dx = dy = dz = vzero<C>();
            return;
        }
    }
    const Corners c = corners<BM>(px, py, pz, d);
    const Vec<C> fff = read_corner<C, float, BM>(g, d, c.x0, c.y0, c.z0, c.vx0 && c.vy0 && c.vz0);
    const Vec<C> cff = read_corner<C, float, BM>(g, d, c.x1, c.y0, c.z0, c.vx1 && c.vy0 && c.vz0);
    const Vec<C> fcf = read_corner<C, float, BM>(g, d, c.x0, c.y1, c.z0, c.vx0 && c.vy1 && c.vz0);
    const Vec<C> ccf = read_corner<C, float, BM>(g, d, c.x1, c.y1, c.z0, c.vx1 && c.vy1 && c.vz0);
    const Vec<C> ffc = read_corner<C, float, BM>(g, d, c.x0, c.y0, c.z1, c.vx0 && c.vy0 && c.vz1);
    const Vec<C> cfc = read_corner<C, float, BM>(g, d, c.x1, c.y0, c.z1, c.vx1 && c.vy0 && c.vz1);
    const Vec<C> fcc = read_corner<C, float, BM>(g, d, c.x0, c.y1, c.z1, c.vx0 && c.vy1 && c.vz1);
    const Vec<C> ccc = read_corner<C, float, BM>(g, d, c.x1, c.y1, c.z1, c.vx1 && c.vy1 && c.vz1);
#pragma unroll
    for (int i = 0; i < C; ++i) {
        auto L = [](float a, float b, float t) { return a + t * (b - a); };
        dx.v[i] = L(L(cff.v[i] - fff.v[i], ccf.v[i] - fcf.v[i], c.wy), L(cfc.v[i] - ffc.v[i], ccc.v[i] - fcc.v[i], c.wy), c.wz);
        dy.v[i] = L(L(fcf.v[i] - fff.v[i], ccf.v[i] - cff.v[i], c.wx), L(fcc.v[i] - ffc.v[i], ccc.v[i] - cfc.v[i], c.wx), c.wz);
        dz.v[i] = L(L(ffc.v[i] - fff.v[i], cfc.v[i] - cff.v[i], c.wx), L(fcc.v[i] - fcf.v[i], ccc.v[i] - ccf.v[i], c.wx), c.wy);
    }
}

// Trilinear value and its spatial derivative from one set of corner reads:
// the value of fetch_linear and the derivative of fetch_grad (ceil corners, as
// read3DGrad; the value is the same, a zero fraction giving a zero weight).
template <int C, int BM>
__device__ __forceinline__ void fetch_linear_grad(const float* __restrict__ g, Dims d, float px, float py, float pz,
                                                  Vec<C>& val, Vec<C>& dx, Vec<C>& dy, Vec<C>& dz) {
    if constexpr (BM == BM_BORDER) {
        if (!border_inside(px, py, pz, d)) {
            val = dx = dy = dz = vzero<C>();
            return;
        }
    }
    const Corners c = corners<BM>(px, py, pz, d);
    const Vec<C> fff = read_corner<C, float, BM>(g, d, c.x0, c.y0, c.z0, c.vx0 && c.vy0 && c.vz0);
    const Vec<C> cff = read_corner<C, float, BM>(g, d, c.x1, c.y0, c.z0, c.vx1 && c.vy0 && c.vz0);
    const Vec<C> fcf = read_corner<C, float, BM>(g, d, c.x0, c.y1, c.z0, c.vx0 && c.vy1 && c.vz0);
    const Vec<C> ccf = read_corner<C, float, BM>(g, d, c.x1, c.y1, c.z0, c.vx1 && c.vy1 && c.vz0);
    const Vec<C> ffc = read_corner<C, float, BM>(g, d, c.x0, c.y0, c.z1, c.vx0 && c.vy0 && c.vz1);
    const Vec<C> cfc = read_corner<C, float, BM>(g, d, c.x1, c.y0, c.z1, c.vx1 && c.vy0 && c.vz1);
    const Vec<C> fcc = read_corner<C, float, BM>(g, d, c.x0, c.y1, c.z1, c.vx0 && c.vy1 && c.vz1);
    const Vec<C> ccc = read_corner<C, float, BM>(g, d, c.x1, c.y1, c.z1, c.vx1 && c.vy1 && c.vz1);
    const Vec<C> v0 = vlerp(vlerp(fff, cff, c.wx), vlerp(fcf, ccf, c.wx), c.wy);
    const Vec<C> v1 = vlerp(vlerp(ffc, cfc, c.wx), vlerp(fcc, ccc, c.wx), c.wy);
    val = vlerp(v0, v1, c.wz);
#pragma unroll
    for (int i = 0; i < C; ++i) {
        auto L = [](float a, float b, float t) { return a + t * (b - a); };
        dx.v[i] = L(L(cff.v[i] - fff.v[i], ccf.v[i] - fcf.v[i], c.wy), L(cfc.v[i] - ffc.v[i], ccc.v[i] - fcc.v[i], c.wy), c.wz);
        dy.v[i] = L(L(fcf.v[i] - fff.v[i], ccf.v[i] - cff.v[i], c.wx), L(fcc.v[i] - ffc.v[i], ccc.v[i] - cfc.v[i], c.wx), c.wz);
        dz.v[i] = L(L(ffc.v[i] - fff.v[i], cfc.v[i] - cff.v[i], c.wx), L(fcc.v[i] - fcf.v[i], ccc.v[i] - ccf.v[i], c.wx), c.wy);
    }
}

// Trilinear scatter (scatterGradInterpolated, resample_grid.cu.cc:760-812 and
// sampling_v2.hpp:458-484).  COUNT: 0 none, 1 +1 per reached corner (uint32
// counter), 2 +w per reached corner (float counter).  With a counter (the
// reference-normalised gradients) BORDER drops the sample unless -1 < p < dims,
// the reference's window, which is wider than the forward's support; without a
// counter (exact adjoints) it drops it outside the forward's half-cell window.
// Corners outside [0, dims) are always dropped under BORDER.
template <int C, int BM, int COUNT>
__device__ __forceinline__ void scatter_linear(float* __restrict__ grad, void* __restrict__ count, Dims d, float px,
                                               float py, float pz, Vec<C> val) {
    if constexpr (BM == BM_BORDER) {
        if constexpr (COUNT == 0) {
            if (!border_inside(px, py, pz, d)) return;
        } else {
            if (!(px > -1.f && px < (float)d.x && py > -1.f && py < (float)d.y && pz > -1.f && pz < (float)d.z))
                return;
        }
    }
    const Corners c = corners<BM>(px, py, pz, d);
    const float cw[3] = {c.wx, c.wy, c.wz};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int sx = k & 1, sy = (k >> 1) & 1, sz = (k >> 2) & 1;
        const bool ok = (sx ? c.vx1 : c.vx0) && (sy ? c.vy1 : c.vy0) && (sz ? c.vz1 : c.vz0);
        if (BM != BM_BORDER || ok) {
            const float w = (sx ? cw[0] : 1.f - cw[0]) * (sy ? cw[1] : 1.f - cw[1]) * (sz ? cw[2] : 1.f - cw[2]);
            const int64_t f = flat3(sx ? c.x1 : c.x0, sy ? c.y1 : c.y0, sz ? c.z1 : c.z0, d);
            atomic_add<C>(grad, f, vscale(val, w));
            if constexpr (COUNT == 1) atomicAdd(reinterpret_cast<unsigned int*>(count) + f, 1u);
            if constexpr (COUNT == 2) atomicAdd(reinterpret_cast<float*>(count) + f, w);
        }
    }
}

// --- frustum transforms (transformations_v2.hpp:69-136) ----------------------
struct Mat4 {
    float4 r0, r1, r2, r3;  // rows of the column-vector matrix
};
__device__ __forceinline__ float4 mul(const Mat4& m, float4 v) {
    return make_float4(m.r0.x * v.x + m.r0.y * v.y + m.r0.z * v.z + m.r0.w * v.w,
                       m.r1.x * v.x + m.r1.y * v.y + m.r1.z * v.z + m.r1.w * v.w,
                       m.r2.x * v.x + m.r2.y * v.y + m.r2.z * v.z + m.r2.w * v.w,
                       m.r3.x * v.x + m.r3.y * v.y + m.r3.z * v.z + m.r3.w * v.w);
}
// h + s * (column j of m)
template <int J>
__device__ __forceinline__ float4 add_col(float4 h, const Mat4& m, float s) {
    const float a = J == 0 ? m.r0.x : J == 1 ? m.r0.y : m.r0.z;
    const float b = J == 0 ? m.r1.x : J == 1 ? m.r1.y : m.r1.z;
    const float c = J == 0 ? m.r2.x : J == 1 ? m.r2.y : m.r2.z;
    const float d = J == 0 ? m.r3.x : J == 1 ? m.r3.y : m.r3.z;
    return make_float4(fmaf(a, s, h.x), fmaf(b, s, h.y), fmaf(c, s, h.z), fmaf(d, s, h.w));
}
__device__ __forceinline__ float3 dehom(float4 h) {
    const float iw = 1.f / h.w;
    return make_float3(h.x * iw, h.y * iw, h.z * iw);
}

// Per (model, camera) constants: MV = V*M, the inverses of MV and P, and two
// products folded on the host in double precision:
//   q (NDC -> OS): rows 0-2 are those of MV^-1 * P^-1, row 3 is row 3 of P^-1,
//     so OS = (q ndc).xyz / (q ndc).w equals MV^-1 (P^-1 ndc / w) for any MV;
//   r (OS -> clip) = P * MV.
// Sample positions use the reference's operation sequence (two products, four
// divisions) so that they round exactly as the reference's: its count
// normalisation and NEAREST lookups jump where a position is integral.  The
// folded forms serve the LOD's finite differences, which vary continuously.
struct CamX {
    Mat4 mv, mv_inv, p, p_inv, q, r;
    float near_, far_, p22, p23;  // frustum near/far, P[2][2], P[2][3]
};

__device__ __forceinline__ float4 ndc_to_os(const CamX& c, float4 ndc) {
    float4 vs = mul(c.p_inv, ndc);
    const float iw = vs.w;
    vs = make_float4(vs.x / iw, vs.y / iw, vs.z / iw, vs.w / iw);
    return mul(c.mv_inv, vs);
}
__device__ __forceinline__ float4 idx_to_ndc(float3 idx, float3 dims_inv) {
    return make_float4(idx.x * dims_inv.x * 2.f - 1.f, idx.y * dims_inv.y * 2.f - 1.f, idx.z * dims_inv.z * 2.f - 1.f,
                       1.f);
}
// NDC depth of the linear-depth coordinate t = idx.z / dims.z (view depth
// linear between near and far).
__device__ __forceinline__ float lindepth_ndc_z(const CamX& c, float idx_z, float dinv_z) {
    const float t = idx_z * dinv_z;
    const float z = -(c.near_ + t * (c.far_ - c.near_));
    return -c.p22 - c.p23 / z;
}
// IDXtoOS: idx -> NDC = idx*dims_inv*2-1 -> VS -> OS
__device__ __forceinline__ float3 idx_to_os(const CamX& c, float3 idx, float3 dims_inv) {
    const float4 o = ndc_to_os(c, idx_to_ndc(idx, dims_inv));
    return make_float3(o.x, o.y, o.z);
}
// IDXtoOSlinearDepth
__device__ __forceinline__ float3 idx_to_os_lindepth(const CamX& c, float3 idx, float3 dims_inv) {
    float4 ndc = idx_to_ndc(idx, dims_inv);
    ndc.z = lindepth_ndc_z(c, idx.z, dims_inv.z);
    const float4 o = ndc_to_os(c, ndc);
    return make_float3(o.x, o.y, o.z);
}
__device__ __forceinline__ float4 os_to_ndc(const CamX& c, float3 p) {
    const float4 vs = mul(c.mv, make_float4(p.x, p.y, p.z, 1.f));
    float4 n = mul(c.p, vs);
    const float iw = n.w;
    return make_float4(n.x / iw, n.y / iw, n.z / iw, n.w / iw);
}
// NDC -> idx of a frustum grid of the given dims; LIN: linear-depth z
template <bool LIN>
__device__ __forceinline__ float3 ndc_to_idx(const CamX& c, float3 n, float3 dims) {
    float3 idx = make_float3((n.x * 0.5f + 0.5f) * dims.x, (n.y * 0.5f + 0.5f) * dims.y, (n.z * 0.5f + 0.5f) * dims.z);
    if constexpr (LIN) {
        const float z = -c.p23 / (n.z + c.p22);
        const float t = -(z + c.near_) / (c.far_ - c.near_);
        idx.z = t * dims.z;
    }
    return idx;
}
// OStoIDX
__device__ __forceinline__ float3 os_to_idx(const CamX& c, float3 p, float3 dims) {
    const float4 n = os_to_ndc(c, p);
    return ndc_to_idx<false>(c, make_float3(n.x, n.y, n.z), dims);
}
// OStoIDXlinearDepth
__device__ __forceinline__ float3 os_to_idx_lindepth(const CamX& c, float3 p, float3 dims) {
    const float4 n = os_to_ndc(c, p);
    return ndc_to_idx<true>(c, make_float3(n.x, n.y, n.z), dims);
}

// --- blend functors (blending.hpp:10-221) -------------------------------------
// One front-to-back step.  C == 1 uses the generic additive template for every
// mode, as the reference (only float2/float4 are specialised).
template <int C>
__device__ __forceinline__ Vec<C> blend(int mode, Vec<C> acc, const Vec<C>& s) {
    if constexpr (C == 1) {
        acc.v[0] += s.v[0];
        return acc;
    } else {
        constexpr int W = C - 1;  // density / opacity channel
        switch (mode) {
            case BL_BEER_LAMBERT: {
                const float dd = fmaxf(acc.v[W] + s.v[W], 0.f);
                const float t = expf(-dd);
#pragma unroll
                for (int i = 0; i < W; ++i) acc.v[i] = acc.v[i] + t * s.v[i];
                acc.v[W] = dd;
                return acc;
            }
            case BL_BEER_LAMBERT_EXCLUSIVE: {
                const float t = expf(-acc.v[W]);
#pragma unroll
                for (int i = 0; i < W; ++i) acc.v[i] = acc.v[i] + t * s.v[i];
                acc.v[W] = acc.v[W] + s.v[W];
                return acc;
            }
            case BL_ALPHA: {
                const float t = 1.f - acc.v[W];
#pragma unroll
                for (int i = 0; i < W; ++i) acc.v[i] = acc.v[i] + t * s.v[i];
                acc.v[W] = acc.v[W] + t * s.v[W];
                return acc;
            }
            case BL_ALPHA_ADDITIVE: {
                const float t = 1.f - s.v[W];
#pragma unroll
                for (int i = 0; i < W; ++i) acc.v[i] = acc.v[i] + t * s.v[i];
                acc.v[W] = acc.v[W] + s.v[W];
                return acc;
            }
            default:
                return vadd(acc, s);
        }
    }
}

// One back-to-front adjoint step (blendGradients).  g: adjoint of the
// accumulator after this cell (updated to the one before it); out: the
// accumulator after this cell (updated to the one before it).  Returns the
// gradient of the cell.  exact=false reproduces the reference formulas; exact
// only changes ALPHA, whose reference bookkeeping is not the adjoint.
template <int C>
__device__ __forceinline__ Vec<C> blend_grad(int mode, bool exact, Vec<C>& g, const Vec<C>& s, Vec<C>& out) {
    if constexpr (C == 1) {
        out.v[0] -= s.v[0];
        return g;
    } else {
        constexpr int W = C - 1;
        Vec<C> gc;
        float dot = 0.f;
#pragma unroll
        for (int i = 0; i < W; ++i) dot += s.v[i] * g.v[i];
        switch (mode) {
            case BL_BEER_LAMBERT: {
                const float e = expf(-out.v[W]);
                out.v[W] = fmaxf(out.v[W] - s.v[W], 0.f);
                const float dd = g.v[W] - e * dot;
#pragma unroll
                for (int i = 0; i < W; ++i) gc.v[i] = e * g.v[i];
                gc.v[W] = dd;
                g.v[W] = dd;
                return gc;
            }
            case BL_BEER_LAMBERT_EXCLUSIVE: {
                out.v[W] = fmaxf(out.v[W] - s.v[W], 0.f);
                const float e = expf(-out.v[W]);
                const float dd = g.v[W] - e * dot;
#pragma unroll
                for (int i = 0; i < W; ++i) gc.v[i] = e * g.v[i];
                gc.v[W] = g.v[W];
                g.v[W] = dd;
                return gc;
            }
            case BL_ALPHA: {
                const float tprev = (1.f - out.v[W]) / (1.f - s.v[W]);
                const float t = exact ? tprev : 1.f - tprev;
                out.v[W] = exact ? 1.f - tprev : tprev;
                const float dd = (1.f - s.v[W]) * g.v[W] - dot;
#pragma unroll
                for (int i = 0; i < W; ++i) gc.v[i] = t * g.v[i];
                gc.v[W] = t * g.v[W];
                g.v[W] = dd;
                return gc;
            }
            case BL_ALPHA_ADDITIVE: {
                out.v[W] = out.v[W] - s.v[W];
                const float t = 1.f - s.v[W];
#pragma unroll
                for (int i = 0; i < W; ++i) gc.v[i] = t * g.v[i];
                gc.v[W] = g.v[W] - dot;
                return gc;
            }
            default:
#pragma unroll
                for (int i = 0; i < C; ++i) out.v[i] -= s.v[i];
                return g;
        }
    }
}

}  // namespace gft
