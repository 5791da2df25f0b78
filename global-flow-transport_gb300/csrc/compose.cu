// Fused kernels for the glue of the render + advect step, each replacing a
// chain of elementwise / reduction tensor ops of the reference's renderer
// (phitest/render/renderer.py and lighting.py compose them from TF ops):
//
//   transmittance    tr[z] = exp(-sum_{z' < z} s[z'])  -- ReduceGridBlend
//                    BEER_LAMBERT (C == 1, inclusive depth sum), the one-cell
//                    BORDER shift and exp of the shadow pass
//                    (lighting.py:236-262), a segmented depth scan;
//   light compose    out = concat(d * (tr * color + ambient), d) * scale
//                    (lighting.py:106-121, renderer.py:1012-1030);
//   image loss       mean((tone(img.rgb + bkg * exp(-img.a)) - target)^2) with
//                    its background composite and tonemapping
//                    (renderer.py:528-541, :632-640, :1048-1052).
//
// Elementwise products and sums use __fmul_rn / __fadd_rn so that they round
// exactly like the separate tensor ops they replace (no FMA contraction).
#include <algorithm>
#include <type_traits>

#include "gft_internal.h"

namespace gft {

constexpr int CP_THREADS = 256;

static unsigned grid_for(int64_t n, int threads) {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (n + threads - 1) / threads, cap = (int64_t)std::max(sms, 1) * 16;
    return (unsigned)std::max<int64_t>(1, std::min(want, cap));
}

// --- transmittance -------------------------------------------------------------
// Forward: tr[z] = exp(-sum_{z' < z} s[z']).  Adjoint (REVERSE): d tr[z] /
// d s[z'] = -tr[z] for z' < z, so gs[z] = sum_{z'' > z} -tr[z''] g[z''].
// Both scans run segmented: a block of 32 consecutive columns x 8 depth
// segments; each thread scans its segment, the segment totals are exchanged
// through shared memory, and each thread starts from the total of the
// segments before (REVERSE: after) its own.  (The 196x196 columns of the
// shadow frustum alone would give one thread per column too few threads to
// hide the latency of 256 dependent steps.)  The sums associate differently
// from a sequential scan: rounding only.
// TS_SEGS: 4, 8 (default) or 16 segments, GFT_KNOB_SCAN_SEGMENTS.
constexpr int TS_COLS = 32;

template <bool REVERSE, int TS_SEGS>
__global__ void __launch_bounds__(TS_COLS* TS_SEGS)
    k_transmittance_seg(const float* __restrict__ a, const float* __restrict__ b, int N, Dims d,
                        float* __restrict__ out) {
    __shared__ float tot[TS_SEGS][TS_COLS];
    const int64_t plane = (int64_t)d.x * d.y;
    const int64_t col = (int64_t)blockIdx.x * TS_COLS + threadIdx.x;
    const int seg = threadIdx.y;
    const bool ok = col < plane * N;
    const int bb = ok ? (int)(col / plane) : 0;
    const int64_t base = (int64_t)bb * plane * d.z + (col - (int64_t)bb * plane);
    const int len = (d.z + TS_SEGS - 1) / TS_SEGS;
    const int z0 = seg * len, z1 = min(z0 + len, d.z);
    // value of one depth step: the density (forward) or -tr * g (adjoint)
    auto val = [&](int z) {
        const int64_t i = base + (int64_t)z * plane;
        return REVERSE ? -__fmul_rn(b[i], a[i]) : a[i];
    };
    float s = 0.f;
    if (ok) {
        for (int z = z0; z < z1; ++z) s = __fadd_rn(s, val(z));
    }
    tot[seg][threadIdx.x] = s;
    __syncthreads();
    if (!ok) return;
    float off = 0.f;
    if (!REVERSE) {
        for (int k = 0; k < seg; ++k) off = __fadd_rn(off, tot[k][threadIdx.x]);
        float acc = off;
        for (int z = z0; z < z1; ++z) {
            const int64_t i = base + (int64_t)z * plane;
            out[i] = expf(-acc);
            acc = __fadd_rn(acc, a[i]);
        }
    } else {
        for (int k = TS_SEGS - 1; k > seg; --k) off = __fadd_rn(off, tot[k][threadIdx.x]);
        float acc = off;
        for (int z = z1 - 1; z >= z0; --z) {
            const int64_t i = base + (int64_t)z * plane;
            out[i] = acc;
            acc = __fadd_rn(acc, val(z));
        }
    }
}

template <bool REVERSE>
static void scan_launch(const float* a, const float* b, int N, Dims d, float* out, cudaStream_t st) {
    const int64_t cols = (int64_t)d.x * d.y * N;
    const unsigned blocks = (unsigned)((cols + TS_COLS - 1) / TS_COLS);
    switch (knob_value(GFT_KNOB_SCAN_SEGMENTS)) {
        case 4: k_transmittance_seg<REVERSE, 4><<<blocks, dim3(TS_COLS, 4), 0, st>>>(a, b, N, d, out); break;
        case 16: k_transmittance_seg<REVERSE, 16><<<blocks, dim3(TS_COLS, 16), 0, st>>>(a, b, N, d, out); break;
        default: k_transmittance_seg<REVERSE, 8><<<blocks, dim3(TS_COLS, 8), 0, st>>>(a, b, N, d, out); break;
    }
}

bool launch_transmittance(const float* s, int N, Dims d, float* out, cudaStream_t st) {
    scan_launch<false>(s, nullptr, N, d, out, st);
    return launched(1, "transmittance launch");
}

// tr, g: the forward output and its adjoint
bool launch_transmittance_grad(const float* tr, const float* g, int N, Dims d, float* gs, cudaStream_t st) {
    scan_launch<true>(tr, g, N, d, gs, st);
    return launched(1, "transmittance gradient launch");
}

// --- light compose ---------------------------------------------------------------
// density, tr [N, V] (V voxels per batch slice, rows), color [V, 3] shared by
// all slices; out [N, cells, 4] in layout L (rows, or the raymarch's bricks).
// One batch slice per blockIdx.y.
template <typename T>
__device__ __forceinline__ void store_cell(T* out, int64_t o, float r, float g, float b, float a) {
    if constexpr (std::is_same<T, float>::value) {
        reinterpret_cast<float4*>(out)[o] = make_float4(r, g, b, a);
    } else {
        __nv_bfloat162 h[2] = {__floats2bfloat162_rn(r, g), __floats2bfloat162_rn(b, a)};
        reinterpret_cast<uint2*>(out)[o] = *reinterpret_cast<const uint2*>(h);
    }
}

// T: the output's storage type (float, or bf16 rounded to nearest even as a
// separate conversion would round the fp32 result).
// FACT (a factored light): color[v, c] = falloff[v] * rgb[c], formed here by
// the same single rounded product as a precomputed colour grid.
struct Rgb {
    float c[3];
};

template <int L, typename T, bool FACT>
__global__ void __launch_bounds__(CP_THREADS)
    k_light_compose(const float* __restrict__ dens, const float* __restrict__ tr, const float* __restrict__ color,
                    const Rgb rgb, Dims d, float ambient, float scale, T* __restrict__ out) {
    const int64_t nvox = voxels(d), b = blockIdx.y;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = b * nvox + v;
        const float dv = dens[i], t = tr[i];
        const float fv = FACT ? color[v] : 0.f;
        float r[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float col = FACT ? __fmul_rn(fv, rgb.c[c]) : color[v * 3 + c];
            const float lc = __fmul_rn(dv, __fadd_rn(__fmul_rn(t, col), ambient));
            r[c] = __fmul_rn(lc, scale);
        }
        int64_t o = i;
        if constexpr (L == LAYOUT_BRICK) {
            int x, y, z;
            unflat32((uint32_t)v, d, x, y, z);
            o = b * brick_cells(d) + brick_index(x, y, z, d);
        }
        const float a = __fmul_rn(dv, scale);
        store_cell<T>(out, o, r[0], r[1], r[2], a);
        if constexpr (L == LAYOUT_BRICK) {
            // the bricks of an odd-sized axis end in a padding cell: the cell
            // at the last index writes zeros there (the sample store's
            // occupancy map reads whole bricks)
            int x, y, z;
            unflat32((uint32_t)v, d, x, y, z);
            const int px = (x == d.x - 1 && (d.x & 1)) ? 1 : 0, py = (y == d.y - 1 && (d.y & 1)) ? 1 : 0,
                      pz = (z == d.z - 1 && (d.z & 1)) ? 1 : 0;
            if (px | py | pz) {
                const int64_t base = b * brick_cells(d);
                for (int k = 1; k < 8; ++k) {
                    const int sx = k & 1, sy = (k >> 1) & 1, sz = (k >> 2) & 1;
                    if ((sx && !px) || (sy && !py) || (sz && !pz)) continue;
                    store_cell<T>(out, base + brick_index(x + sx, y + sy, z + sz, d), 0.f, 0.f, 0.f, 0.f);
                }
            }
        }
    }
}

// g_d = g3 * s + sum_c (g_c * s) * (t * color_c + ambient);
// g_t = sum_c (g_c * s) * d * color_c.  g in layout L.
template <int L>
__global__ void __launch_bounds__(CP_THREADS)
    k_light_compose_grad(const float* __restrict__ dens, const float* __restrict__ tr,
                         const float* __restrict__ color, const float* __restrict__ g, Dims d, float ambient,
                         float scale, float* __restrict__ gd, float* __restrict__ gt) {
    const int64_t nvox = voxels(d), b = blockIdx.y;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = b * nvox + v;
        int64_t o = i;
        if constexpr (L == LAYOUT_BRICK) {
            int x, y, z;
            unflat32((uint32_t)v, d, x, y, z);
            o = b * brick_cells(d) + brick_index(x, y, z, d);
        }
        const float dv = dens[i], t = tr[i];
        const float4 gi = reinterpret_cast<const float4*>(g)[o];
        const float gl[3] = {__fmul_rn(gi.x, scale), __fmul_rn(gi.y, scale), __fmul_rn(gi.z, scale)};
        float sd = 0.f, st = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float col = color[v * 3 + c];
            sd = __fadd_rn(sd, __fmul_rn(gl[c], __fadd_rn(__fmul_rn(t, col), ambient)));
            st = __fadd_rn(st, __fmul_rn(__fmul_rn(gl[c], dv), col));
        }
        gd[i] = __fadd_rn(__fmul_rn(gi.w, scale), sd);
        gt[i] = st;
    }
}

// The adjoint of the factored composition from the raymarch gradient
// projected onto (P, Q) = (scale rgb . g_rgb, scale (ambient sum(g_rgb) + g_a))
// per cell: g_d = Q + t f P, g_t = d f P (the colour's per-voxel factor f
// leaves the sums over samples).
template <int L>
__global__ void __launch_bounds__(CP_THREADS)
    k_light_compose_factored_grad(const float* __restrict__ dens, const float* __restrict__ tr,
                                  const float* __restrict__ fall, const float* __restrict__ g2, Dims d,
                                  float* __restrict__ gd, float* __restrict__ gt) {
    const int64_t nvox = voxels(d), b = blockIdx.y;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = b * nvox + v;
        int64_t o = i;
        if constexpr (L == LAYOUT_BRICK) {
            int x, y, z;
            unflat32((uint32_t)v, d, x, y, z);
            o = b * brick_cells(d) + brick_index(x, y, z, d);
        }
        const float2 pq = reinterpret_cast<const float2*>(g2)[o];
        const float fp = __fmul_rn(fall[v], pq.x);
        gd[i] = __fadd_rn(pq.y, __fmul_rn(tr[i], fp));
        gt[i] = __fmul_rn(dens[i], fp);
    }
}

// From per-camera sums: P, Q = sum over the slice's cameras of the camera's
// value sums divided by its weight sums (where positive), in camera order;
// then as above.  Brick layout.
__global__ void __launch_bounds__(CP_THREADS)
    k_light_compose_factored_grad_cameras(const float* __restrict__ dens, const float* __restrict__ tr,
                                          const float* __restrict__ fall, const float* __restrict__ g2,
                                          const float* __restrict__ wsum, int ncam, Dims d, float* __restrict__ gd,
                                          float* __restrict__ gt) {
    const int64_t nvox = voxels(d), b = blockIdx.y, cells = brick_cells(d);
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = b * nvox + v;
        int x, y, z;
        unflat32((uint32_t)v, d, x, y, z);
        const int64_t o = brick_index(x, y, z, d);
        float P = 0.f, Q = 0.f;
        for (int c = 0; c < ncam; ++c) {
            const int64_t pc = (b * ncam + c) * cells + o;
            const float w = __ldcs(wsum + pc);
            if (w > 0.f) {
                const float2 s = __ldcs(reinterpret_cast<const float2*>(g2) + pc);
                P += s.x / w;
                Q += s.y / w;
            }
        }
        const float fp = __fmul_rn(fall[v], P);
        gd[i] = __fadd_rn(Q, __fmul_rn(tr[i], fp));
        gt[i] = __fmul_rn(dens[i], fp);
    }
}

bool launch_light_compose_factored_grad_cameras(const float* dens, const float* tr, const float* fall,
                                                const float* g2, const float* wsum, int ncam, int N, Dims d,
                                                float* gd, float* gt, cudaStream_t st) {
    const dim3 grid(grid_for(voxels(d), CP_THREADS), N);
    k_light_compose_factored_grad_cameras<<<grid, CP_THREADS, 0, st>>>(dens, tr, fall, g2, wsum, ncam, d, gd, gt);
    return launched(1, "light compose gradient launch");
}

template <typename T, bool FACT>
static void light_compose_t(const float* dens, const float* tr, const float* color, const Rgb& rgb, int N, Dims d,
                            float ambient, float scale, int layout, void* out, cudaStream_t st) {
    const dim3 grid(grid_for(voxels(d), CP_THREADS), N);
    if (layout == LAYOUT_BRICK)
        k_light_compose<LAYOUT_BRICK, T, FACT><<<grid, CP_THREADS, 0, st>>>(dens, tr, color, rgb, d, ambient, scale,
                                                                            (T*)out);
    else
        k_light_compose<LAYOUT_FLAT, T, FACT><<<grid, CP_THREADS, 0, st>>>(dens, tr, color, rgb, d, ambient, scale,
                                                                           (T*)out);
}

bool launch_light_compose(const float* dens, const float* tr, const float* color, const float* rgb3, int N, Dims d,
                          float ambient, float scale, int layout, bool bf16, void* out, cudaStream_t st) {
    Rgb rgb = {{0.f, 0.f, 0.f}};
    if (rgb3 != nullptr) rgb = Rgb{{rgb3[0], rgb3[1], rgb3[2]}};
    if (rgb3 != nullptr) {
        if (bf16)
            light_compose_t<__nv_bfloat16, true>(dens, tr, color, rgb, N, d, ambient, scale, layout, out, st);
        else
            light_compose_t<float, true>(dens, tr, color, rgb, N, d, ambient, scale, layout, out, st);
    } else if (bf16) {
        light_compose_t<__nv_bfloat16, false>(dens, tr, color, rgb, N, d, ambient, scale, layout, out, st);
    } else {
        light_compose_t<float, false>(dens, tr, color, rgb, N, d, ambient, scale, layout, out, st);
    }
    return launched(1, "light compose launch");
}

bool launch_light_compose_factored_grad(const float* dens, const float* tr, const float* fall, const float* g2,
                                        int N, Dims d, int layout, float* gd, float* gt, cudaStream_t st) {
    const dim3 grid(grid_for(voxels(d), CP_THREADS), N);
    if (layout == LAYOUT_BRICK)
        k_light_compose_factored_grad<LAYOUT_BRICK><<<grid, CP_THREADS, 0, st>>>(dens, tr, fall, g2, d, gd, gt);
    else
        k_light_compose_factored_grad<LAYOUT_FLAT><<<grid, CP_THREADS, 0, st>>>(dens, tr, fall, g2, d, gd, gt);
    return launched(1, "light compose gradient launch");
}

bool launch_light_compose_grad(const float* dens, const float* tr, const float* color, const float* g, int N, Dims d,
                               float ambient, float scale, int layout, float* gd, float* gt, cudaStream_t st) {
    const dim3 grid(grid_for(voxels(d), CP_THREADS), N);
    if (layout == LAYOUT_BRICK)
        k_light_compose_grad<LAYOUT_BRICK><<<grid, CP_THREADS, 0, st>>>(dens, tr, color, g, d, ambient, scale, gd, gt);
    else
        k_light_compose_grad<LAYOUT_FLAT><<<grid, CP_THREADS, 0, st>>>(dens, tr, color, g, d, ambient, scale, gd, gt);
    return launched(1, "light compose gradient launch");
}

// --- image loss ------------------------------------------------------------------
// loss = mean((tone(img.rgb + bkg * exp(-img.a)) - target)^2) over pixels and
// rgb.  tone is the renderer's tonemapping (renderer.py:528-541): NONE;
// CLIP_NEGATIVE max(c, 0); SATURATE clip(c, 0, 1); NORMALIZE over the whole
// batch: y = c - min(c) where min(c) < 0 (else c), then y / max(y) where
// max(y) > 0 (else y).  Adjoints follow the frameworks' rules: max(c, 0) and
// clip pass the gradient where 0 <= c (<= 1); the gradient of a full min / max
// reduction is shared evenly by the elements equal to it.
struct Bkg {
    float c[3];
};

// Per-block partial sums (fixed order), then one block sums the partials in
// index order: deterministic.
constexpr int LOSS_BLOCKS_MAX = 1024;

__device__ __forceinline__ float block_sum(float v, float* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();  // sh may still be read by a previous call
    if (l == 0) sh[w] = v;
    __syncthreads();
    float r = 0.f;
    if (threadIdx.x == 0) {
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
    }
    return r;
}

// NaN-propagating min / max (a NaN pixel makes the normalisation NaN, as the
// tensor reductions do)
__device__ __forceinline__ float nan_min(float a, float b) { return (b < a || b != b) ? b : a; }
__device__ __forceinline__ float nan_max(float a, float b) { return (b > a || b != b) ? b : a; }

template <bool MAX>
__device__ __forceinline__ float block_ext(float v, float* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float x = __shfl_xor_sync(0xffffffffu, v, o);
        v = MAX ? nan_max(v, x) : nan_min(v, x);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    float r = sh[0];
    if (threadIdx.x == 0) {
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) r = MAX ? nan_max(r, sh[i]) : nan_min(r, sh[i]);
    }
    return r;
}

// Composite of pixel i, channel c, and exp(-alpha)
__device__ __forceinline__ float composite(float px, float bkg, float e) { return __fadd_rn(px, __fmul_rn(bkg, e)); }

// Statistics of NORMALIZE in the workspace: st[0] = min(c), st[1] = max(y)
// (max(c) - min(c) where min(c) < 0), st[2] and st[3] the adjoint's shares of
// the max and min reductions.
__device__ __forceinline__ float tone(int tm, float c, const float* st) {
    switch (tm) {
        case GFT_TONEMAP_CLIP_NEGATIVE: return c < 0.f ? 0.f : c;
        case GFT_TONEMAP_SATURATE: return c < 0.f ? 0.f : (c > 1.f ? 1.f : c);
        case GFT_TONEMAP_NORMALIZE: {
            const float mn = st[0], mx = st[1];
            const float y = mn < 0.f ? __fadd_rn(c, -mn) : c;
            return mx > 0.f ? __fdiv_rn(y, mx) : y;
        }
        default: return c;
    }
}

__global__ void __launch_bounds__(CP_THREADS)
    k_tone_stats_partial(const float* __restrict__ img, int64_t npix, Bkg bkg, float* __restrict__ part) {
    __shared__ float sh[CP_THREADS / 32];
    float mn = INFINITY, mx = -INFINITY;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = reinterpret_cast<const float4*>(img)[i];
        const float e = expf(-a.w);
        const float px[3] = {a.x, a.y, a.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float v = composite(px[c], bkg.c[c], e);
            mn = nan_min(mn, v);
            mx = nan_max(mx, v);
        }
    }
    const float rmn = block_ext<false>(mn, sh);
    const float rmx = block_ext<true>(mx, sh);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = rmn;
        part[2 * blockIdx.x + 1] = rmx;
    }
}

__global__ void __launch_bounds__(CP_THREADS)
    k_tone_stats_final(const float* __restrict__ part, int nparts, float* __restrict__ st) {
    __shared__ float sh[CP_THREADS / 32];
    float mn = INFINITY, mx = -INFINITY;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        mn = nan_min(mn, part[2 * i]);
        mx = nan_max(mx, part[2 * i + 1]);
    }
    const float rmn = block_ext<false>(mn, sh);
    const float rmx = block_ext<true>(mx, sh);
    if (threadIdx.x == 0) {
        st[0] = rmn;
        // max over y = c - min is max(c) - min: rounding is monotonic
        st[1] = rmn < 0.f ? __fadd_rn(rmx, -rmn) : rmx;
    }
}

__global__ void __launch_bounds__(CP_THREADS)
    k_image_loss_partial(const float* __restrict__ img, const float* __restrict__ tgt, int64_t npix, Bkg bkg, int tm,
                         const float* __restrict__ st, float* __restrict__ partial) {
    __shared__ float sh[CP_THREADS / 32];
    float acc = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = reinterpret_cast<const float4*>(img)[i];
        const float e = expf(-a.w);
        const float px[3] = {a.x, a.y, a.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float diff = __fadd_rn(tone(tm, composite(px[c], bkg.c[c], e), st), -tgt[i * 3 + c]);
            acc = fmaf(diff, diff, acc);
        }
    }
    const float r = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = r;
}

__global__ void __launch_bounds__(CP_THREADS)
    k_image_loss_final(const float* __restrict__ partial, int nparts, float inv_n, float* __restrict__ loss) {
    __shared__ float sh[CP_THREADS / 32];
    float acc = 0.f;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += partial[i];
    const float r = block_sum(acc, sh);
    if (threadIdx.x == 0) *loss = r * inv_n;
}

// NORMALIZE adjoint, first pass: with G = d loss / d z = 2 (z - t) / n,
// per block: sum G z, sum G, #(y == max y), #(c == min c).
__global__ void __launch_bounds__(CP_THREADS)
    k_tone_grad_partial(const float* __restrict__ img, const float* __restrict__ tgt, int64_t npix, Bkg bkg,
                        float two_inv_n, const float* __restrict__ gloss, const float* __restrict__ st,
                        float* __restrict__ part, unsigned int* __restrict__ cnt) {
    __shared__ float sh[CP_THREADS / 32];
    const float gs = __fmul_rn(*gloss, two_inv_n);
    const float mn = st[0], mx = st[1];
    float sgz = 0.f, sg = 0.f;
    unsigned int nmax = 0, nmin = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = reinterpret_cast<const float4*>(img)[i];
        const float e = expf(-a.w);
        const float px[3] = {a.x, a.y, a.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float v = composite(px[c], bkg.c[c], e);
            const float y = mn < 0.f ? __fadd_rn(v, -mn) : v;
            const float z = mx > 0.f ? __fdiv_rn(y, mx) : y;
            const float g = __fmul_rn(gs, __fadd_rn(z, -tgt[i * 3 + c]));
            sgz = fmaf(g, z, sgz);
            sg += g;
            nmax += (y == mx) ? 1u : 0u;
            nmin += (v == mn) ? 1u : 0u;
        }
    }
    const float r0 = block_sum(sgz, sh);
    const float r1 = block_sum(sg, sh);
    // counts: exact integer sums, one warp reduction each
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        nmax += __shfl_xor_sync(0xffffffffu, nmax, o);
        nmin += __shfl_xor_sync(0xffffffffu, nmin, o);
    }
    __shared__ unsigned int shc[2][CP_THREADS / 32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        shc[0][w] = nmax;
        shc[1][w] = nmin;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int a = 0, b = 0;
        for (int k = 0; k < CP_THREADS / 32; ++k) a += shc[0][k], b += shc[1][k];
        part[2 * blockIdx.x] = r0;
        part[2 * blockIdx.x + 1] = r1;
        cnt[2 * blockIdx.x] = a;
        cnt[2 * blockIdx.x + 1] = b;
    }
}

// st[2] = (d loss / d max y) / #max, st[3] = (d loss / d min c) / #min (0 when
// that normalisation step is not taken): d loss / d max = -sum G z / max, and
// d loss / d min = -sum_i d loss / d y_i.
__global__ void __launch_bounds__(CP_THREADS)
    k_tone_grad_final(const float* __restrict__ part, const unsigned int* __restrict__ cnt, int nparts,
                      float* __restrict__ st) {
    __shared__ float sh[CP_THREADS / 32];
    float a = 0.f, b = 0.f;
    unsigned long long na = 0, nb = 0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
        a += part[2 * i];
        b += part[2 * i + 1];
    }
    const float sgz = block_sum(a, sh);
    const float sg = block_sum(b, sh);
    if (threadIdx.x == 0) {
        for (int i = 0; i < nparts; ++i) na += cnt[2 * i], nb += cnt[2 * i + 1];
        const float mn = st[0], mx = st[1];
        float gmax = 0.f, gy_sum = sg;
        if (mx > 0.f) {
            const float dmx = -sgz / mx;
            gmax = na > 0 ? dmx / (float)na : 0.f;
            gy_sum = sg / mx + dmx;
        }
        st[2] = gmax;
        st[3] = (mn < 0.f && nb > 0) ? -gy_sum / (float)nb : 0.f;
    }
}

// d loss / d rgb_c = tone'(c) 2 (tone(c) - t_c) / n; d c / d a = -bkg_c exp(-a).
__global__ void __launch_bounds__(CP_THREADS)
    k_image_loss_grad(const float* __restrict__ img, const float* __restrict__ tgt, int64_t npix, Bkg bkg, int tm,
                      const float* __restrict__ st, float two_inv_n, const float* __restrict__ gloss,
                      float* __restrict__ gimg) {
    const float gs = __fmul_rn(*gloss, two_inv_n);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = reinterpret_cast<const float4*>(img)[i];
        const float e = expf(-a.w);
        const float px[3] = {a.x, a.y, a.z};
        float g[3], ga = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float v = composite(px[c], bkg.c[c], e);
            const float diff = __fadd_rn(tone(tm, v, st), -tgt[i * 3 + c]);
            float gc = __fmul_rn(gs, diff);
            if (tm == GFT_TONEMAP_CLIP_NEGATIVE) {
                gc = v >= 0.f ? gc : 0.f;
            } else if (tm == GFT_TONEMAP_SATURATE) {
                gc = (v >= 0.f && v <= 1.f) ? gc : 0.f;
            } else if (tm == GFT_TONEMAP_NORMALIZE) {
                const float mn = st[0], mx = st[1];
                const float y = mn < 0.f ? __fadd_rn(v, -mn) : v;
                if (mx > 0.f) gc = __fadd_rn(__fdiv_rn(gc, mx), y == mx ? st[2] : 0.f);
                if (mn < 0.f && v == mn) gc = __fadd_rn(gc, st[3]);
            }
            g[c] = gc;
            ga = __fadd_rn(ga, __fmul_rn(gc, bkg.c[c]));
        }
        reinterpret_cast<float4*>(gimg)[i] = make_float4(g[0], g[1], g[2], -__fmul_rn(ga, e));
    }
}

int image_loss_blocks(int64_t npix) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((npix + CP_THREADS - 1) / CP_THREADS, LOSS_BLOCKS_MAX));
}

// ws floats: [0, 4) statistics, [4, 4 + nb) loss partials, then 2 nb floats of
// the statistics / adjoint partials and 2 nb uint counts
size_t image_loss_ws_floats(int64_t npix) { return 4 + (size_t)image_loss_blocks(npix) * 5; }

bool launch_image_loss(const float* img, const float* tgt, int64_t npix, const float bkg[3], int tonemap, float* ws,
                       float* loss, cudaStream_t st) {
    const int nb = image_loss_blocks(npix);
    const Bkg b{{bkg[0], bkg[1], bkg[2]}};
    float* stats = ws;
    float* partial = ws + 4;
    float* part2 = partial + nb;
    int n = 2;
    if (tonemap == GFT_TONEMAP_NORMALIZE) {
        k_tone_stats_partial<<<nb, CP_THREADS, 0, st>>>(img, npix, b, part2);
        k_tone_stats_final<<<1, CP_THREADS, 0, st>>>(part2, nb, stats);
        n += 2;
    }
    k_image_loss_partial<<<nb, CP_THREADS, 0, st>>>(img, tgt, npix, b, tonemap, stats, partial);
    k_image_loss_final<<<1, CP_THREADS, 0, st>>>(partial, nb, 1.f / (float)(npix * 3), loss);
    return launched(n, "image loss launch");
}

bool launch_image_loss_grad(const float* img, const float* tgt, int64_t npix, const float bkg[3], int tonemap,
                            float* ws, const float* gloss, float* gimg, cudaStream_t st) {
    const Bkg b{{bkg[0], bkg[1], bkg[2]}};
    const float two_inv_n = 2.f / (float)(npix * 3);
    int n = 1;
    if (tonemap == GFT_TONEMAP_NORMALIZE) {
        const int nb = image_loss_blocks(npix);
        float* stats = ws;
        float* part2 = ws + 4 + nb;
        unsigned int* cnt = reinterpret_cast<unsigned int*>(part2 + 2 * nb);
        k_tone_stats_partial<<<nb, CP_THREADS, 0, st>>>(img, npix, b, part2);
        k_tone_stats_final<<<1, CP_THREADS, 0, st>>>(part2, nb, stats);
        k_tone_grad_partial<<<nb, CP_THREADS, 0, st>>>(img, tgt, npix, b, two_inv_n, gloss, stats, part2, cnt);
        k_tone_grad_final<<<1, CP_THREADS, 0, st>>>(part2, cnt, nb, stats);
        n += 4;
    }
    k_image_loss_grad<<<grid_for(npix, CP_THREADS), CP_THREADS, 0, st>>>(img, tgt, npix, b, tonemap,
                                                                          tonemap == GFT_TONEMAP_NORMALIZE ? ws : nullptr,
                                                                          two_inv_n, gloss, gimg);
    return launched(n, "image loss gradient launch");
}

}  // namespace gft
