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
//   image loss       mean((img.rgb + bkg * exp(-img.a) - target)^2) with its
//                    background composite (renderer.py:1048-1052).
//
// Elementwise products and sums use __fmul_rn / __fadd_rn so that they round
// exactly like the separate tensor ops they replace (no FMA contraction).
#include <algorithm>

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
template <int L>
__global__ void __launch_bounds__(CP_THREADS)
    k_light_compose(const float* __restrict__ dens, const float* __restrict__ tr, const float* __restrict__ color,
                    Dims d, float ambient, float scale, float* __restrict__ out) {
    const int64_t nvox = voxels(d), b = blockIdx.y;
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = b * nvox + v;
        const float dv = dens[i], t = tr[i];
        float r[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float lc = __fmul_rn(dv, __fadd_rn(__fmul_rn(t, color[v * 3 + c]), ambient));
            r[c] = __fmul_rn(lc, scale);
        }
        int64_t o = i;
        if constexpr (L == LAYOUT_BRICK) {
            int x, y, z;
            unflat32((uint32_t)v, d, x, y, z);
            o = b * brick_cells(d) + brick_index(x, y, z, d);
        }
        reinterpret_cast<float4*>(out)[o] = make_float4(r[0], r[1], r[2], __fmul_rn(dv, scale));
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

bool launch_light_compose(const float* dens, const float* tr, const float* color, int N, Dims d, float ambient,
                          float scale, int layout, float* out, cudaStream_t st) {
    const dim3 grid(grid_for(voxels(d), CP_THREADS), N);
    if (layout == LAYOUT_BRICK)
        k_light_compose<LAYOUT_BRICK><<<grid, CP_THREADS, 0, st>>>(dens, tr, color, d, ambient, scale, out);
    else
        k_light_compose<LAYOUT_FLAT><<<grid, CP_THREADS, 0, st>>>(dens, tr, color, d, ambient, scale, out);
    return launched(1, "light compose launch");
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
struct Bkg {
    float c[3];
};

// Per-block partial sums of the squared differences (fixed order), then one
// block sums the partials in index order: deterministic.
constexpr int LOSS_BLOCKS_MAX = 1024;

__device__ __forceinline__ float block_sum(float v, float* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    float r = 0.f;
    if (threadIdx.x == 0) {
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
    }
    return r;
}

__global__ void __launch_bounds__(CP_THREADS)
    k_image_loss_partial(const float* __restrict__ img, const float* __restrict__ tgt, int64_t npix, Bkg bkg,
                         float* __restrict__ partial) {
    __shared__ float sh[CP_THREADS / 32];
    float acc = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = reinterpret_cast<const float4*>(img)[i];
        const float e = expf(-a.w);
        const float px[3] = {a.x, a.y, a.z};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float diff = __fadd_rn(__fadd_rn(px[c], __fmul_rn(bkg.c[c], e)), -tgt[i * 3 + c]);
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

// d loss / d rgb_c = 2 (rgb_c - t_c) / n; d rgb_c / d a = -bkg_c exp(-a).
__global__ void __launch_bounds__(CP_THREADS)
    k_image_loss_grad(const float* __restrict__ img, const float* __restrict__ tgt, int64_t npix, Bkg bkg,
                      float two_inv_n, const float* __restrict__ gloss, float* __restrict__ gimg) {
    const float gs = __fmul_rn(*gloss, two_inv_n);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = reinterpret_cast<const float4*>(img)[i];
        const float e = expf(-a.w);
        const float px[3] = {a.x, a.y, a.z};
        float g[3], ga = 0.f;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float diff = __fadd_rn(__fadd_rn(px[c], __fmul_rn(bkg.c[c], e)), -tgt[i * 3 + c]);
            g[c] = __fmul_rn(gs, diff);
            ga = __fadd_rn(ga, __fmul_rn(g[c], bkg.c[c]));
        }
        reinterpret_cast<float4*>(gimg)[i] = make_float4(g[0], g[1], g[2], -__fmul_rn(ga, e));
    }
}

int image_loss_blocks(int64_t npix) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((npix + CP_THREADS - 1) / CP_THREADS, LOSS_BLOCKS_MAX));
}

bool launch_image_loss(const float* img, const float* tgt, int64_t npix, const float bkg[3], float* partial,
                       float* loss, cudaStream_t st) {
    const int nb = image_loss_blocks(npix);
    const Bkg b{{bkg[0], bkg[1], bkg[2]}};
    k_image_loss_partial<<<nb, CP_THREADS, 0, st>>>(img, tgt, npix, b, partial);
    k_image_loss_final<<<1, CP_THREADS, 0, st>>>(partial, nb, 1.f / (float)(npix * 3), loss);
    return launched(2, "image loss launch");
}

bool launch_image_loss_grad(const float* img, const float* tgt, int64_t npix, const float bkg[3], const float* gloss,
                            float* gimg, cudaStream_t st) {
    const Bkg b{{bkg[0], bkg[1], bkg[2]}};
    k_image_loss_grad<<<grid_for(npix, CP_THREADS), CP_THREADS, 0, st>>>(img, tgt, npix, b,
                                                                          2.f / (float)(npix * 3), gloss, gimg);
    return launched(1, "image loss gradient launch");
}

}  // namespace gft
