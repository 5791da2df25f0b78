// Fused raymarch (RaymarchGridTransform) forward and adjoint.
//
// Forward semantics: kRaymarchGridTransformLindepth (raymarch_grid.cu.cc:107-143).
// One thread per pixel; the rays of all (batch, camera) pairs of a call run in
// one launch (grid.z = pair), where the reference launches once per camera
// with a host constant-buffer upload in between.  A warp covers an 8x4 pixel
// tile so that the 32 rays of a warp gather from neighbouring voxels.
#include "gft_internal.h"

namespace gft {

constexpr int RM_BX = 8, RM_BY = 16;  // 128 threads, warp = 8x4 pixels

template <int C, typename S, int BM, bool LIN>
__global__ void __launch_bounds__(RM_BX* RM_BY)
    k_raymarch_fwd(const S* __restrict__ in, Dims din, int W, int H, int D, int filter, int blend_mode,
                   float* __restrict__ out, const __grid_constant__ PairTable tab) {
    const int p = blockIdx.z;
    const int x = blockIdx.x * RM_BX + threadIdx.x;
    const int y = blockIdx.y * RM_BY + threadIdx.y;
    if (x >= W || y >= H) return;
    const CamX& cam = tab.cam[p];
    const S* g = in + (size_t)tab.in_batch[p] * voxels(din) * C;
    const float3 dinv = make_float3(1.f / (float)W, 1.f / (float)H, 1.f / (float)D);
    const float zmax = (float)max(D - 1, 1);
    const float3 nearp = idx_to_os(cam, make_float3(x + 0.5f, y + 0.5f, 0.5f), dinv);
    const float3 farp = idx_to_os(cam, make_float3(x + 0.5f, y + 0.5f, zmax + 0.5f), dinv);
    const float3 step = make_float3((farp.x - nearp.x) / zmax, (farp.y - nearp.y) / zmax, (farp.z - nearp.z) / zmax);
    float3 pos = nearp;
    Vec<C> acc = vzero<C>();
    for (int i = 0; i < D; ++i) {
        Vec<C> smp;
        if constexpr (LIN) {
            smp = fetch_linear<C, S, BM>(g, din, pos.x - 0.5f, pos.y - 0.5f, pos.z - 0.5f);
        } else {
            smp = fetch<C, S, BM, true>(filter, g, din, pos.x - 0.5f, pos.y - 0.5f, pos.z - 0.5f);
        }
        acc = blend<C>(blend_mode, acc, smp);
        pos.x += step.x;
        pos.y += step.y;
        pos.z += step.z;
    }
    store<C>(out, ((int64_t)tab.out_slot[p] * H + y) * W + x, acc);
}

// Adjoint: back to front from the far end point, re-sampling (LINEAR only as the
// reference gradient op) and scattering each cell gradient trilinearly.
// EXACT: scatter straight into the batch gradient.  Otherwise scatter into the
// pair's buffer together with the trilinear weights, normalised afterwards.
template <int C, typename S, int BM, bool EXACT>
__global__ void __launch_bounds__(RM_BX* RM_BY)
    k_raymarch_bwd(const S* __restrict__ in, Dims din, int W, int H, int D, int blend_mode,
                   const float* __restrict__ out, const float* __restrict__ dout, float* __restrict__ grad,
                   float* __restrict__ buf, float* __restrict__ cnt, const __grid_constant__ PairTable tab) {
    const int p = blockIdx.z;
    const int x = blockIdx.x * RM_BX + threadIdx.x;
    const int y = blockIdx.y * RM_BY + threadIdx.y;
    if (x >= W || y >= H) return;
    const CamX& cam = tab.cam[p];
    const int64_t nvox = voxels(din);
    const S* g = in + (size_t)tab.in_batch[p] * nvox * C;
    float* dst;
    float* count = nullptr;
    if constexpr (EXACT) {
        dst = grad + (size_t)tab.in_batch[p] * nvox * C;
    } else {
        dst = buf + (size_t)(tab.pair_base + p) * nvox * C;
        count = cnt + (size_t)(tab.pair_base + p) * nvox;
    }
    const float3 dinv = make_float3(1.f / (float)W, 1.f / (float)H, 1.f / (float)D);
    const float zmax = (float)max(D - 1, 1);
    const float3 nearp = idx_to_os(cam, make_float3(x + 0.5f, y + 0.5f, 0.5f), dinv);
    const float3 farp = idx_to_os(cam, make_float3(x + 0.5f, y + 0.5f, zmax + 0.5f), dinv);
    const float3 step = make_float3((farp.x - nearp.x) / zmax, (farp.y - nearp.y) / zmax, (farp.z - nearp.z) / zmax);
    float3 pos = farp;
    const int64_t pix = ((int64_t)tab.out_slot[p] * H + y) * W + x;
    Vec<C> acc = loadf<C>(out, pix);
    Vec<C> go = loadf<C>(dout, pix);
    for (int i = D - 1; i >= 0; --i) {
        const Vec<C> smp = fetch_linear<C, S, BM>(g, din, pos.x - 0.5f, pos.y - 0.5f, pos.z - 0.5f);
        const Vec<C> gc = blend_grad<C>(blend_mode, EXACT, go, smp, acc);
        if constexpr (EXACT) {
            scatter_linear<C, BM, 0>(dst, nullptr, din, pos.x - 0.5f, pos.y - 0.5f, pos.z - 0.5f, gc);
        } else {
            scatter_linear<C, BM, 2>(dst, count, din, pos.x - 0.5f, pos.y - 0.5f, pos.z - 0.5f, gc);
        }
        pos.x -= step.x;
        pos.y -= step.y;
        pos.z -= step.z;
    }
}

// grad[b] = sum over the pairs of batch b of buf / cnt where cnt > 0
// (kNormalize3DGradients<T,true,AddGrad>, raymarch_grid.cu.cc:319-341).
template <int C>
__global__ void k_raymarch_normalize(const float* __restrict__ buf, const float* __restrict__ cnt, int64_t nvox,
                                     const int* __restrict__ pair_batch_dummy, int npairs_per_batch, int N,
                                     float* __restrict__ grad) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nvox * N) return;
    const int b = (int)(t / nvox);
    const int64_t v = t - (int64_t)b * nvox;
    Vec<C> acc = vzero<C>();
    for (int k = 0; k < npairs_per_batch; ++k) {
        const int64_t pidx = (int64_t)b * npairs_per_batch + k;
        const float n = cnt[pidx * nvox + v];
        if (n > 0.f) {
            const float w = 1.0f / n;
            const Vec<C> gb = loadf<C>(buf, pidx * nvox + v);
            acc = vadd(acc, vscale(gb, w));
        }
    }
    store<C>(grad, t, acc);
}

template <int C, typename S, int BM>
static void fwd_dispatch_lin(bool lin, dim3 grid, dim3 block, cudaStream_t s, const void* in, const RaymarchArgs& a,
                             float* out, const PairTable& t) {
    if (lin)
        k_raymarch_fwd<C, S, BM, true><<<grid, block, 0, s>>>((const S*)in, a.din, a.W, a.H, a.D, a.filter, a.blend,
                                                               out, t);
    else
        k_raymarch_fwd<C, S, BM, false><<<grid, block, 0, s>>>((const S*)in, a.din, a.W, a.H, a.D, a.filter, a.blend,
                                                                out, t);
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
    for (const PairTable& t : make_tables(pairs)) {
        const dim3 grid((a.W + RM_BX - 1) / RM_BX, (a.H + RM_BY - 1) / RM_BY, t.n);
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

template <int C, typename S, int BM>
static void bwd_dispatch_exact(bool exact, dim3 grid, dim3 block, cudaStream_t s, const RaymarchArgs& a,
                               const float* out, const float* dout, float* grad, float* buf, float* cnt,
                               const PairTable& t) {
    if (exact)
        k_raymarch_bwd<C, S, BM, true><<<grid, block, 0, s>>>((const S*)a.input, a.din, a.W, a.H, a.D, a.blend, out,
                                                               dout, grad, buf, cnt, t);
    else
        k_raymarch_bwd<C, S, BM, false><<<grid, block, 0, s>>>((const S*)a.input, a.din, a.W, a.H, a.D, a.blend, out,
                                                                dout, grad, buf, cnt, t);
}

template <int C, typename S>
static void bwd_dispatch_bm(bool exact, dim3 grid, dim3 block, cudaStream_t s, const RaymarchArgs& a,
                            const float* out, const float* dout, float* grad, float* buf, float* cnt,
                            const PairTable& t) {
    switch (a.boundary) {
        case BM_BORDER: bwd_dispatch_exact<C, S, BM_BORDER>(exact, grid, block, s, a, out, dout, grad, buf, cnt, t); break;
        case BM_CLAMP: bwd_dispatch_exact<C, S, BM_CLAMP>(exact, grid, block, s, a, out, dout, grad, buf, cnt, t); break;
        default: bwd_dispatch_exact<C, S, BM_WRAP>(exact, grid, block, s, a, out, dout, grad, buf, cnt, t); break;
    }
}

bool launch_raymarch_bwd(const RaymarchArgs& a, const std::vector<Pair>& pairs, const float* out,
                         const float* dout, bool exact, float* grad, float* ws_buf, float* ws_cnt,
                         cudaStream_t s) {
    const int64_t nvox = voxels(a.din);
    if (exact) {
        if (!cuda_ok(cudaMemsetAsync(grad, 0, sizeof(float) * nvox * a.C * a.N, s), "zero gradient")) return false;
    } else {
        const size_t np = pairs.size();
        if (!cuda_ok(cudaMemsetAsync(ws_buf, 0, sizeof(float) * nvox * a.C * np, s), "zero buffer")) return false;
        if (!cuda_ok(cudaMemsetAsync(ws_cnt, 0, sizeof(float) * nvox * np, s), "zero counter")) return false;
    }
    const dim3 block(RM_BX, RM_BY, 1);
    for (const PairTable& t : make_tables(pairs)) {
        const dim3 grid((a.W + RM_BX - 1) / RM_BX, (a.H + RM_BY - 1) / RM_BY, t.n);
        if (a.dtype == 0) {
            if (a.C == 4) bwd_dispatch_bm<4, float>(exact, grid, block, s, a, out, dout, grad, ws_buf, ws_cnt, t);
            else if (a.C == 2) bwd_dispatch_bm<2, float>(exact, grid, block, s, a, out, dout, grad, ws_buf, ws_cnt, t);
            else bwd_dispatch_bm<1, float>(exact, grid, block, s, a, out, dout, grad, ws_buf, ws_cnt, t);
        } else {
            if (a.C == 4) bwd_dispatch_bm<4, __nv_bfloat16>(exact, grid, block, s, a, out, dout, grad, ws_buf, ws_cnt, t);
            else if (a.C == 2) bwd_dispatch_bm<2, __nv_bfloat16>(exact, grid, block, s, a, out, dout, grad, ws_buf, ws_cnt, t);
            else bwd_dispatch_bm<1, __nv_bfloat16>(exact, grid, block, s, a, out, dout, grad, ws_buf, ws_cnt, t);
        }
        if (!launched(1, "raymarch backward launch")) return false;
    }
    if (!exact) {
        // pairs are ordered batch-major with the same count per batch
        const int per_batch = (int)(pairs.size() / a.N);
        const int64_t total = nvox * a.N;
        const int threads = 256;
        const unsigned blocks = (unsigned)((total + threads - 1) / threads);
        if (a.C == 4) k_raymarch_normalize<4><<<blocks, threads, 0, s>>>(ws_buf, ws_cnt, nvox, nullptr, per_batch, a.N, grad);
        else if (a.C == 2) k_raymarch_normalize<2><<<blocks, threads, 0, s>>>(ws_buf, ws_cnt, nvox, nullptr, per_batch, a.N, grad);
        else k_raymarch_normalize<1><<<blocks, threads, 0, s>>>(ws_buf, ws_cnt, nvox, nullptr, per_batch, a.N, grad);
        if (!launched(1, "raymarch normalize launch")) return false;
    }
    return true;
}

}  // namespace gft
