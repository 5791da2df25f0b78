// Depth reduce-blend (ReduceGridBlend) and its adjoint.
//
// Semantics: kBlend / kBlendGrad (reduce_blend.cu.cc:34-75).  One thread per
// (batch, y, x) column walks the depth axis; consecutive threads own
// consecutive x so every depth step is a coalesced row access.  The loop is
// unrolled so several depth loads are in flight per thread.
#include "gft_internal.h"

namespace gft {

constexpr int BL_THREADS = 256;

template <int C, bool KEEP>
__global__ void __launch_bounds__(BL_THREADS)
    k_blend_fwd(const float* __restrict__ in, int N, Dims d, int mode, float* __restrict__ out) {
    const int64_t plane = (int64_t)d.x * d.y;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= plane * N) return;
    const int b = (int)(t / plane);
    const int64_t col = t - (int64_t)b * plane;
    const float* src = in + (size_t)b * plane * d.z * C;
    Vec<C> acc = vzero<C>();
#pragma unroll 4
    for (int z = 0; z < d.z; ++z) {
        const Vec<C> v = loadf<C>(src, (int64_t)z * plane + col);
        acc = blend<C>(mode, acc, v);
        if constexpr (KEEP) store<C>(out, ((int64_t)b * d.z + z) * plane + col, acc);
    }
    if constexpr (!KEEP) store<C>(out, (int64_t)b * plane + col, acc);
}

template <int C, bool KEEP>
__global__ void __launch_bounds__(BL_THREADS)
    k_blend_bwd(const float* __restrict__ dy, const float* __restrict__ y, const float* __restrict__ x, int N, Dims d,
                int mode, bool exact, float* __restrict__ gx) {
    const int64_t plane = (int64_t)d.x * d.y;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= plane * N) return;
    const int b = (int)(t / plane);
    const int64_t col = t - (int64_t)b * plane;
    const size_t vol = (size_t)b * plane * d.z;
    Vec<C> g = vzero<C>(), prev = vzero<C>();
    if constexpr (!KEEP) {
        g = loadf<C>(dy, (int64_t)b * plane + col);
        prev = loadf<C>(y, (int64_t)b * plane + col);
    }
    for (int z = d.z - 1; z >= 0; --z) {
        const int64_t i = (int64_t)vol + (int64_t)z * plane + col;
        if constexpr (KEEP) {
            g = vadd(g, loadf<C>(dy, i));
            prev = loadf<C>(y, i);
        }
        const Vec<C> s = loadf<C>(x, i);
        const Vec<C> gc = blend_grad<C>(mode, exact, g, s, prev);
        store<C>(gx, i, gc);
    }
}

template <int C>
static void fwd_launch(bool keep, unsigned blocks, cudaStream_t s, const float* in, int N, Dims d, int mode, float* out) {
    if (keep) k_blend_fwd<C, true><<<blocks, BL_THREADS, 0, s>>>(in, N, d, mode, out);
    else k_blend_fwd<C, false><<<blocks, BL_THREADS, 0, s>>>(in, N, d, mode, out);
}

bool launch_blend_fwd(const float* in, int N, int C, Dims d, int mode, bool keep_dims, float* out, cudaStream_t s) {
    const int64_t cols = (int64_t)d.x * d.y * N;
    const unsigned blocks = (unsigned)((cols + BL_THREADS - 1) / BL_THREADS);
    if (C == 4) fwd_launch<4>(keep_dims, blocks, s, in, N, d, mode, out);
    else if (C == 2) fwd_launch<2>(keep_dims, blocks, s, in, N, d, mode, out);
    else fwd_launch<1>(keep_dims, blocks, s, in, N, d, mode, out);
    return launched(1, "reduce blend launch");
}

template <int C>
static void bwd_launch(bool keep, unsigned blocks, cudaStream_t s, const float* dy, const float* y, const float* x,
                       int N, Dims d, int mode, bool exact, float* gx) {
    if (keep) k_blend_bwd<C, true><<<blocks, BL_THREADS, 0, s>>>(dy, y, x, N, d, mode, exact, gx);
    else k_blend_bwd<C, false><<<blocks, BL_THREADS, 0, s>>>(dy, y, x, N, d, mode, exact, gx);
}

bool launch_blend_bwd(const float* dy, const float* y, const float* x, int N, int C, Dims d, int mode,
                      bool keep_dims, bool exact, float* gx, cudaStream_t s) {
    const int64_t cols = (int64_t)d.x * d.y * N;
    const unsigned blocks = (unsigned)((cols + BL_THREADS - 1) / BL_THREADS);
    if (C == 4) bwd_launch<4>(keep_dims, blocks, s, dy, y, x, N, d, mode, exact, gx);
    else if (C == 2) bwd_launch<2>(keep_dims, blocks, s, dy, y, x, N, d, mode, exact, gx);
    else bwd_launch<1>(keep_dims, blocks, s, dy, y, x, N, d, mode, exact, gx);
    return launched(1, "reduce blend gradient launch");
}

}  // namespace gft
