// FP64 check step: double-precision recomputations on the GPU of two FP32
// results of the step whose errors compound along a ray -- the shadow
// transmittance (exp of a depth sum over up to 256 light-frustum cells) and
// the accumulated density of the raymarch (a sum over up to 256 samples) --
// on a strided sample of columns / rays, reporting the largest absolute and
// relative deviation of the FP32 result.  The recomputation uses the FP32
// inputs the step used (the sampled light-frustum densities; the raymarch
// input grid), so the reported error is that of the FP32 scan / march alone:
// positions, trilinear weights, sums and exponentials in double.
//
// Results: two doubles (max |fp32 - fp64|, max |fp64|), whose ratio is the
// max-norm relative error, reduced with atomicMax on their bit patterns
// (non-negative doubles order like their bits); the launchers zero them first.
#include "gft_internal.h"

namespace gft {

constexpr int CK_THREADS = 256;

__device__ __forceinline__ void warp_max_to(double* result, double abs_err, double ref_max) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        abs_err = fmax(abs_err, __shfl_down_sync(0xffffffffu, abs_err, o));
        ref_max = fmax(ref_max, __shfl_down_sync(0xffffffffu, ref_max, o));
    }
    if ((threadIdx.x & 31u) == 0) {
        atomicMax(reinterpret_cast<unsigned long long*>(result), (unsigned long long)__double_as_longlong(abs_err));
        atomicMax(reinterpret_cast<unsigned long long*>(result) + 1,
                  (unsigned long long)__double_as_longlong(ref_max));
    }
}

__device__ __forceinline__ void deviation(double got, double ref, double& abs_err, double& ref_max) {
    abs_err = fmax(abs_err, fabs(got - ref));
    ref_max = fmax(ref_max, fabs(ref));
}

// tr[z] = exp(-sum_{z' < z} x[z']) per column of a [N, D, H, W, 1] grid.
__global__ void __launch_bounds__(CK_THREADS)
    k_transmittance_check(const float* __restrict__ x, const float* __restrict__ tr, int N, Dims d, int stride,
                          double* result) {
    const int64_t plane = (int64_t)d.x * d.y;
    const int64_t col = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * stride;
    double abs_err = 0.0, ref_max = 0.0;
    if (col < plane * N) {
        const int64_t b = col / plane;
        const int64_t base = b * plane * d.z + (col - b * plane);
        double e = 0.0;
        for (int z = 0; z < d.z; ++z) {
            const int64_t i = base + (int64_t)z * plane;
            deviation((double)tr[i], exp(-e), abs_err, ref_max);
            e += (double)x[i];
        }
    }
    warp_max_to(result, abs_err, ref_max);
}

bool launch_transmittance_check(const float* x, const float* tr, int N, Dims d, int stride, double* result,
                                cudaStream_t s) {
    if (!cuda_ok(cudaMemsetAsync(result, 0, 2 * sizeof(double), s), "zero check result")) return false;
    const int64_t cols = ((int64_t)d.x * d.y * N + stride - 1) / stride;
    k_transmittance_check<<<(unsigned)((cols + CK_THREADS - 1) / CK_THREADS), CK_THREADS, 0, s>>>(x, tr, N, d, stride,
                                                                                                  result);
    return launched(1, "transmittance check launch");
}

// --- raymarch: density channel of a BEER_LAMBERT / LINEAR / BORDER march -------
__device__ __forceinline__ void mul4d(const double* m, const double v[4], double o[4]) {
#pragma unroll
    for (int r = 0; r < 4; ++r) o[r] = m[4 * r] * v[0] + m[4 * r + 1] * v[1] + m[4 * r + 2] * v[2] + m[4 * r + 3] * v[3];
}

// IDXtoOS in double: NDC = idx / dims * 2 - 1, VS = P^-1 NDC / w, OS = MV^-1 VS
__device__ __forceinline__ void idx_to_os_d(const CamD& c, double ix, double iy, double iz, double W, double H,
                                            double D, double os[3]) {
    const double ndc[4] = {ix / W * 2.0 - 1.0, iy / H * 2.0 - 1.0, iz / D * 2.0 - 1.0, 1.0};
    double vs[4], o[4];
    mul4d(c.pi, ndc, vs);
    const double iw = 1.0 / vs[3];
    for (int k = 0; k < 4; ++k) vs[k] *= iw;
    mul4d(c.mvi, vs, o);
    os[0] = o[0];
    os[1] = o[1];
    os[2] = o[2];
}

// Last channel of the trilinear BORDER fetch at grid coordinate p (cell
// centres at integers), in double: 0 where p + 0.5 leaves [0, dims), corners
// outside the grid read 0.
template <int C, typename S, int L>
__device__ __forceinline__ double fetch_last_d(const S* __restrict__ g, Dims d, double px, double py, double pz) {
    if (!(px + 0.5 >= 0.0 && px + 0.5 < d.x && py + 0.5 >= 0.0 && py + 0.5 < d.y && pz + 0.5 >= 0.0 &&
          pz + 0.5 < d.z))
        return 0.0;
    const double fx = floor(px), fy = floor(py), fz = floor(pz);
    const int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
    const double wx = px - fx, wy = py - fy, wz = pz - fz;
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int x = x0 + (k & 1), y = y0 + ((k >> 1) & 1), z = z0 + ((k >> 2) & 1);
        if (x < 0 || y < 0 || z < 0 || x >= d.x || y >= d.y || z >= d.z) continue;
        const double w = ((k & 1) ? wx : 1.0 - wx) * (((k >> 1) & 1) ? wy : 1.0 - wy) * (((k >> 2) & 1) ? wz : 1.0 - wz);
        acc += w * (double)Load<C, S>::at(g, cell_index<L>(x, y, z, d)).v[C - 1];
    }
    return acc;
}

template <int C, typename S, int L>
__global__ void __launch_bounds__(CK_THREADS)
    k_raymarch_check(const S* __restrict__ in, Dims din, const __grid_constant__ CheckTable tab, int W, int H, int D,
                     const float* __restrict__ img, int stride, double* result) {
    const int p = blockIdx.y;
    const int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * stride;
    double abs_err = 0.0, ref_max = 0.0;
    if (ray < (int64_t)W * H) {
        const int y = (int)(ray / W), x = (int)(ray - (int64_t)y * W);
        const CamD& cam = tab.cam[p];
        const S* g = in + (size_t)tab.in_batch[p] * slice_cells<L>(din) * C;
        const double zmax = (double)max(D - 1, 1);
        double nearp[3], farp[3], st[3];
        idx_to_os_d(cam, x + 0.5, y + 0.5, 0.5, W, H, D, nearp);
        idx_to_os_d(cam, x + 0.5, y + 0.5, zmax + 0.5, W, H, D, farp);
        for (int k = 0; k < 3; ++k) st[k] = (farp[k] - nearp[k]) / zmax;
        double dens = 0.0;
        for (int i = 0; i < D; ++i) {
            const double s = fetch_last_d<C, S, L>(g, din, nearp[0] + i * st[0] - 0.5, nearp[1] + i * st[1] - 0.5,
                                                   nearp[2] + i * st[2] - 0.5);
            dens = C == 1 ? dens + s : fmax(dens + s, 0.0);
        }
        const double got = (double)img[((int64_t)tab.out_slot[p] * H * W + ray) * C + (C - 1)];
        deviation(got, dens, abs_err, ref_max);
    }
    warp_max_to(result, abs_err, ref_max);
}

template <int C, typename S>
static void rm_check_c(const void* in, int layout, Dims din, const CheckTable& t, int W, int H, int D,
                       const float* img, int stride, double* result, cudaStream_t s) {
    const int64_t rays = ((int64_t)W * H + stride - 1) / stride;
    const dim3 grid((unsigned)((rays + CK_THREADS - 1) / CK_THREADS), (unsigned)t.n);
    if (layout == LAYOUT_BRICK)
        k_raymarch_check<C, S, LAYOUT_BRICK><<<grid, CK_THREADS, 0, s>>>((const S*)in, din, t, W, H, D, img, stride,
                                                                        result);
    else
        k_raymarch_check<C, S, LAYOUT_FLAT><<<grid, CK_THREADS, 0, s>>>((const S*)in, din, t, W, H, D, img, stride,
                                                                       result);
}

bool launch_raymarch_check(const void* in, int dtype, int layout, int C, Dims din, const std::vector<CheckTable>& tabs,
                           int W, int H, int D, const float* img, int stride, double* result, cudaStream_t s) {
    if (!cuda_ok(cudaMemsetAsync(result, 0, 2 * sizeof(double), s), "zero check result")) return false;
    for (const CheckTable& t : tabs) {
        if (dtype == 0) {
            if (C == 4) rm_check_c<4, float>(in, layout, din, t, W, H, D, img, stride, result, s);
            else if (C == 2) rm_check_c<2, float>(in, layout, din, t, W, H, D, img, stride, result, s);
            else rm_check_c<1, float>(in, layout, din, t, W, H, D, img, stride, result, s);
        } else {
            if (C == 4) rm_check_c<4, __nv_bfloat16>(in, layout, din, t, W, H, D, img, stride, result, s);
            else if (C == 2) rm_check_c<2, __nv_bfloat16>(in, layout, din, t, W, H, D, img, stride, result, s);
            else rm_check_c<1, __nv_bfloat16>(in, layout, din, t, W, H, D, img, stride, result, s);
        }
        if (!launched(1, "raymarch check launch")) return false;
    }
    return true;
}

}  // namespace gft
