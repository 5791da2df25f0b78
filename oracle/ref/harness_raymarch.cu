// C entry points onto the reference's raymarch launchers (raymarch_grid.cu.cc),
// for generating golden vectors.  ORACLE / TEST INFRASTRUCTURE ONLY.
// The declarations mirror raymarch_grid.cc:150-167 (DECLARE_GPU_SPEC).
#include <cuda_runtime.h>
#include <stdint.h>

#include "raymarch_grid.hpp"

#define DECL(C)                                                                                                  \
    template <>                                                                                                  \
    void RaymarchGridKernel<GPUDevice, float, C>::operator()(                                                    \
        const GPUDevice& d, const float* input, const long long int* input_shape, const float* M, const float* V, \
        const float* P, const float* frustum, int32_t numCameras, const Sampling::FilterMode filterMode,          \
        const Sampling::BoundaryMode boundaryMode, const Blending::BlendMode blendMode, const bool globalSampling, \
        float* output, const long long int* output_shape);                                                       \
    template <>                                                                                                  \
    void RaymarchGridGradKernel<GPUDevice, float, C>::operator()(                                                \
        const GPUDevice& d, const float* input, float* inputGrads, float* sampleBuffer,                          \
        sampleCount_t* sampleCounter, const long long int* input_shape, const float* M, const float* V,          \
        const float* P, const float* frustum, int32_t numCameras, const Sampling::FilterMode filterMode,          \
        const Sampling::BoundaryMode boundaryMode, const Blending::BlendMode blendMode, const bool globalSampling, \
        const float* output, const float* outputGrads, const long long int* output_shape);
DECL(1)
DECL(2)
DECL(4)
#undef DECL

extern "C" {

// output_shape6 = [N, V, D, H, W, C] (D = depth samples); M/V/P/F host arrays.
int ref_raymarch_fwd(const float* in, const long long* in_shape, const float* M, const float* V, const float* P,
                     const float* F, int nc, int filter, int boundary, int blend, int global, float* out,
                     const long long* out_shape6) {
    GPUDevice d;
    const auto fm = (Sampling::FilterMode)filter;
    const auto bm = (Sampling::BoundaryMode)boundary;
    const auto bl = (Blending::BlendMode)blend;
    switch (in_shape[4]) {
        case 1: RaymarchGridKernel<GPUDevice, float, 1>()(d, in, in_shape, M, V, P, F, nc, fm, bm, bl, global, out, out_shape6); break;
        case 2: RaymarchGridKernel<GPUDevice, float, 2>()(d, in, in_shape, M, V, P, F, nc, fm, bm, bl, global, out, out_shape6); break;
        case 4: RaymarchGridKernel<GPUDevice, float, 4>()(d, in, in_shape, M, V, P, F, nc, fm, bm, bl, global, out, out_shape6); break;
        default: return -1;
    }
    return (int)cudaDeviceSynchronize();
}

// sample_buffer: D*H*W*C floats, sample_counter: D*H*W floats (raymarch_grid.cc:420-436)
int ref_raymarch_bwd(const float* in, float* in_grad, float* sample_buffer, float* sample_counter,
                     const long long* in_shape, const float* M, const float* V, const float* P, const float* F, int nc,
                     int filter, int boundary, int blend, int global, const float* out, const float* out_grad,
                     const long long* out_shape6) {
    GPUDevice d;
    const auto fm = (Sampling::FilterMode)filter;
    const auto bm = (Sampling::BoundaryMode)boundary;
    const auto bl = (Blending::BlendMode)blend;
    switch (in_shape[4]) {
        case 1: RaymarchGridGradKernel<GPUDevice, float, 1>()(d, in, in_grad, sample_buffer, sample_counter, in_shape, M, V, P, F, nc, fm, bm, bl, global, out, out_grad, out_shape6); break;
        case 2: RaymarchGridGradKernel<GPUDevice, float, 2>()(d, in, in_grad, sample_buffer, sample_counter, in_shape, M, V, P, F, nc, fm, bm, bl, global, out, out_grad, out_shape6); break;
        case 4: RaymarchGridGradKernel<GPUDevice, float, 4>()(d, in, in_grad, sample_buffer, sample_counter, in_shape, M, V, P, F, nc, fm, bm, bl, global, out, out_grad, out_shape6); break;
        default: return -1;
    }
    return (int)cudaDeviceSynchronize();
}

}  // extern "C"
