// C entry points onto the reference's resampling launchers (resample_grid.cu.cc),
// for generating golden vectors.  ORACLE / TEST INFRASTRUCTURE ONLY.
// Declarations as in resample_grid.cc:253-266, :449-467, :628-648, :805-826, :981-984.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "resample_grid.hpp"

#define DECL(C)                                                                                                 \
    template <>                                                                                                 \
    void SampleGridKernel<GPUDevice, float, C>::operator()(                                                     \
        const GPUDevice& d, const void* input, const long long int* input_shape, const float* M, const float* V, \
        const float* P, const float* frustum, int32_t numCameras, uint8_t* mipAtlas,                            \
        const Sampling::CoordinateMode coordinateMode, const Sampling::SamplerSettings, const bool globalSampling, \
        void* output, const long long int* output_shape);
DECL(1)
DECL(2)
DECL(4)
#undef DECL

#define GRAD_DECL(NAME)                                                                                          \
    void NAME(const void* _input, const long long int* input_shape, const float* M, const float* V, const float* P, \
              const float* _frustum, int32_t numCameras, const Sampling::CoordinateMode coordinateMode,          \
              const Sampling::SamplerSettings samplingSettings, const bool globalSampling, const void* _output_grad, \
              const long long int* output_shape, void* _input_grad, uint32_t* sample_count_buffer);
GRAD_DECL(SampleRGridGradKernelLauncher)
GRAD_DECL(SampleRGGridGradKernelLauncher)
GRAD_DECL(SampleRGBAGridGradKernelLauncher)
#undef GRAD_DECL

#define LUT_DECL(NAME)                                                                                           \
    void NAME(const void* input, const long long int* input_shape, int32_t numCameras, const float* lookup,      \
              uint8_t* mipAtlas, const Sampling::CoordinateMode coordinateMode, Sampling::SamplerSettings,        \
              const bool globalSampling, const bool relative, const bool normalized, void* output,               \
              const long long int* output_shape);
LUT_DECL(SampleRGridLuTKernelLauncher)
LUT_DECL(SampleRGGridLuTKernelLauncher)
LUT_DECL(SampleRGBAGridLuTKernelLauncher)
#undef LUT_DECL

#define LUTG_DECL(NAME)                                                                                          \
    void NAME(const void* _input, const long long int* input_shape, int32_t numCameras, const float* _lookup,    \
              const Sampling::CoordinateMode coordinateMode, const Sampling::SamplerSettings samplingSettings,   \
              const bool globalSampling, const bool relative, const bool normalized, const void* _output_grad,   \
              const long long int* output_shape, void* _input_grad, void* _lookup_grad,                         \
              uint32_t* sample_count_buffer);
LUTG_DECL(SampleRGridLuTGradKernelLauncher)
LUTG_DECL(SampleRGGridLuTGradKernelLauncher)
LUTG_DECL(SampleRGBAGridLuTGradKernelLauncher)
#undef LUTG_DECL

void ComputeLoDKernelLauncher(const long long int* input_shape, const float* MV, const float* P,
                              const float* _frustum, const Sampling::CoordinateMode coordinateMode, void* output,
                              const long long int* output_shape);

// The op constructors zero the settings and set the attributes
// (resample_grid.cc:274-305); setupMipAtlas then caps the level count
// (resample_grid.cc:201-220).
static Sampling::SamplerSettings settings(const long long* in_shape, int filter, int boundary, int mip, int levels,
                                          float bias, float cco) {
    Sampling::SamplerSettings s;
    memset(&s, 0, sizeof(s));
    s.filterMode = (decltype(s.filterMode))filter;
    s.boundaryMode = (decltype(s.boundaryMode))boundary;
    s.mipMode = (decltype(s.mipMode))mip;
    s.mipLevel = levels;
    s.mipBias = bias;
    s.cellCenterOffset = cco;
    for (int m = 1; m < s.mipLevel + 1; ++m) {
        long long e = (in_shape[1] >> m) * (in_shape[2] >> m) * (in_shape[3] >> m);
        if (e <= 0) {
            s.mipLevel = m - 1;
            break;
        }
    }
    return s;
}

extern "C" {

// out_shape6 = [N, V or 1, Do, Ho, Wo, C]; mip_atlas: device scratch (see make_golden.py)
int ref_sample_transform(const float* in, const long long* in_shape, const float* M, const float* V, const float* P,
                         const float* F, int nc, uint8_t* mip_atlas, int coord_mode, int filter, int boundary, int mip,
                         int levels, float bias, int global, float* out, const long long* out_shape6) {
    GPUDevice d;
    const auto s = settings(in_shape, filter, boundary, mip, levels, bias, 0.5f);
    const auto cm = (Sampling::CoordinateMode)coord_mode;
    switch (in_shape[4]) {
        case 1: SampleGridKernel<GPUDevice, float, 1>()(d, in, in_shape, M, V, P, F, nc, mip_atlas, cm, s, global, out, out_shape6); break;
        case 2: SampleGridKernel<GPUDevice, float, 2>()(d, in, in_shape, M, V, P, F, nc, mip_atlas, cm, s, global, out, out_shape6); break;
        case 4: SampleGridKernel<GPUDevice, float, 4>()(d, in, in_shape, M, V, P, F, nc, mip_atlas, cm, s, global, out, out_shape6); break;
        default: return -1;
    }
    return (int)cudaDeviceSynchronize();
}

int ref_sample_transform_grad(const float* in, const long long* in_shape, const float* M, const float* V,
                              const float* P, const float* F, int nc, int coord_mode, int filter, int boundary,
                              int global, const float* out_grad, const long long* out_shape6, float* in_grad,
                              uint32_t* counts) {
    const auto s = settings(in_shape, filter, boundary, 0, 0, 0.f, 0.5f);
    const auto cm = (Sampling::CoordinateMode)coord_mode;
    switch (in_shape[4]) {
        case 1: SampleRGridGradKernelLauncher(in, in_shape, M, V, P, F, nc, cm, s, global, out_grad, out_shape6, in_grad, counts); break;
        case 2: SampleRGGridGradKernelLauncher(in, in_shape, M, V, P, F, nc, cm, s, global, out_grad, out_shape6, in_grad, counts); break;
        case 4: SampleRGBAGridGradKernelLauncher(in, in_shape, M, V, P, F, nc, cm, s, global, out_grad, out_shape6, in_grad, counts); break;
        default: return -1;
    }
    return (int)cudaDeviceSynchronize();
}

int ref_sample_lut(const float* in, const long long* in_shape, int nc, const float* lut, uint8_t* mip_atlas,
                   int filter, int boundary, int mip, int levels, float bias, float cco, int global, int relative,
                   int normalized, float* out, const long long* out_shape6) {
    const auto s = settings(in_shape, filter, boundary, mip, levels, bias, cco);
    switch (in_shape[4]) {
        case 1: SampleRGridLuTKernelLauncher(in, in_shape, nc, lut, mip_atlas, Sampling::LuT, s, global, relative, normalized, out, out_shape6); break;
        case 2: SampleRGGridLuTKernelLauncher(in, in_shape, nc, lut, mip_atlas, Sampling::LuT, s, global, relative, normalized, out, out_shape6); break;
        case 4: SampleRGBAGridLuTKernelLauncher(in, in_shape, nc, lut, mip_atlas, Sampling::LuT, s, global, relative, normalized, out, out_shape6); break;
        default: return -1;
    }
    return (int)cudaDeviceSynchronize();
}

int ref_sample_lut_grad(const float* in, const long long* in_shape, int nc, const float* lut, int filter,
                        int boundary, float cco, int global, int relative, int normalized, const float* out_grad,
                        const long long* out_shape6, float* in_grad, float* lut_grad, uint32_t* counts) {
    const auto s = settings(in_shape, filter, boundary, 0, 0, 0.f, cco);
    switch (in_shape[4]) {
        case 1: SampleRGridLuTGradKernelLauncher(in, in_shape, nc, lut, Sampling::LuT, s, global, relative, normalized, out_grad, out_shape6, in_grad, lut_grad, counts); break;
        case 2: SampleRGGridLuTGradKernelLauncher(in, in_shape, nc, lut, Sampling::LuT, s, global, relative, normalized, out_grad, out_shape6, in_grad, lut_grad, counts); break;
        case 4: SampleRGBAGridLuTGradKernelLauncher(in, in_shape, nc, lut, Sampling::LuT, s, global, relative, normalized, out_grad, out_shape6, in_grad, lut_grad, counts); break;
        default: return -1;
    }
    return (int)cudaDeviceSynchronize();
}

// in_shape5 / out_shape5 = [num, D, H, W, 4]
int ref_lod_transform(const long long* in_shape5, const float* MV, const float* P, const float* F, int inverse,
                      float* out, const long long* out_shape5) {
    ComputeLoDKernelLauncher(in_shape5, MV, P, F, inverse ? Sampling::TransformLinDepthReverse : Sampling::TransformLinDepth,
                             out, out_shape5);
    return (int)cudaDeviceSynchronize();
}

}  // extern "C"
