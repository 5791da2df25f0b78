// C entry points onto the reference's reduce-blend launchers (reduce_blend.cu.cc),
// for generating golden vectors.  ORACLE / TEST INFRASTRUCTURE ONLY.
// Declarations as in reduce_blend.cc:50-58 and :140-149.
#include <cuda_runtime.h>

#include "blending_settings.hpp"

void GridBlendRKernelLauncher(const float*, const long long int*, const Blending::BlendMode, const bool, float*,
                              const long long int*);
void GridBlendRGKernelLauncher(const float*, const long long int*, const Blending::BlendMode, const bool, float*,
                               const long long int*);
void GridBlendRGBAKernelLauncher(const float*, const long long int*, const Blending::BlendMode, const bool, float*,
                                 const long long int*);
void ReduceGridBlendRGradKernelLauncher(const float*, float*, const long long int*, const Blending::BlendMode,
                                        const bool, const float*, const float*, const long long int*);
void ReduceGridBlendRGGradKernelLauncher(const float*, float*, const long long int*, const Blending::BlendMode,
                                         const bool, const float*, const float*, const long long int*);
void ReduceGridBlendRGBAGradKernelLauncher(const float*, float*, const long long int*, const Blending::BlendMode,
                                           const bool, const float*, const float*, const long long int*);

extern "C" {

// out_shape5 = [N, D or 1, H, W, C] as ReduceGridBlendOp passes it (reduce_blend.cc:96-99)
int ref_blend_fwd(const float* in, const long long* in_shape, int mode, int keep, float* out,
                  const long long* out_shape5) {
    const auto m = (Blending::BlendMode)mode;
    try {
        switch (in_shape[4]) {
            case 1: GridBlendRKernelLauncher(in, in_shape, m, keep, out, out_shape5); break;
            case 2: GridBlendRGKernelLauncher(in, in_shape, m, keep, out, out_shape5); break;
            case 4: GridBlendRGBAKernelLauncher(in, in_shape, m, keep, out, out_shape5); break;
            default: return -1;
        }
    } catch (...) {
        return -2;
    }
    return (int)cudaDeviceSynchronize();
}

int ref_blend_bwd(const float* in, float* in_grad, const long long* in_shape, int mode, int keep, const float* out,
                  const float* out_grad, const long long* out_shape5) {
    const auto m = (Blending::BlendMode)mode;
    try {
        switch (in_shape[4]) {
            case 1: ReduceGridBlendRGradKernelLauncher(in, in_grad, in_shape, m, keep, out, out_grad, out_shape5); break;
            case 2: ReduceGridBlendRGGradKernelLauncher(in, in_grad, in_shape, m, keep, out, out_grad, out_shape5); break;
            case 4: ReduceGridBlendRGBAGradKernelLauncher(in, in_grad, in_shape, m, keep, out, out_grad, out_shape5); break;
            default: return -1;
        }
    } catch (...) {
        return -2;
    }
    return (int)cudaDeviceSynchronize();
}

}  // extern "C"
