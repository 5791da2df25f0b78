/*
 * gft.h -- C ABI of the GB300 render + advect hot path (libgft.so).
 *
 * Every entry point replaces one op of the reference's TensorFlow custom-op
 * libraries (phitest/render/cuda/src/{resample_grid,reduce_blend,raymarch_grid}.cc)
 * with the same inputs, attributes and output layout, as plain pointers:
 *
 *   - tensors are NDHWC, channel counts C in {1, 2, 4} (C == 3 is rejected as in
 *     resample_grid.cc:330-331);
 *   - tensor data pointers are DEVICE pointers; the caller allocates every
 *     output, gradient and workspace buffer (query sizes with *_workspace_size);
 *   - alignment: a tensor of C channels is accessed C elements at a time, so
 *     its pointer is a multiple of C x element bytes (16 for C == 4 fp32, 8
 *     for C == 4 bf16); RGB + density images, light-composition outputs and
 *     lookup tables (4 floats per entry) are 16-byte aligned; workspaces and
 *     sample stores are 16-byte aligned.  cudaMalloc and the torch allocator
 *     give 256 bytes.  A misaligned tensor is GFT_ERR_INVALID_ARGUMENT, a
 *     misaligned workspace or sample store GFT_ERR_WORKSPACE;
 *   - 4x4 matrices and frustum parameters are HOST pointers (the reference
 *     declares them HostMemory, resample_grid.cc:1070-1105): 16 floats read
 *     column-major, i.e. numpy ``matrix.transpose()`` flattened, as
 *     phitest/render/renderer.py:108-111 passes them; frustum = [near, far,
 *     left, right, top, bottom] (camera.py:61-62);
 *   - ``stream`` is a cudaStream_t (NULL = legacy default stream); every call is
 *     stream-ordered, never synchronises the device, allocates no device memory
 *     and keeps no per-call global state, so calls are re-entrant and can be
 *     captured into CUDA graphs;
 *   - every function returns a gft_status and never exits the process; the
 *     message of the last failure on the calling thread is gft_last_error().
 *
 * Enum values equal the reference's (sampling_settings_v2.hpp:9-10,
 * sampling_settings.hpp:14-18 and :56-65, blending_settings.hpp:6-12).
 */
#ifndef GFT_H
#define GFT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

typedef enum {
    GFT_OK = 0,
    GFT_ERR_INVALID_ARGUMENT = 1, /* TF errors::InvalidArgument */
    GFT_ERR_UNIMPLEMENTED = 2,    /* TF errors::Unimplemented */
    GFT_ERR_CUDA = 3,             /* TF errors::Internal after a CUDA failure */
    GFT_ERR_WORKSPACE = 4         /* workspace missing or too small */
} gft_status;

typedef enum { GFT_FILTER_NEAREST = 0, GFT_FILTER_LINEAR = 1, GFT_FILTER_MIN = 2, GFT_FILTER_MAX = 3 } gft_filter;
typedef enum { GFT_BOUNDARY_BORDER = 0, GFT_BOUNDARY_CLAMP = 1, GFT_BOUNDARY_WRAP = 2 } gft_boundary;
typedef enum { GFT_MIP_NONE = 0, GFT_MIP_NEAREST = 1, GFT_MIP_LINEAR = 2 } gft_mip;
typedef enum {
    GFT_BLEND_BEER_LAMBERT = 0,
    GFT_BLEND_BEER_LAMBERT_EXCLUSIVE = 1,
    GFT_BLEND_ALPHA = 2,
    GFT_BLEND_ALPHA_ADDITIVE = 3,
    GFT_BLEND_ADDITIVE = 4
} gft_blend;
typedef enum {
    GFT_COORD_TRANSFORM_LINDEPTH = 0,
    GFT_COORD_TRANSFORM_LINDEPTH_REVERSE = 1,
    GFT_COORD_TRANSFORM = 3,
    GFT_COORD_TRANSFORM_REVERSE = 4
} gft_coord;
/* Storage type of density-like inputs; all arithmetic is fp32. */
typedef enum { GFT_DTYPE_F32 = 0, GFT_DTYPE_BF16 = 1 } gft_dtype;
/* OR-ed into the input_dtype of gft_raymarch_grid_transform(_grad): the input
 * grid, and the input gradient the adjoint writes, are stored per batch slice
 * in 2x2x2-voxel bricks instead of NDHWC rows: voxel (x, y, z) of a D x H x W
 * slice is cell ((z/2 * ceil(H/2) + y/2) * ceil(W/2) + x/2) * 8 +
 * (z%2)*4 + (y%2)*2 + x%2 of ceil(D/2)*ceil(H/2)*ceil(W/2)*8 cells (each C
 * values); cells outside the grid are never read.  A warp's corner gathers
 * then touch fewer cache lines.  LINEAR interpolation only.  No counterpart in
 * the reference (which reads NDHWC rows); gft_light_compose writes this
 * layout directly. */
#define GFT_LAYOUT_BRICK 0x10
/* GFT_GRAD_REFERENCE reproduces the reference's gradient normalisations
 * (per-voxel sample count for resample/lookup, resample_grid.cu.cc:814-832;
 * per-camera sum of trilinear weights for raymarch, raymarch_grid.cu.cc:519-568).
 * GFT_GRAD_EXACT returns the true adjoint of the forward op. */
typedef enum { GFT_GRAD_REFERENCE = 0, GFT_GRAD_EXACT = 1 } gft_grad_mode;
/* MacCormack clamp of VelocityGrid.warp (data_structures.py:870-905). */
typedef enum { GFT_CLAMP_NONE = 0, GFT_CLAMP_MC_SMOOTH = 1, GFT_CLAMP_NEGATIVE = 2 } gft_clamp;

const char* gft_last_error(void);
const char* gft_version(void);
/* Kernels this library has launched in the process so far (all threads). */
unsigned long long gft_launch_count(void);

/* ---- RaymarchGridTransform (raymarch_grid.cc:28-52, launcher raymarch_grid.cu.cc:222-294) ----
 * input  [N, D, H, W, C] (input_dtype storage)
 * matrix_m num_m x 16 (num_m == N), matrix_v / matrix_p num_cameras x 16, frustum num_cameras x 6
 * output_shape = (depth samples, height, width)
 * output [N, separate_camera_batch ? num_cameras : 1, height, width, C] fp32 */
gft_status gft_raymarch_grid_transform(
    const void* input, int32_t input_dtype, const int64_t input_shape[5],
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
    int32_t interpolation, int32_t boundary, int32_t blending_mode, int32_t separate_camera_batch,
    float* output, void* stream);

/* ---- RaymarchGridTransformGrad (raymarch_grid.cc:56-76, launcher raymarch_grid.cu.cc:451-574) ----
 * output / output_grad are the forward result and its gradient (same shape as the
 * forward output); input_grad [N, D, H, W, C] fp32 is overwritten.
 * LINEAR interpolation only (raymarch_grid.cc:65). */
size_t gft_raymarch_grid_transform_grad_workspace_size(
    const int64_t input_shape[5], int32_t num_cameras, int32_t separate_camera_batch, int32_t grad_mode);
gft_status gft_raymarch_grid_transform_grad(
    const void* input, int32_t input_dtype, const int64_t input_shape[5],
    const float* output, const float* output_grad,
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
    int32_t interpolation, int32_t boundary, int32_t blending_mode, int32_t separate_camera_batch,
    int32_t grad_mode, float* input_grad, void* workspace, size_t workspace_bytes, void* stream);
/* Sample store (no counterpart in the reference, whose gradient re-samples the
 * grid): gft_raymarch_grid_transform_store is gft_raymarch_grid_transform
 * (LINEAR interpolation) that also writes the ray samples it blends that can
 * be non-zero, within each ray's clipped step range, into `samples` (an
 * internal layout: per camera, 8x16-pixel tile, depth sample and warp a
 * ballot word and a pool offset, occupancy maps of the input, then a pool of
 * C-float cells that warps fill in chunks).  gft_raymarch_grid_transform_grad_stored
 * is gft_raymarch_grid_transform_grad reading those samples instead of
 * re-sampling the input; input, geometry, output_shape and samples_bytes must
 * be those of the store call, with the input unchanged in between.  The
 * adjoint then uses the samples at the forward's positions, which differ from
 * re-sampled ones by float rounding only.
 * samples_bytes may be anything from gft_raymarch_grid_transform_samples_min_size
 * (no pool) to gft_raymarch_grid_transform_samples_size (a pool for every
 * sample the launch could store): samples that do not fit the pool are not
 * stored and the adjoint re-samples the grid for them, with the same result
 * up to rounding.  Typical plumes store a few percent of the full bound. */
size_t gft_raymarch_grid_transform_samples_size(
    const int64_t input_shape[5], int32_t num_cameras, const int32_t output_shape[3],
    int32_t separate_camera_batch);
size_t gft_raymarch_grid_transform_samples_min_size(
    const int64_t input_shape[5], int32_t num_cameras, const int32_t output_shape[3],
    int32_t separate_camera_batch);
gft_status gft_raymarch_grid_transform_store(
    const void* input, int32_t input_dtype, const int64_t input_shape[5],
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
    int32_t interpolation, int32_t boundary, int32_t blending_mode, int32_t separate_camera_batch,
    float* output, float* samples, size_t samples_bytes, void* stream);
gft_status gft_raymarch_grid_transform_grad_stored(
    const void* input, int32_t input_dtype, const int64_t input_shape[5],
    const float* output, const float* output_grad,
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
    int32_t interpolation, int32_t boundary, int32_t blending_mode, int32_t separate_camera_batch,
    int32_t grad_mode, const float* samples, size_t samples_bytes, float* input_grad,
    void* workspace, size_t workspace_bytes, void* stream);
/* gft_raymarch_grid_transform_grad_projected: gft_raymarch_grid_transform_grad_stored
 * (samples may be NULL: the grid is re-sampled, as gft_raymarch_grid_transform_grad)
 * whose gradient is accumulated already projected onto two channels:
 * input_grad [N, cells, 2] holds (projection[0..3] . g, projection[4..7] . g)
 * per cell for the 4-channel gradient g of the plain call.  Each sample's
 * 4-channel adjoint is projected before its trilinear reduction, so the
 * reductions move half the bytes; the result equals the projection of the
 * plain gradient up to float rounding.  4 channels, GFT_LAYOUT_BRICK,
 * GFT_GRAD_REFERENCE or GFT_GRAD_EXACT (with GFT_GRAD_WEIGHTS_READY as
 * usual), also GFT_GRAD_DETERMINISTIC (two int64 sums per cell; the bound
 * of the fixed point scales by the larger of sum |projection[0..3]| and
 * sum |projection[4..7]|); the same workspace.  No counterpart in the
 * reference. */
/* OR'ed into grad_mode of gft_raymarch_grid_transform_grad_projected with
 * GFT_GRAD_REFERENCE (not GFT_GRAD_WEIGHTS_READY): the reference
 * normalisation in one pass.  input_grad [pairs, cells, 2] receives, per
 * (batch, camera) pair, the projected corner sums unnormalised, and the
 * first pairs x cells floats of the workspace the pair's per-voxel sums of
 * the trilinear weights (both in the brick layout, cells =
 * ceil(D/2)*ceil(H/2)*ceil(W/2)*8); the caller divides each pair's sums by
 * its weight sums where those are positive and adds the pairs
 * (gft_light_compose_factored_grad_cameras does so).  The reference
 * divides each camera's gradient by that camera's sample weights
 * (raymarch_grid.cu.cc:519-568) after a separate counting pass; here both
 * sums come from the same walk over the samples. */
#define GFT_GRAD_CAMERA_SUMS 0x800
gft_status gft_raymarch_grid_transform_grad_projected(
    const void* input, int32_t input_dtype, const int64_t input_shape[5],
    const float* output, const float* output_grad,
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
    int32_t interpolation, int32_t boundary, int32_t blending_mode, int32_t separate_camera_batch,
    int32_t grad_mode, const float* samples, size_t samples_bytes, const float projection[8],
    float* input_grad, void* workspace, size_t workspace_bytes, void* stream);
/* The geometry-only first pass of the GFT_GRAD_REFERENCE raymarch gradient:
 * per (batch, camera) pair the reciprocals of the per-voxel sums of the
 * trilinear weights of all ray samples (the reference's float sampleCounter,
 * raymarch_grid.cu.cc:446-456; 0 where no sample reaches a voxel), written
 * into the workspace of gft_raymarch_grid_transform_grad in an internal
 * layout (2x2x2-voxel bricks).  It needs neither the forward output nor its
 * gradient, so a caller can run it on another stream while the forward pass
 * is still running; the gradient call
 * then takes grad_mode GFT_GRAD_REFERENCE | GFT_GRAD_WEIGHTS_READY, the same
 * geometry and workspace, and skips the pass.  No counterpart in the
 * reference, whose gradient kernel accumulates the sums itself. */
#define GFT_GRAD_WEIGHTS_READY 0x100
/* OR'ed into grad_mode of the raymarch gradients (_grad, _grad_stored,
 * _multi_grad, _views_grad) and of gft_advect_grad: a deterministic adjoint.
 * No counterpart in the reference, whose gradient scatters accumulate with
 * floating-point atomics in whatever order the threads arrive, so its
 * gradients differ from run to run in the last bits.  Here every scatter adds
 * fixed-point int64 contributions (integer addition does not depend on the
 * order) whose power-of-two scale comes from a bound on each voxel's partial
 * sums computed on the GPU from maxima of the inputs; the result is then
 * converted to fp32.  Gradients are bit-identical from run to run and as
 * accurate as the float path or more.  Raymarch: BEER_LAMBERT or ADDITIVE
 * blending (any mode with C == 1); with GFT_GRAD_WEIGHTS_READY the workspace
 * must hold the weight sums of gft_raymarch_grid_transform_grad_weights_mode
 * called with the flag (integer sums; the same input shape, C included); the
 * workspace size queries take the flag (larger workspaces; for the advection
 * gradient gft_advect_grad_workspace_size_mode).  Advection: both lookup
 * scatters; with GFT_GRAD_FORWARD_READY the workspace must be that size and
 * hold gft_advect's intermediate at its start as usual.  Non-finite inputs
 * give a NaN gradient. */
#define GFT_GRAD_DETERMINISTIC 0x400
gft_status gft_raymarch_grid_transform_grad_weights(
    const int64_t input_shape[5],
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
    int32_t boundary, int32_t separate_camera_batch, void* workspace, size_t workspace_bytes, void* stream);
/* The same with grad_mode GFT_GRAD_REFERENCE or GFT_GRAD_REFERENCE |
 * GFT_GRAD_DETERMINISTIC (then the deterministic adjoint's integer weight
 * sums, in its workspace layout, ahead of a gradient call with
 * GFT_GRAD_WEIGHTS_READY | GFT_GRAD_DETERMINISTIC). */
gft_status gft_raymarch_grid_transform_grad_weights_mode(
    const int64_t input_shape[5],
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
    int32_t boundary, int32_t separate_camera_batch, int32_t grad_mode, void* workspace, size_t workspace_bytes,
    void* stream);

/* ---- RaymarchGridTransform over cameras of different image sizes ----
 * No counterpart op in the reference, which takes one output_shape per call
 * (raymarch_grid.cc:28-52): the reference renders uneven camera batches with
 * one call per image size.  Global sampling (every batch slice with every
 * camera).  output_shapes = num_cameras x (depth samples, height, width);
 * output (and output_grad) hold, for each batch slice n and camera c, an
 * H_c x W_c x C image, the cameras one after another: camera c of slice n
 * starts at pixel n * P + P_c, with P = sum of all H_c W_c and P_c the sum over
 * the cameras before c.  All cameras run in one launch (up to 16 per launch).
 * Semantics per camera are those of gft_raymarch_grid_transform(_grad). */
gft_status gft_raymarch_grid_transform_multi(
    const void* input, int32_t input_dtype, const int64_t input_shape[5],
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t* output_shapes,
    int32_t interpolation, int32_t boundary, int32_t blending_mode, float* output, void* stream);
size_t gft_raymarch_grid_transform_multi_grad_workspace_size(
    const int64_t input_shape[5], int32_t num_cameras, int32_t grad_mode);
gft_status gft_raymarch_grid_transform_multi_grad(
    const void* input, int32_t input_dtype, const int64_t input_shape[5],
    const float* output, const float* output_grad,
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t* output_shapes,
    int32_t interpolation, int32_t boundary, int32_t blending_mode,
    int32_t grad_mode, float* input_grad, void* workspace, size_t workspace_bytes, void* stream);
gft_status gft_raymarch_grid_transform_multi_grad_weights(
    const int64_t input_shape[5],
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t* output_shapes,
    int32_t boundary, void* workspace, size_t workspace_bytes, void* stream);
/* ---- RaymarchGridTransform over views bound to batch slices ----
 * No counterpart op in the reference.  As the _multi functions, but camera c
 * renders only batch slice camera_batch[c] (int32, host, num_cameras entries
 * in [0, N)): a batch of frames, each seen by its own cameras of their own
 * image sizes (the reference renders them with one call per frame and image
 * size).  output (and output_grad) hold the cameras' images one after another,
 * camera c starting at pixel P_c = sum over the cameras before c of H W; the
 * input gradient of slice n sums the adjoints of the cameras that render it.
 * The workspace of the reference-normalised gradient holds one weight-sum
 * grid per camera.  Up to 16 cameras per launch. */
gft_status gft_raymarch_grid_transform_views(
    const void* input, int32_t input_dtype, const int64_t input_shape[5],
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t* camera_batch, const int32_t* output_shapes,
    int32_t interpolation, int32_t boundary, int32_t blending_mode, float* output, void* stream);
size_t gft_raymarch_grid_transform_views_grad_workspace_size(
    const int64_t input_shape[5], int32_t num_cameras, int32_t grad_mode);
gft_status gft_raymarch_grid_transform_views_grad(
    const void* input, int32_t input_dtype, const int64_t input_shape[5],
    const float* output, const float* output_grad,
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t* camera_batch, const int32_t* output_shapes,
    int32_t interpolation, int32_t boundary, int32_t blending_mode,
    int32_t grad_mode, float* input_grad, void* workspace, size_t workspace_bytes, void* stream);
gft_status gft_raymarch_grid_transform_views_grad_weights(
    const int64_t input_shape[5],
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t* camera_batch, const int32_t* output_shapes,
    int32_t boundary, void* workspace, size_t workspace_bytes, void* stream);

/* ---- SampleGridTransform (resample_grid.cc:23-61, :268-447; launcher resample_grid.cu.cc:289-438) ----
 * output [N, separate_camera_batch ? num_cameras : 1, Do, Ho, Wo, C] fp32.
 * The workspace holds the mip pyramid (empty without mips) and, for the
 * forward coordinate modes with mips, an occupancy map of the input that
 * lets samples reading only zeros skip their LOD and fetches.
 * interpolation | GFT_SAMPLE_DENSE: the input is known to be dense (e.g. a
 * gradient), so the occupancy map is not built; the result is the same. */
#define GFT_SAMPLE_DENSE 0x100
size_t gft_sample_grid_transform_workspace_size(const int64_t input_shape[5], int32_t mipmapping, int32_t num_mipmaps);
gft_status gft_sample_grid_transform(
    const void* input, int32_t input_dtype, const int64_t input_shape[5],
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
    int32_t interpolation, int32_t boundary, int32_t mipmapping, int32_t num_mipmaps, float mip_bias,
    int32_t coordinate_mode, float cell_center_offset, int32_t separate_camera_batch,
    float* output, void* workspace, size_t workspace_bytes, void* stream);

/* ---- SampleGridTransformGrad (resample_grid.cc:64-84, :469-625; launcher resample_grid.cu.cc:863-1018) ----
 * Trilinear scatter adjoint (no mips, as the reference op).  output_grad
 * [N, V or 1, Do, Ho, Wo, C]; input_grad [N, D, H, W, C] overwritten. */
size_t gft_sample_grid_transform_grad_workspace_size(const int64_t input_shape[5]);
gft_status gft_sample_grid_transform_grad(
    const int64_t input_shape[5], const float* output_grad, const int64_t output_grad_shape[6],
    const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras,
    int32_t interpolation, int32_t boundary, int32_t coordinate_mode, float cell_center_offset,
    int32_t separate_camera_batch, int32_t grad_mode,
    float* input_grad, void* workspace, size_t workspace_bytes, void* stream);

/* ---- SampleGridLut (resample_grid.cc:86-109, :650-802; launcher resample_grid.cu.cc:498-660) ----
 * lookup [V, Do, Ho, Wo, 4] fp32 (x, y, z, LOD); output [N, V or 1, Do, Ho, Wo, C] fp32. */
size_t gft_sample_grid_lut_workspace_size(const int64_t input_shape[5], int32_t mipmapping, int32_t num_mipmaps);
gft_status gft_sample_grid_lut(
    const void* input, int32_t input_dtype, const int64_t input_shape[5],
    const float* lookup, const int64_t lookup_shape[5],
    int32_t interpolation, int32_t boundary, int32_t mipmapping, int32_t num_mipmaps, float mip_bias,
    float cell_center_offset, int32_t separate_camera_batch, int32_t relative_coords, int32_t normalized_coords,
    float* output, void* workspace, size_t workspace_bytes, void* stream);

/* ---- SampleGridLutGrad (resample_grid.cc:113-134, :828-979; launcher resample_grid.cu.cc:1083-1251) ----
 * input_grad [N, D, H, W, C] and lookup_grad [V, Do, Ho, Wo, 4] overwritten. */
size_t gft_sample_grid_lut_grad_workspace_size(const int64_t input_shape[5]);
gft_status gft_sample_grid_lut_grad(
    const float* input, const int64_t input_shape[5], const float* output_grad,
    const float* lookup, const int64_t lookup_shape[5],
    int32_t interpolation, int32_t boundary, float cell_center_offset,
    int32_t separate_camera_batch, int32_t relative_coords, int32_t normalized_coords, int32_t grad_mode,
    float* input_grad, float* lookup_grad, void* workspace, size_t workspace_bytes, void* stream);

/* ---- LodTransform (resample_grid.cc:136-154, :986-1064; kComputeLoD3D resample_grid.cu.cc:1288-1363) ----
 * output [num, Do, Ho, Wo, 4]: sampling position (xyz) and LOD (w). */
gft_status gft_lod_transform(
    const int32_t input_shape[3], const float* matrix_mv, const float* matrix_p, const float* frustum,
    int32_t num, const int32_t output_shape[3], int32_t inverse_transform, float* output, void* stream);

/* ---- ReduceGridBlend / ReduceGridBlendGrad (reduce_blend.cc:23-48; reduce_blend.cu.cc:34-244) ----
 * input [N, D, H, W, C]; output [N, D, H, W, C] (keep_dims) or [N, H, W, C]. */
gft_status gft_reduce_grid_blend(
    const float* input, const int64_t input_shape[5], int32_t blending_mode, int32_t keep_dims,
    float* output, void* stream);
gft_status gft_reduce_grid_blend_grad(
    const float* output_grad, const float* output, const float* input, const int64_t input_shape[5],
    int32_t blending_mode, int32_t keep_dims, int32_t grad_mode, float* input_grad, void* stream);

/* ---- Fused advection (VelocityGrid.warp, data_structures.py:870-905) ----
 * The reference composes it from SampleGridLut calls (renderer.py:445-460) on
 * lut = -dt * centered(v) (:819-833, :864-868); here one fused pass per stage.
 * density [N, D, H, W, C] (density_dtype); velocity components fp32 staggered
 * x [D, H, W+1], y [D, H+1, W], z [D+1, H, W] (shared by the N batch slices);
 * order 1 = semi-Lagrangian, 2 = MacCormack; boundary of the lookups. */
size_t gft_advect_workspace_size(const int64_t density_shape[5], int32_t order);
gft_status gft_advect(
    const void* density, int32_t density_dtype, const int64_t density_shape[5],
    const float* vel_x, const float* vel_y, const float* vel_z, float dt,
    int32_t order, int32_t clamp, int32_t boundary,
    float* output, void* workspace, size_t workspace_bytes, void* stream);
/* Allocation-free variant of gft_advect.  No counterpart in the reference.
 * For callers that cannot hand the library device memory: hosts whose device
 * memory belongs to an allocator they cannot call from the advection call site
 * (a plugin host or foreign-language runtime without a device allocator, or a
 * fixed-budget real-time loop that forbids new allocations).  Same arguments as
 * gft_advect minus the workspace; the MacCormack intermediate lives in a static
 * device array of gft_advect_noalloc_max_elements() floats (16 MiB, held by
 * every device that loads the library until the process exits), so
 * D*H*W*C above that limit is rejected with GFT_ERR_INVALID_ARGUMENT (order 1
 * needs no scratch and has no limit).  The function calls no cudaMalloc /
 * cudaFree and no allocating library routine.  Each call outside stream
 * capture looks up the array's device address on the current device (the
 * device current on the calling thread, which must own ``stream``); a call
 * made while ``stream`` is being captured reuses the address of that device's
 * last lookup, so make a first call on each device before any stream capture.
 * Every call shares the one array and each call overwrites it before reading
 * it, so nothing needs clearing, but calls whose kernels overlap on the GPU
 * (different streams without ordering) race on it. */
size_t gft_advect_noalloc_max_elements(void);
gft_status gft_advect_noalloc(
    const void* density, int32_t density_dtype, const int64_t density_shape[5],
    const float* vel_x, const float* vel_y, const float* vel_z, float dt,
    int32_t order, int32_t clamp, int32_t boundary, float* output, void* stream);
/* Gradient of gft_advect w.r.t. density and the staggered velocity components,
 * all overwritten.  In GFT_GRAD_REFERENCE mode each lookup's input gradient is
 * divided by its per-voxel sample count as the reference SampleGridLutGrad does.
 * grad_mode | GFT_GRAD_FORWARD_READY (order 2, N == 1 only): the workspace is
 * the one gft_advect was given for the same fp32 density, velocity, dt and
 * boundary, and still holds the MacCormack intermediate (the semi-Lagrangian
 * grid) that gft_advect left at its start; the gradient reads it instead of
 * recomputing it.  No counterpart in the reference, whose gradient re-runs its
 * lookups. */
#define GFT_GRAD_FORWARD_READY 0x200
size_t gft_advect_grad_workspace_size(const int64_t density_shape[5], int32_t order);
/* The workspace of gft_advect_grad for grad_mode (with its flags): larger with
 * GFT_GRAD_DETERMINISTIC (int64 scatter targets), else the size above. */
size_t gft_advect_grad_workspace_size_mode(const int64_t density_shape[5], int32_t order, int32_t grad_mode);
gft_status gft_advect_grad(
    const float* density, const int64_t density_shape[5],
    const float* vel_x, const float* vel_y, const float* vel_z, float dt,
    int32_t order, int32_t clamp, int32_t boundary, int32_t grad_mode,
    const float* output_grad,
    float* density_grad, float* vel_x_grad, float* vel_y_grad, float* vel_z_grad,
    void* workspace, size_t workspace_bytes, void* stream);

/* ---- Pipeline fusions (no counterpart op in the reference) ----
 * Each replaces a chain of tensor ops with which the reference's renderer
 * composes the shadow pass, the lighting and the image loss
 * (phitest/render/lighting.py:106-121 and :236-262, renderer.py:1012-1052);
 * elementwise products and sums round like those separate ops.
 *
 * gft_transmittance: input [N, D, H, W, 1] (light-frustum density x depth step),
 * output[z] = exp(-sum_{z' < z} input[z']) along D: ReduceGridBlend
 * BEER_LAMBERT keep_dims, the one-cell shift in depth and exp. */
gft_status gft_transmittance(const float* input, const int64_t shape[5], float* output, void* stream);
gft_status gft_transmittance_grad(const float* output, const float* output_grad, const int64_t shape[5],
                                  float* input_grad, void* stream);
/* gft_light_compose: density, transmittance [N, D, H, W, 1] (shape), light_color
 * [D, H, W, 3] shared by the batch; output [N, D, H, W, 4] =
 * concat(density * (transmittance * light_color + ambient), density) * scale,
 * in NDHWC rows (output_layout 0) or in the raymarch's brick layout
 * (output_layout GFT_LAYOUT_BRICK); the gradient reads output_grad (fp32) in
 * that layout.  output_layout | GFT_DTYPE_BF16: the output is stored in bf16
 * (the fp32 result rounded to nearest even), ready as a BF16-storage raymarch
 * input; output_grad stays fp32. */
gft_status gft_light_compose(const float* density, const float* transmittance, const float* light_color,
                             const int64_t shape[5], float ambient, float scale, int32_t output_layout,
                             void* output, void* stream);
gft_status gft_light_compose_grad(const float* density, const float* transmittance, const float* light_color,
                                  const int64_t shape[5], float ambient, float scale, int32_t output_layout,
                                  const float* output_grad, float* density_grad, float* transmittance_grad,
                                  void* stream);
/* A light whose colour is a per-voxel falloff times a constant colour (a
 * point or spot light: falloff x color x intensity, phitest/render/lighting.py:49-70,
 * the shadow map multiplied in at :144-147): gft_light_compose_factored is gft_light_compose
 * with light_color[v, c] = falloff[v] * light_rgb[c] (falloff [D, H, W, 1],
 * light_rgb 3 host floats), formed by the same rounded product as a
 * precomputed colour grid, so the output is identical.  Its adjoint needs
 * only two sums of the raymarch gradient g per cell:
 * (P, Q) = (scale rgb . g_rgb, scale (ambient (g_r + g_g + g_b) + g_density)),
 * i.e. the projection that gft_light_compose_projection writes (8 floats, for
 * gft_raymarch_grid_transform_grad_projected); then
 * density_grad = Q + transmittance * falloff * P and
 * transmittance_grad = density * falloff * P.  projected_grad [N, cells, 2]
 * fp32 in output_layout (rows or bricks).  No counterpart in the reference,
 * which forms the 4-channel gradient and differentiates the composition by
 * tensor ops. */
gft_status gft_light_compose_factored(const float* density, const float* transmittance, const float* falloff,
                                      const float light_rgb[3], const int64_t shape[5], float ambient, float scale,
                                      int32_t output_layout, void* output, void* stream);
gft_status gft_light_compose_projection(const float light_rgb[3], float ambient, float scale, float projection[8]);
gft_status gft_light_compose_factored_grad(const float* density, const float* transmittance, const float* falloff,
                                           const int64_t shape[5], int32_t output_layout,
                                           const float* projected_grad, float* density_grad,
                                           float* transmittance_grad, void* stream);
/* The same adjoint from per-camera sums (GFT_GRAD_CAMERA_SUMS): for batch
 * slice b, (P, Q) = sum over its num_cameras pairs c = b * num_cameras + k of
 * camera_sums[c] / weight_sums[c] where weight_sums[c] > 0; camera_sums
 * [N * num_cameras, cells, 2] and weight_sums [N * num_cameras, cells] in the
 * brick layout. */
gft_status gft_light_compose_factored_grad_cameras(const float* density, const float* transmittance,
                                                   const float* falloff, const int64_t shape[5], int32_t num_cameras,
                                                   const float* camera_sums, const float* weight_sums,
                                                   float* density_grad, float* transmittance_grad, void* stream);
/* gft_image_loss: image [pixels, 4] (rgb + density), target [pixels, 3],
 * background = 3 host floats; *loss (device) = mean over pixels and rgb of
 * (rgb + background * exp(-density) - target)^2, summed in a fixed order.
 * gft_image_loss_grad: image_grad [pixels, 4] for the device scalar loss_grad. */
size_t gft_image_loss_workspace_size(int64_t pixels);
gft_status gft_image_loss(const float* image, const float* target, const float background[3], int64_t pixels,
                          float* loss, void* workspace, size_t workspace_bytes, void* stream);
gft_status gft_image_loss_grad(const float* image, const float* target, const float background[3], int64_t pixels,
                               const float* loss_grad, float* image_grad, void* stream);
/* gft_image_loss_tonemap(_grad): the same loss of the tonemapped composite,
 * mean((tone(rgb + background * exp(-density)) - target)^2), with the
 * renderer's tonemapping folded in (phitest/render/renderer.py:528-541,
 * applied at :639-640): GFT_TONEMAP_NONE; CLIP_NEGATIVE max(c, 0);
 * SATURATE clip(c, 0, 1); NORMALIZE over all pixels and channels of the call,
 * c - min(c) where min(c) < 0, then divided by its maximum where that is > 0
 * (two reductions more; the gradient needs the workspace too, of the same
 * size, and four more launches).  Gradients: max(c, 0) and clip pass where
 * 0 <= c (<= 1); a full min / max reduction shares its gradient evenly among
 * the elements equal to it, as TensorFlow and PyTorch do.  The plain
 * gft_image_loss(_grad) are the GFT_TONEMAP_NONE case. */
#define GFT_TONEMAP_NONE 0
#define GFT_TONEMAP_CLIP_NEGATIVE 1
#define GFT_TONEMAP_SATURATE 2
#define GFT_TONEMAP_NORMALIZE 3
gft_status gft_image_loss_tonemap(const float* image, const float* target, const float background[3], int64_t pixels,
                                  int32_t tonemap, float* loss, void* workspace, size_t workspace_bytes,
                                  void* stream);
gft_status gft_image_loss_tonemap_grad(const float* image, const float* target, const float background[3],
                                       int64_t pixels, int32_t tonemap, const float* loss_grad, float* image_grad,
                                       void* workspace, size_t workspace_bytes, void* stream);

/* ---- Launch-configuration knobs (no counterpart in the reference) ----
 * Process-wide settings of how some kernels are launched, chosen per workload
 * by gft.autotune (which times the candidates with CUDA events).  They change
 * the launch shape only: results are the same for every value (bit for bit
 * for the gathers; up to the association of the sums for the segmented scans
 * and the order of the floating-point atomic additions for the scatters).  A launch reads them when it is issued, so a
 * captured CUDA graph keeps the values of its capture.
 *   GFT_KNOB_RAYMARCH_BLOCKS_PER_SM  0 (default): one block per 8x16-pixel tile;
 *                                    1-32: a persistent grid of that many
 *                                    blocks per SM walking the tiles
 *   GFT_KNOB_ADVECT_THREADS          threads per block of the advection
 *                                    kernels: 64, 128 or 256 (default)
 *   GFT_KNOB_RESAMPLE_THREADS        threads per block of the
 *                                    SampleGridTransform forward: 64, 128 or
 *                                    256 (default)
 *   GFT_KNOB_SCAN_SEGMENTS           depth segments per column of the
 *                                    transmittance scans: 4, 8 (default) or 16
 *   GFT_KNOB_WEIGHTS_BLOCKS_PER_SM   the grid of the reference-normalised
 *                                    gradient's weight pass alone: 0
 *                                    (default) as the other raymarch
 *                                    kernels, 1-32 a persistent grid of that
 *                                    many blocks per SM (a small grid leaves
 *                                    room for the kernels it overlaps when it
 *                                    runs ahead on another stream)
 *   GFT_KNOB_WEIGHTS_PIPELINE        0 (default) or 1: a GFT_GRAD_REFERENCE
 *                                    raymarch gradient whose weight sums are
 *                                    not ready (no GFT_GRAD_WEIGHTS_READY,
 *                                    not deterministic, at most 64 pairs)
 *                                    computes them camera by camera on a
 *                                    side stream the library owns (created
 *                                    when the knob is set to 1), each
 *                                    camera's weight pass running beside the
 *                                    previous camera's scatter, which then
 *                                    runs camera by camera; the side stream
 *                                    forks from and joins the call's stream
 *                                    through events, so a CUDA-graph capture
 *                                    records it
 * gft_set_knob returns GFT_ERR_INVALID_ARGUMENT for an unknown knob or value. */
#define GFT_KNOB_RAYMARCH_BLOCKS_PER_SM 0
#define GFT_KNOB_ADVECT_THREADS 1
#define GFT_KNOB_RESAMPLE_THREADS 2
#define GFT_KNOB_SCAN_SEGMENTS 3
#define GFT_KNOB_WEIGHTS_BLOCKS_PER_SM 4
#define GFT_KNOB_WEIGHTS_PIPELINE 5
#define GFT_KNOB_COUNT 6
gft_status gft_set_knob(int32_t knob, int32_t value);
int32_t gft_get_knob(int32_t knob);

/* ---- FP64 check step (no counterpart in the reference) ----
 * Double-precision recomputations on the GPU of the two FP32 results of the
 * step whose rounding compounds along a ray, on a strided sample, from the
 * same FP32 inputs the step used.  result (device, 16-byte aligned): two
 * doubles, overwritten: the largest |fp32 - fp64| and the largest |fp64|
 * over the sample (their ratio is the max-norm relative error).
 *
 * gft_transmittance_check: input and output of gft_transmittance
 * [N, D, H, W, 1]; every column_stride-th (n, h, w) column recomputed as
 * exp(-sum) in double. */
gft_status gft_transmittance_check(const float* input, const float* output, const int64_t shape[5],
                                   int32_t column_stride, double* result, void* stream);
/* gft_raymarch_check: the density (last) channel of a BEER_LAMBERT (C > 1:
 * d = max(d + s, 0); C == 1: a sum), LINEAR, BORDER raymarch
 * (gft_raymarch_grid_transform with separate camera batches) recomputed in
 * double -- camera inverses, sample positions near + i*step, trilinear
 * weights and the sum -- for every ray_stride-th pixel of every (batch,
 * camera) pair, against output [N, V, H, W, C].  input_dtype may carry
 * GFT_LAYOUT_BRICK. */
gft_status gft_raymarch_check(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                              const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
                              const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
                              const float* output, int32_t ray_stride, double* result, void* stream);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif
#endif /* GFT_H */
