// extern "C" entry points of libgft.so (declared in include/gft.h): argument
// checks with the reference ops' error classes, camera set-up and dispatch to
// the launchers.  No entry point allocates device memory or synchronises.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <string>
#include <vector>

#include "../../include/gft.h"
#include "gft_internal.h"

namespace gft {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

static std::atomic<unsigned long long> g_launches{0};

// launch-configuration knobs, defaults as documented in gft.h
static std::atomic<int> g_knobs[GFT_KNOB_COUNT] = {{0}, {256}, {256}, {8}, {0}, {0}};
int knob_value(int k) { return (k >= 0 && k < GFT_KNOB_COUNT) ? g_knobs[k].load(std::memory_order_relaxed) : 0; }
int sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return std::max(sms, 1);
}
unsigned raymarch_blocks(int tiles) {
    const int k = knob_value(GFT_KNOB_RAYMARCH_BLOCKS_PER_SM);
    if (k <= 0) return (unsigned)std::max(tiles, 1);
    return (unsigned)std::max(1, std::min(tiles, k * sm_count()));
}
unsigned weights_blocks(int tiles) {
    const int k = knob_value(GFT_KNOB_WEIGHTS_BLOCKS_PER_SM);
    if (k <= 0) return raymarch_blocks(tiles);
    return (unsigned)std::max(1, std::min(tiles, k * sm_count()));
}

bool launched(int n, const char* what) {
    g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed);
    return cuda_ok(cudaGetLastError(), what);
}

// column-major 16 floats -> row-major double 4x4 (the column-vector matrix)
static void mat_from_flat(const float* m16, double a[4][4]) {
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) a[r][c] = (double)m16[c * 4 + r];
}
static void matmul4(const double a[4][4], const double b[4][4], double o[4][4]) {
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += a[r][k] * b[k][c];
            o[r][c] = s;
        }
}
// Gauss-Jordan with partial pivoting; a singular matrix yields non-finite entries.
static void inverse4(const double a_in[4][4], double inv[4][4]) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 8; ++c) a[r][c] = c < 4 ? a_in[r][c] : (c - 4 == r ? 1.0 : 0.0);
    for (int col = 0; col < 4; ++col) {
        int piv = col;
        for (int r = col + 1; r < 4; ++r)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (piv != col)
            for (int c = 0; c < 8; ++c) std::swap(a[piv][c], a[col][c]);
        const double d = a[col][col];
        for (int c = 0; c < 8; ++c) a[col][c] /= d;
        for (int r = 0; r < 4; ++r) {
            if (r == col) continue;
            const double f = a[r][col];
            for (int c = 0; c < 8; ++c) a[r][c] -= f * a[col][c];
        }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) inv[r][c] = a[r][c + 4];
}
static Mat4 to_mat4(const double a[4][4]) {
    Mat4 m;
    m.r0 = make_float4((float)a[0][0], (float)a[0][1], (float)a[0][2], (float)a[0][3]);
    m.r1 = make_float4((float)a[1][0], (float)a[1][1], (float)a[1][2], (float)a[1][3]);
    m.r2 = make_float4((float)a[2][0], (float)a[2][1], (float)a[2][2], (float)a[2][3]);
    m.r3 = make_float4((float)a[3][0], (float)a[3][1], (float)a[3][2], (float)a[3][3]);
    return m;
}

static CamX make_cam(const float* M, const float* V, const float* P, const float* F) {
    double m[4][4], v[4][4], p[4][4], mv[4][4], mvi[4][4], pi[4][4], q[4][4], r[4][4];
    mat_from_flat(M, m);
    mat_from_flat(V, v);
    mat_from_flat(P, p);
    matmul4(v, m, mv);
    inverse4(mv, mvi);
    inverse4(p, pi);
    // q: rows 0-2 of MV^-1 P^-1 and row 3 of P^-1 (NDC -> OS, see CamX); r = P MV
    matmul4(mvi, pi, q);
    for (int j = 0; j < 4; ++j) q[3][j] = pi[3][j];
    matmul4(p, mv, r);
    CamX c;
    c.mv = to_mat4(mv);
    c.mv_inv = to_mat4(mvi);
    c.p = to_mat4(p);
    c.p_inv = to_mat4(pi);
    c.q = to_mat4(q);
    c.r = to_mat4(r);
    c.near_ = F[0];
    c.far_ = F[1];
    c.p22 = (float)p[2][2];
    c.p23 = (float)p[2][3];
    return c;
}

std::vector<Pair> make_pairs(const float* M, int num_m, const float* V, const float* P, const float* F,
                             int num_cameras, int batch, bool separate) {
    static const float eye[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    std::vector<Pair> out;
    const int nv = separate ? num_cameras : 1;
    for (int b = 0; b < batch; ++b) {
        const float* mb = (M == nullptr) ? eye : M + 16 * (num_m == 1 ? 0 : b);
        for (int vi = 0; vi < nv; ++vi) {
            const int c = separate ? vi : b;
            Pair p;
            p.cam = make_cam(mb, V + 16 * c, P + 16 * c, F + 6 * c);
            p.in_batch = b;
            p.out_slot = b * nv + vi;
            p.camera = c;
            out.push_back(p);
        }
    }
    return out;
}

std::vector<PairTable> make_tables(const std::vector<Pair>& pairs) {
    std::vector<PairTable> out;
    for (size_t i = 0; i < pairs.size(); i += MAX_PAIRS) {
        PairTable t;
        std::memset(&t, 0, sizeof(t));
        t.pair_base = (int)i;
        t.n = (int)std::min<size_t>(MAX_PAIRS, pairs.size() - i);
        for (int k = 0; k < t.n; ++k) {
            t.cam[k] = pairs[i + k].cam;
            t.in_batch[k] = pairs[i + k].in_batch;
            t.out_slot[k] = pairs[i + k].out_slot;
            t.rw[k] = pairs[i + k].W;
            t.rh[k] = pairs[i + k].H;
            t.rd[k] = pairs[i + k].D;
            t.pix0[k] = pairs[i + k].pix0;
        }
        out.push_back(t);
    }
    return out;
}

}  // namespace gft

using namespace gft;

namespace {

gft_status fail(gft_status s, const std::string& msg) {
    set_error(msg);
    return s;
}

bool grid_shape_ok(const int64_t* s, std::string& why) {
    if (s == nullptr) {
        why = "shape pointer is NULL";
        return false;
    }
    for (int i = 0; i < 5; ++i)
        if (s[i] <= 0) {
            why = "Invalid input shape (NDHWC): all dimensions must be positive";
            return false;
        }
    if (s[1] > INT32_MAX || s[2] > INT32_MAX || s[3] > INT32_MAX) {
        why = "grid dimension too large";
        return false;
    }
    return true;
}

bool channels_ok(int64_t c) { return c == 1 || c == 2 || c == 4; }

// The raymarch kernels index a grid slice (rows or bricks) with 32-bit cell
// arithmetic, as the resampling and advection kernels do.
bool raymarch_grid_ok(const int64_t* s, std::string& why) {
    if (!grid_shape_ok(s, why)) return false;
    if (brick_cells(Dims{(int)s[3], (int)s[2], (int)s[1]}) >= MAX_SLICE_CELLS) {
        why = "a grid slice has 2^32 or more cells";
        return false;
    }
    return true;
}

Dims dims_of(const int64_t* s) { return Dims{(int)s[3], (int)s[2], (int)s[1]}; }

gft_status check_cameras(const float* M, int num_m, int64_t batch, const float* V, const float* P, const float* F,
                         int num_cameras, int separate) {
    if (V == nullptr || P == nullptr || F == nullptr) return fail(GFT_ERR_INVALID_ARGUMENT, "camera arrays must not be NULL");
    if (num_cameras <= 0) return fail(GFT_ERR_INVALID_ARGUMENT, "camera batch size mismatch");
    if (M == nullptr || num_m != batch) return fail(GFT_ERR_INVALID_ARGUMENT, "model matrix batch size mismatch");
    if (!separate && num_cameras != batch)
        return fail(GFT_ERR_INVALID_ARGUMENT, "camera batch must match data batch when not using global sampling.");
    return GFT_OK;
}

bool enum_in(int v, int lo, int hi) { return v >= lo && v <= hi; }

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Vector accesses need aligned device pointers: a tensor of C channels is
// read and written C elements at a time (16 bytes for C == 4 fp32, 8 for
// C == 4 bf16), the RGB-plus-density images and lookup tables as float4, and
// workspaces and sample stores hold float4 / float2 regions.  cudaMalloc and
// the torch allocator return 256-byte aligned buffers; a misaligned pointer
// is an argument error here instead of a misaligned access in a kernel.
size_t vec_bytes(int64_t C, int32_t dtype) { return (size_t)C * (dtype == GFT_DTYPE_BF16 ? 2 : 4); }

gft_status check_aligned(std::initializer_list<const void*> ptrs, size_t a) {
    for (const void* p : ptrs)
        if (reinterpret_cast<uintptr_t>(p) % a != 0)
            return fail(GFT_ERR_INVALID_ARGUMENT,
                        "device pointer not aligned to its " + std::to_string(a) + "-byte channel vector");
    return GFT_OK;
}

gft_status check_workspace_aligned(const void* ws) {
    if (reinterpret_cast<uintptr_t>(ws) % 16 != 0)
        return fail(GFT_ERR_WORKSPACE, "workspace or sample store not 16-byte aligned");
    return GFT_OK;
}

// Raymarch pairs of one image size: pair k writes output slot out_slot.
void set_uniform_images(std::vector<Pair>& pairs, int D, int H, int W) {
    for (Pair& p : pairs) {
        p.W = W;
        p.H = H;
        p.D = D;
        p.pix0 = (int64_t)p.out_slot * H * W;
    }
}

}  // namespace

extern "C" {

const char* gft_last_error(void) { return g_last_error.c_str(); }

const char* gft_version(void) { return "gft-gb300 0.1 (sm_103a)"; }

unsigned long long gft_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

gft_status gft_set_knob(int32_t knob, int32_t value) {
    bool ok = false;
    switch (knob) {
        case GFT_KNOB_RAYMARCH_BLOCKS_PER_SM:
        case GFT_KNOB_WEIGHTS_BLOCKS_PER_SM: ok = value >= 0 && value <= 32; break;
        case GFT_KNOB_ADVECT_THREADS:
        case GFT_KNOB_RESAMPLE_THREADS: ok = value == 64 || value == 128 || value == 256; break;
        case GFT_KNOB_SCAN_SEGMENTS: ok = value == 4 || value == 8 || value == 16; break;
        case GFT_KNOB_WEIGHTS_PIPELINE: ok = value == 0 || value == 1; break;
        default: return fail(GFT_ERR_INVALID_ARGUMENT, "unknown knob");
    }
    if (!ok) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid knob value");
    // the side stream is made now, outside any stream capture, where a device
    // is present (else at the first gradient call that uses it)
    if (knob == GFT_KNOB_WEIGHTS_PIPELINE && value == 1 && !prepare_side_stream()) (void)cudaGetLastError();
    g_knobs[knob].store(value, std::memory_order_relaxed);
    return GFT_OK;
}

int32_t gft_get_knob(int32_t knob) { return knob_value(knob); }

// ---------------------------------------------------------------- raymarch
static gft_status raymarch_fwd_impl(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                                    const float* matrix_m, int32_t num_m, const float* matrix_v,
                                    const float* matrix_p, const float* frustum, int32_t num_cameras,
                                    const int32_t output_shape[3], int32_t interpolation, int32_t boundary,
                                    int32_t blending_mode, int32_t separate_camera_batch, float* output,
                                    float* samples, size_t samples_bytes, void* stream);

gft_status gft_raymarch_grid_transform(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                                       const float* matrix_m, int32_t num_m, const float* matrix_v,
                                       const float* matrix_p, const float* frustum, int32_t num_cameras,
                                       const int32_t output_shape[3], int32_t interpolation, int32_t boundary,
                                       int32_t blending_mode, int32_t separate_camera_batch, float* output,
                                       void* stream) {
    return raymarch_fwd_impl(input, input_dtype, input_shape, matrix_m, num_m, matrix_v, matrix_p, frustum,
                             num_cameras, output_shape, interpolation, boundary, blending_mode,
                             separate_camera_batch, output, nullptr, 0, stream);
}

gft_status gft_raymarch_grid_transform_store(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                                             const float* matrix_m, int32_t num_m, const float* matrix_v,
                                             const float* matrix_p, const float* frustum, int32_t num_cameras,
                                             const int32_t output_shape[3], int32_t interpolation, int32_t boundary,
                                             int32_t blending_mode, int32_t separate_camera_batch, float* output,
                                             float* samples, size_t samples_bytes, void* stream) {
    if (interpolation != GFT_FILTER_LINEAR)
        return fail(GFT_ERR_INVALID_ARGUMENT, "the sample store supports LINEAR interpolation only");
    if (samples == nullptr) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    return raymarch_fwd_impl(input, input_dtype, input_shape, matrix_m, num_m, matrix_v, matrix_p, frustum,
                             num_cameras, output_shape, interpolation, boundary, blending_mode,
                             separate_camera_batch, output, samples, samples_bytes, stream);
}

size_t gft_raymarch_grid_transform_samples_size(const int64_t input_shape[5], int32_t num_cameras,
                                                const int32_t output_shape[3], int32_t separate_camera_batch) {
    std::string why;
    if (!grid_shape_ok(input_shape, why) || !channels_ok(input_shape[4]) || output_shape == nullptr ||
        output_shape[0] < 1 || output_shape[1] < 1 || output_shape[2] < 1 || num_cameras < 1)
        return 0;
    std::vector<Pair> pairs((size_t)input_shape[0] * (separate_camera_batch ? (size_t)num_cameras : 1));
    set_uniform_images(pairs, output_shape[0], output_shape[1], output_shape[2]);
    return align256(raymarch_store_bytes(pairs, (int)input_shape[4], (int)input_shape[0], dims_of(input_shape)));
}

size_t gft_raymarch_grid_transform_samples_min_size(const int64_t input_shape[5], int32_t num_cameras,
                                                    const int32_t output_shape[3], int32_t separate_camera_batch) {
    std::string why;
    if (!grid_shape_ok(input_shape, why) || !channels_ok(input_shape[4]) || output_shape == nullptr ||
        output_shape[0] < 1 || output_shape[1] < 1 || output_shape[2] < 1 || num_cameras < 1)
        return 0;
    std::vector<Pair> pairs((size_t)input_shape[0] * (separate_camera_batch ? (size_t)num_cameras : 1));
    set_uniform_images(pairs, output_shape[0], output_shape[1], output_shape[2]);
    return align256(raymarch_store_min_bytes(pairs, (int)input_shape[0], dims_of(input_shape)));
}

static gft_status raymarch_fwd_impl(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                                    const float* matrix_m, int32_t num_m, const float* matrix_v,
                                    const float* matrix_p, const float* frustum, int32_t num_cameras,
                                    const int32_t output_shape[3], int32_t interpolation, int32_t boundary,
                                    int32_t blending_mode, int32_t separate_camera_batch, float* output,
                                    float* samples, size_t samples_bytes, void* stream) {
    std::string why;
    if (!raymarch_grid_ok(input_shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!channels_ok(input_shape[4])) return fail(GFT_ERR_UNIMPLEMENTED, "Only 1,2 and 4 Channel supported.");
    if (output_shape == nullptr || output_shape[0] < 1 || output_shape[1] < 1 || output_shape[2] < 1)
        return fail(GFT_ERR_INVALID_ARGUMENT, "All shape dimensions must be positive (output_shape)");
    if (!enum_in(interpolation, 0, 3)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid filter mode");
    if (!enum_in(boundary, 0, 2)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid boundary mode");
    if (!enum_in(blending_mode, 0, 4) || blending_mode == GFT_BLEND_BEER_LAMBERT_EXCLUSIVE)
        return fail(GFT_ERR_INVALID_ARGUMENT, "invalid blend mode");
    const int layout = (input_dtype & GFT_LAYOUT_BRICK) ? LAYOUT_BRICK : LAYOUT_FLAT;
    input_dtype &= ~GFT_LAYOUT_BRICK;
    if (!enum_in(input_dtype, 0, 1)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid input dtype");
    if (layout == LAYOUT_BRICK && interpolation != GFT_FILTER_LINEAR)
        return fail(GFT_ERR_INVALID_ARGUMENT, "the brick layout supports LINEAR interpolation only");
    gft_status st = check_cameras(matrix_m, num_m, input_shape[0], matrix_v, matrix_p, frustum, num_cameras,
                                  separate_camera_batch);
    if (st != GFT_OK) return st;
    if (input == nullptr || output == nullptr) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    RaymarchArgs a;
    a.input = input;
    a.dtype = input_dtype;
    a.layout = layout;
    a.N = (int)input_shape[0];
    a.C = (int)input_shape[4];
    a.din = dims_of(input_shape);
    a.D = output_shape[0];
    a.H = output_shape[1];
    a.W = output_shape[2];
    a.filter = interpolation;
    a.boundary = boundary;
    a.blend = blending_mode;
    auto pairs = make_pairs(matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras, a.N,
                            separate_camera_batch != 0);
    set_uniform_images(pairs, a.D, a.H, a.W);
    a.n_slots = (int)pairs.size();
    if (samples != nullptr) {
        if (samples_bytes < raymarch_store_min_bytes(pairs, a.N, a.din))
            return fail(GFT_ERR_WORKSPACE, "raymarch sample store too small");
    }
    if ((st = check_aligned({input}, vec_bytes(a.C, input_dtype))) != GFT_OK ||
        (st = check_aligned({output}, vec_bytes(a.C, 0))) != GFT_OK || (st = check_workspace_aligned(samples)) != GFT_OK)
        return st;
    if (samples != nullptr) {
        a.store = raymarch_store_layout(samples, samples_bytes, pairs, a.C, a.N, a.din);
        if (!launch_raymarch_occupancy(a, as_stream(stream))) return GFT_ERR_CUDA;
    }
    if (!launch_raymarch_fwd(a, pairs, output, as_stream(stream))) return GFT_ERR_CUDA;
    return GFT_OK;
}

// Raymarch gradient workspace for `pairs` (batch, camera) pairs: the
// per-pair reciprocal weight sums of the reference normalisation, plus the
// integer accumulators of the deterministic adjoint.
static size_t raymarch_grad_ws(const int64_t* input_shape, size_t pairs, int32_t grad_mode) {
    const bool det = (grad_mode & GFT_GRAD_DETERMINISTIC) != 0;
    grad_mode &= ~(GFT_GRAD_WEIGHTS_READY | GFT_GRAD_DETERMINISTIC | GFT_GRAD_CAMERA_SUMS);
    if (det) return raymarch_det_bytes((int)input_shape[0], (int)input_shape[4], dims_of(input_shape), pairs);
    if (grad_mode == GFT_GRAD_EXACT) return 0;
    return align256(sizeof(float) * (size_t)brick_cells(dims_of(input_shape)) * pairs);
}

size_t gft_raymarch_grid_transform_grad_workspace_size(const int64_t input_shape[5], int32_t num_cameras,
                                                       int32_t separate_camera_batch, int32_t grad_mode) {
    std::string why;
    if (!grid_shape_ok(input_shape, why)) return 0;
    const size_t pairs = (size_t)input_shape[0] * (separate_camera_batch ? (size_t)std::max(num_cameras, 1) : 1);
    return raymarch_grad_ws(input_shape, pairs, grad_mode);
}

// The deterministic adjoint's bound holds for these blend modes.
static bool det_blend_ok(int blend, int64_t C) {
    return C == 1 || blend == GFT_BLEND_BEER_LAMBERT || blend == GFT_BLEND_ADDITIVE;
}

static gft_status raymarch_grad_impl(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                                     const float* output, const float* output_grad, const float* matrix_m,
                                     int32_t num_m, const float* matrix_v, const float* matrix_p,
                                     const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
                                     int32_t interpolation, int32_t boundary, int32_t blending_mode,
                                     int32_t separate_camera_batch, int32_t grad_mode, const float* samples,
                                     size_t samples_bytes, float* input_grad, void* workspace,
                                     size_t workspace_bytes, void* stream, const float* projection = nullptr);

gft_status gft_raymarch_grid_transform_grad(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                                            const float* output, const float* output_grad, const float* matrix_m,
                                            int32_t num_m, const float* matrix_v, const float* matrix_p,
                                            const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
                                            int32_t interpolation, int32_t boundary, int32_t blending_mode,
                                            int32_t separate_camera_batch, int32_t grad_mode, float* input_grad,
                                            void* workspace, size_t workspace_bytes, void* stream) {
    return raymarch_grad_impl(input, input_dtype, input_shape, output, output_grad, matrix_m, num_m, matrix_v,
                              matrix_p, frustum, num_cameras, output_shape, interpolation, boundary, blending_mode,
                              separate_camera_batch, grad_mode, nullptr, 0, input_grad, workspace, workspace_bytes,
                              stream);
}

gft_status gft_raymarch_grid_transform_grad_stored(
    const void* input, int32_t input_dtype, const int64_t input_shape[5], const float* output,
    const float* output_grad, const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t output_shape[3], int32_t interpolation,
    int32_t boundary, int32_t blending_mode, int32_t separate_camera_batch, int32_t grad_mode, const float* samples,
    size_t samples_bytes, float* input_grad, void* workspace, size_t workspace_bytes, void* stream) {
    if (samples == nullptr) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    return raymarch_grad_impl(input, input_dtype, input_shape, output, output_grad, matrix_m, num_m, matrix_v,
                              matrix_p, frustum, num_cameras, output_shape, interpolation, boundary, blending_mode,
                              separate_camera_batch, grad_mode, samples, samples_bytes, input_grad, workspace,
                              workspace_bytes, stream);
}

gft_status gft_raymarch_grid_transform_grad_projected(
    const void* input, int32_t input_dtype, const int64_t input_shape[5], const float* output,
    const float* output_grad, const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
    const float* frustum, int32_t num_cameras, const int32_t output_shape[3], int32_t interpolation,
    int32_t boundary, int32_t blending_mode, int32_t separate_camera_batch, int32_t grad_mode, const float* samples,
    size_t samples_bytes, const float projection[8], float* input_grad, void* workspace, size_t workspace_bytes,
    void* stream) {
    if (projection == nullptr) return fail(GFT_ERR_INVALID_ARGUMENT, "projection is NULL");
    return raymarch_grad_impl(input, input_dtype, input_shape, output, output_grad, matrix_m, num_m, matrix_v,
                              matrix_p, frustum, num_cameras, output_shape, interpolation, boundary, blending_mode,
                              separate_camera_batch, grad_mode, samples, samples_bytes, input_grad, workspace,
                              workspace_bytes, stream, projection);
}

static gft_status raymarch_grad_impl(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                                     const float* output, const float* output_grad, const float* matrix_m,
                                     int32_t num_m, const float* matrix_v, const float* matrix_p,
                                     const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
                                     int32_t interpolation, int32_t boundary, int32_t blending_mode,
                                     int32_t separate_camera_batch, int32_t grad_mode, const float* samples,
                                     size_t samples_bytes, float* input_grad, void* workspace,
                                     size_t workspace_bytes, void* stream, const float* projection) {
    std::string why;
    if (!raymarch_grid_ok(input_shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!channels_ok(input_shape[4])) return fail(GFT_ERR_UNIMPLEMENTED, "Only 1,2 and 4 Channel supported.");
    if (output_shape == nullptr || output_shape[0] < 1 || output_shape[1] < 1 || output_shape[2] < 1)
        return fail(GFT_ERR_INVALID_ARGUMENT, "All shape dimensions must be positive (output_shape)");
    if (interpolation != GFT_FILTER_LINEAR)
        return fail(GFT_ERR_INVALID_ARGUMENT, "gradient supports LINEAR interpolation only");
    if (!enum_in(boundary, 0, 2)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid boundary mode");
    if (!enum_in(blending_mode, 0, 4) || blending_mode == GFT_BLEND_BEER_LAMBERT_EXCLUSIVE)
        return fail(GFT_ERR_INVALID_ARGUMENT, "invalid blend mode");
    const bool weights_ready = (grad_mode & GFT_GRAD_WEIGHTS_READY) != 0;
    const bool det = (grad_mode & GFT_GRAD_DETERMINISTIC) != 0;
    const bool camera_sums = (grad_mode & GFT_GRAD_CAMERA_SUMS) != 0;
    const int32_t ws_mode = grad_mode;
    grad_mode &= ~(GFT_GRAD_WEIGHTS_READY | GFT_GRAD_DETERMINISTIC | GFT_GRAD_CAMERA_SUMS);
    const int layout = (input_dtype & GFT_LAYOUT_BRICK) ? LAYOUT_BRICK : LAYOUT_FLAT;
    input_dtype &= ~GFT_LAYOUT_BRICK;
    if (!enum_in(grad_mode, 0, 1) || !enum_in(input_dtype, 0, 1)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid enum");
    if (weights_ready && grad_mode != GFT_GRAD_REFERENCE)
        return fail(GFT_ERR_INVALID_ARGUMENT, "GFT_GRAD_WEIGHTS_READY needs GFT_GRAD_REFERENCE");
    if (det && !det_blend_ok(blending_mode, input_shape[4]))
        return fail(GFT_ERR_UNIMPLEMENTED, "deterministic gradient: BEER_LAMBERT or ADDITIVE blending only");
    if (projection != nullptr) {
        if (input_shape[4] != 4) return fail(GFT_ERR_INVALID_ARGUMENT, "projected gradient: 4 channels only");
        if (layout != LAYOUT_BRICK) return fail(GFT_ERR_INVALID_ARGUMENT, "projected gradient: brick layout only");
    }
    if (camera_sums && (projection == nullptr || grad_mode != GFT_GRAD_REFERENCE || weights_ready || det))
        return fail(GFT_ERR_INVALID_ARGUMENT,
                    "GFT_GRAD_CAMERA_SUMS: projected GFT_GRAD_REFERENCE gradient without GFT_GRAD_WEIGHTS_READY "
                    "or GFT_GRAD_DETERMINISTIC");
    gft_status st = check_cameras(matrix_m, num_m, input_shape[0], matrix_v, matrix_p, frustum, num_cameras,
                                  separate_camera_batch);
    if (st != GFT_OK) return st;
    if (!input || !output || !output_grad || !input_grad) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    const size_t need = gft_raymarch_grid_transform_grad_workspace_size(input_shape, num_cameras,
                                                                        separate_camera_batch, ws_mode);
    if (need > 0 && (workspace == nullptr || workspace_bytes < need))
        return fail(GFT_ERR_WORKSPACE, "raymarch gradient workspace too small");
    RaymarchArgs a;
    a.input = input;
    a.dtype = input_dtype;
    a.layout = layout;
    a.N = (int)input_shape[0];
    a.C = (int)input_shape[4];
    a.din = dims_of(input_shape);
    a.D = output_shape[0];
    a.H = output_shape[1];
    a.W = output_shape[2];
    a.filter = interpolation;
    a.boundary = boundary;
    a.blend = blending_mode;
    auto pairs = make_pairs(matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras, a.N,
                            separate_camera_batch != 0);
    set_uniform_images(pairs, a.D, a.H, a.W);
    a.n_slots = (int)pairs.size();
    a.det = det;
    if (samples != nullptr) {
        if (samples_bytes < raymarch_store_min_bytes(pairs, a.N, a.din))
            return fail(GFT_ERR_WORKSPACE, "raymarch sample store too small");
        a.store = raymarch_store_layout(const_cast<float*>(samples), samples_bytes, pairs, a.C, a.N, a.din);
    }
    a.camera_sums = camera_sums;
    if (projection != nullptr) {
        a.project = true;
        for (int c = 0; c < 4; ++c) {
            a.proj.a[c] = projection[c];
            a.proj.b[c] = projection[4 + c];
        }
    }
    if ((st = check_aligned({input}, vec_bytes(a.C, input_dtype))) != GFT_OK ||
        (st = check_aligned({output, output_grad}, vec_bytes(a.C, 0))) != GFT_OK ||
        (st = check_aligned({input_grad}, vec_bytes(a.project ? 2 : a.C, 0))) != GFT_OK ||
        (st = check_workspace_aligned(samples)) != GFT_OK || (st = check_workspace_aligned(workspace)) != GFT_OK)
        return st;
    float* cnt = need > 0 ? reinterpret_cast<float*>(workspace) : nullptr;
    if (!launch_raymarch_bwd(a, pairs, output, output_grad, grad_mode == GFT_GRAD_EXACT, weights_ready, input_grad,
                             cnt, as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

static gft_status raymarch_weights_impl_abi(const int64_t input_shape[5], const float* matrix_m, int32_t num_m,
                                            const float* matrix_v, const float* matrix_p, const float* frustum,
                                            int32_t num_cameras, const int32_t output_shape[3], int32_t boundary,
                                            int32_t separate_camera_batch, int32_t grad_mode, void* workspace,
                                            size_t workspace_bytes, void* stream);

gft_status gft_raymarch_grid_transform_grad_weights(const int64_t input_shape[5], const float* matrix_m,
                                                    int32_t num_m, const float* matrix_v, const float* matrix_p,
                                                    const float* frustum, int32_t num_cameras,
                                                    const int32_t output_shape[3], int32_t boundary,
                                                    int32_t separate_camera_batch, void* workspace,
                                                    size_t workspace_bytes, void* stream) {
    return raymarch_weights_impl_abi(input_shape, matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras,
                                     output_shape, boundary, separate_camera_batch, GFT_GRAD_REFERENCE, workspace,
                                     workspace_bytes, stream);
}

gft_status gft_raymarch_grid_transform_grad_weights_mode(const int64_t input_shape[5], const float* matrix_m,
                                                         int32_t num_m, const float* matrix_v,
                                                         const float* matrix_p, const float* frustum,
                                                         int32_t num_cameras, const int32_t output_shape[3],
                                                         int32_t boundary, int32_t separate_camera_batch,
                                                         int32_t grad_mode, void* workspace, size_t workspace_bytes,
                                                         void* stream) {
    return raymarch_weights_impl_abi(input_shape, matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras,
                                     output_shape, boundary, separate_camera_batch, grad_mode, workspace,
                                     workspace_bytes, stream);
}

static gft_status raymarch_weights_impl_abi(const int64_t input_shape[5], const float* matrix_m, int32_t num_m,
                                            const float* matrix_v, const float* matrix_p, const float* frustum,
                                            int32_t num_cameras, const int32_t output_shape[3], int32_t boundary,
                                            int32_t separate_camera_batch, int32_t grad_mode, void* workspace,
                                            size_t workspace_bytes, void* stream) {
    const bool det = (grad_mode & GFT_GRAD_DETERMINISTIC) != 0;
    if ((grad_mode & ~GFT_GRAD_DETERMINISTIC) != GFT_GRAD_REFERENCE)
        return fail(GFT_ERR_INVALID_ARGUMENT, "weight sums: GFT_GRAD_REFERENCE (| GFT_GRAD_DETERMINISTIC) only");
    std::string why;
    if (!raymarch_grid_ok(input_shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (output_shape == nullptr || output_shape[0] < 1 || output_shape[1] < 1 || output_shape[2] < 1)
        return fail(GFT_ERR_INVALID_ARGUMENT, "All shape dimensions must be positive (output_shape)");
    if (!enum_in(boundary, 0, 2)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid boundary mode");
    gft_status st = check_cameras(matrix_m, num_m, input_shape[0], matrix_v, matrix_p, frustum, num_cameras,
                                  separate_camera_batch);
    if (st != GFT_OK) return st;
    const size_t need = gft_raymarch_grid_transform_grad_workspace_size(input_shape, num_cameras,
                                                                        separate_camera_batch, grad_mode);
    if (workspace == nullptr || workspace_bytes < need)
        return fail(GFT_ERR_WORKSPACE, "raymarch gradient workspace too small");
    if ((st = check_workspace_aligned(workspace)) != GFT_OK) return st;
    RaymarchArgs a{};
    a.N = (int)input_shape[0];
    a.C = (int)input_shape[4];
    a.din = dims_of(input_shape);
    a.D = output_shape[0];
    a.H = output_shape[1];
    a.W = output_shape[2];
    a.filter = GFT_FILTER_LINEAR;
    a.boundary = boundary;
    auto pairs = make_pairs(matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras, a.N,
                            separate_camera_batch != 0);
    set_uniform_images(pairs, a.D, a.H, a.W);
    a.n_slots = (int)pairs.size();
    const bool ok = det ? launch_raymarch_weights_det(a, pairs, reinterpret_cast<float*>(workspace), as_stream(stream))
                        : launch_raymarch_weights(a, pairs, reinterpret_cast<float*>(workspace), as_stream(stream));
    return ok ? GFT_OK : GFT_ERR_CUDA;
}

// ---------------------------------------------------------------- raymarch, cameras of different image sizes
static bool multi_shapes_ok(const int32_t* shapes, int32_t num_cameras, std::string& why) {
    if (shapes == nullptr || num_cameras <= 0) {
        why = "output_shapes must hold num_cameras x 3 positive sizes";
        return false;
    }
    for (int c = 0; c < 3 * num_cameras; ++c)
        if (shapes[c] < 1) {
            why = "All shape dimensions must be positive (output_shapes)";
            return false;
        }
    return true;
}

// Every (batch, camera) pair with its own image; the output of batch slice n
// holds the cameras' images one after another.
// camera_batch == nullptr: every (batch, camera) pair, the output of batch
// slice n holding the cameras' images one after another.  Otherwise one pair
// per camera c, rendering batch slice camera_batch[c], the output holding the
// cameras' images one after another.
static std::vector<Pair> multi_pairs(const float* M, int num_m, const float* V, const float* P, const float* F,
                                     int num_cameras, int batch, const int32_t* shapes,
                                     const int32_t* camera_batch = nullptr) {
    std::vector<Pair> pairs;
    if (camera_batch == nullptr) {
        pairs = make_pairs(M, num_m, V, P, F, num_cameras, batch, true);
    } else {
        for (int c = 0; c < num_cameras; ++c) {
            const int b = camera_batch[c];
            Pair p;
            p.cam = make_cam(M + 16 * (num_m == 1 ? 0 : b), V + 16 * c, P + 16 * c, F + 6 * c);
            p.in_batch = b;
            p.out_slot = c;
            p.camera = c;
            pairs.push_back(p);
        }
    }
    int64_t per_batch = 0;
    for (int c = 0; c < num_cameras; ++c) per_batch += (int64_t)shapes[3 * c + 1] * shapes[3 * c + 2];
    for (Pair& p : pairs) {
        int64_t off = 0;
        for (int c = 0; c < p.camera; ++c) off += (int64_t)shapes[3 * c + 1] * shapes[3 * c + 2];
        p.D = shapes[3 * p.camera];
        p.H = shapes[3 * p.camera + 1];
        p.W = shapes[3 * p.camera + 2];
        p.pix0 = (camera_batch == nullptr ? (int64_t)p.in_batch * per_batch : 0) + off;
    }
    return pairs;
}

static bool camera_batch_ok(const int32_t* camera_batch, int num_cameras, int64_t batch, std::string& why) {
    if (camera_batch == nullptr) {
        why = "camera_batch is NULL";
        return false;
    }
    for (int c = 0; c < num_cameras; ++c)
        if (camera_batch[c] < 0 || camera_batch[c] >= batch) {
            why = "camera_batch entries must lie in [0, batch)";
            return false;
        }
    return true;
}

static gft_status multi_fwd_impl(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                                 const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
                                 const float* frustum, int32_t num_cameras, const int32_t* camera_batch,
                                 const int32_t* output_shapes, int32_t interpolation, int32_t boundary,
                                 int32_t blending_mode, float* output, void* stream) {
    std::string why;
    if (!raymarch_grid_ok(input_shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!channels_ok(input_shape[4])) return fail(GFT_ERR_UNIMPLEMENTED, "Only 1,2 and 4 Channel supported.");
    if (!multi_shapes_ok(output_shapes, num_cameras, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!enum_in(interpolation, 0, 3) || !enum_in(boundary, 0, 2) || !enum_in(blending_mode, 0, 4) ||
        !enum_in(input_dtype, 0, 1))
        return fail(GFT_ERR_INVALID_ARGUMENT, "invalid enum");
    gft_status st = check_cameras(matrix_m, num_m, input_shape[0], matrix_v, matrix_p, frustum, num_cameras, 1);
    if (st != GFT_OK) return st;
    if (camera_batch != nullptr && !camera_batch_ok(camera_batch, num_cameras, input_shape[0], why))
        return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!input || !output) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    RaymarchArgs a{};
    a.input = input;
    a.dtype = input_dtype;
    a.N = (int)input_shape[0];
    a.C = (int)input_shape[4];
    a.din = dims_of(input_shape);
    a.filter = interpolation;
    a.boundary = boundary;
    a.blend = blending_mode;
    const auto pairs = multi_pairs(matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras, a.N, output_shapes,
                                   camera_batch);
    a.n_slots = (int)pairs.size();
    if ((st = check_aligned({input}, vec_bytes(a.C, input_dtype))) != GFT_OK ||
        (st = check_aligned({output}, vec_bytes(a.C, 0))) != GFT_OK)
        return st;
    if (!launch_raymarch_fwd(a, pairs, output, as_stream(stream))) return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_raymarch_grid_transform_multi(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                                             const float* matrix_m, int32_t num_m, const float* matrix_v,
                                             const float* matrix_p, const float* frustum, int32_t num_cameras,
                                             const int32_t* output_shapes, int32_t interpolation, int32_t boundary,
                                             int32_t blending_mode, float* output, void* stream) {
    return multi_fwd_impl(input, input_dtype, input_shape, matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras,
                          nullptr, output_shapes, interpolation, boundary, blending_mode, output, stream);
}

gft_status gft_raymarch_grid_transform_views(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                                             const float* matrix_m, int32_t num_m, const float* matrix_v,
                                             const float* matrix_p, const float* frustum, int32_t num_cameras,
                                             const int32_t* camera_batch, const int32_t* output_shapes,
                                             int32_t interpolation, int32_t boundary, int32_t blending_mode,
                                             float* output, void* stream) {
    if (camera_batch == nullptr) return fail(GFT_ERR_INVALID_ARGUMENT, "camera_batch is NULL");
    return multi_fwd_impl(input, input_dtype, input_shape, matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras,
                          camera_batch, output_shapes, interpolation, boundary, blending_mode, output, stream);
}

size_t gft_raymarch_grid_transform_views_grad_workspace_size(const int64_t input_shape[5], int32_t num_cameras,
                                                             int32_t grad_mode) {
    std::string why;
    if (!grid_shape_ok(input_shape, why)) return 0;
    return raymarch_grad_ws(input_shape, (size_t)std::max(num_cameras, 1), grad_mode);
}

size_t gft_raymarch_grid_transform_multi_grad_workspace_size(const int64_t input_shape[5], int32_t num_cameras,
                                                             int32_t grad_mode) {
    return gft_raymarch_grid_transform_grad_workspace_size(input_shape, num_cameras, 1, grad_mode);
}

static gft_status multi_grad_impl(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                                  const float* output, const float* output_grad, const float* matrix_m, int32_t num_m,
                                  const float* matrix_v, const float* matrix_p, const float* frustum,
                                  int32_t num_cameras, const int32_t* camera_batch, const int32_t* output_shapes,
                                  int32_t interpolation, int32_t boundary, int32_t blending_mode, int32_t grad_mode,
                                  float* input_grad, void* workspace, size_t workspace_bytes, void* stream) {
    std::string why;
    if (!raymarch_grid_ok(input_shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!channels_ok(input_shape[4])) return fail(GFT_ERR_UNIMPLEMENTED, "Only 1,2 and 4 Channel supported.");
    if (!multi_shapes_ok(output_shapes, num_cameras, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (interpolation != GFT_FILTER_LINEAR)
        return fail(GFT_ERR_INVALID_ARGUMENT, "gradient supports LINEAR interpolation only");
    if (!enum_in(boundary, 0, 2)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid boundary mode");
    if (!enum_in(blending_mode, 0, 4) || blending_mode == GFT_BLEND_BEER_LAMBERT_EXCLUSIVE)
        return fail(GFT_ERR_INVALID_ARGUMENT, "invalid blend mode");
    const bool weights_ready = (grad_mode & GFT_GRAD_WEIGHTS_READY) != 0;
    const bool det = (grad_mode & GFT_GRAD_DETERMINISTIC) != 0;
    const int32_t ws_mode = grad_mode;
    grad_mode &= ~(GFT_GRAD_WEIGHTS_READY | GFT_GRAD_DETERMINISTIC);
    if (!enum_in(grad_mode, 0, 1) || !enum_in(input_dtype, 0, 1)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid enum");
    if (weights_ready && grad_mode != GFT_GRAD_REFERENCE)
        return fail(GFT_ERR_INVALID_ARGUMENT, "GFT_GRAD_WEIGHTS_READY needs GFT_GRAD_REFERENCE");
    if (det && weights_ready)
        return fail(GFT_ERR_INVALID_ARGUMENT, "GFT_GRAD_DETERMINISTIC computes its own weight sums");
    if (det && !det_blend_ok(blending_mode, input_shape[4]))
        return fail(GFT_ERR_UNIMPLEMENTED, "deterministic gradient: BEER_LAMBERT or ADDITIVE blending only");
    gft_status st = check_cameras(matrix_m, num_m, input_shape[0], matrix_v, matrix_p, frustum, num_cameras, 1);
    if (st != GFT_OK) return st;
    if (camera_batch != nullptr && !camera_batch_ok(camera_batch, num_cameras, input_shape[0], why))
        return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!input || !output || !output_grad || !input_grad) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    const size_t need =
        camera_batch != nullptr
            ? gft_raymarch_grid_transform_views_grad_workspace_size(input_shape, num_cameras, ws_mode)
            : gft_raymarch_grid_transform_multi_grad_workspace_size(input_shape, num_cameras, ws_mode);
    if (need > 0 && (workspace == nullptr || workspace_bytes < need))
        return fail(GFT_ERR_WORKSPACE, "raymarch gradient workspace too small");
    RaymarchArgs a{};
    a.input = input;
    a.dtype = input_dtype;
    a.N = (int)input_shape[0];
    a.C = (int)input_shape[4];
    a.din = dims_of(input_shape);
    a.filter = interpolation;
    a.boundary = boundary;
    a.blend = blending_mode;
    const auto pairs = multi_pairs(matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras, a.N, output_shapes,
                                   camera_batch);
    a.n_slots = (int)pairs.size();
    a.det = det;
    if ((st = check_aligned({input}, vec_bytes(a.C, input_dtype))) != GFT_OK ||
        (st = check_aligned({output, output_grad, input_grad}, vec_bytes(a.C, 0))) != GFT_OK ||
        (st = check_workspace_aligned(workspace)) != GFT_OK)
        return st;
    float* cnt = need > 0 ? reinterpret_cast<float*>(workspace) : nullptr;
    if (!launch_raymarch_bwd(a, pairs, output, output_grad, grad_mode == GFT_GRAD_EXACT, weights_ready, input_grad,
                             cnt, as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_raymarch_grid_transform_multi_grad(const void* input, int32_t input_dtype,
                                                  const int64_t input_shape[5], const float* output,
                                                  const float* output_grad, const float* matrix_m, int32_t num_m,
                                                  const float* matrix_v, const float* matrix_p, const float* frustum,
                                                  int32_t num_cameras, const int32_t* output_shapes,
                                                  int32_t interpolation, int32_t boundary, int32_t blending_mode,
                                                  int32_t grad_mode, float* input_grad, void* workspace,
                                                  size_t workspace_bytes, void* stream) {
    return multi_grad_impl(input, input_dtype, input_shape, output, output_grad, matrix_m, num_m, matrix_v, matrix_p,
                           frustum, num_cameras, nullptr, output_shapes, interpolation, boundary, blending_mode,
                           grad_mode, input_grad, workspace, workspace_bytes, stream);
}

gft_status gft_raymarch_grid_transform_views_grad(const void* input, int32_t input_dtype,
                                                  const int64_t input_shape[5], const float* output,
                                                  const float* output_grad, const float* matrix_m, int32_t num_m,
                                                  const float* matrix_v, const float* matrix_p, const float* frustum,
                                                  int32_t num_cameras, const int32_t* camera_batch,
                                                  const int32_t* output_shapes, int32_t interpolation,
                                                  int32_t boundary, int32_t blending_mode, int32_t grad_mode,
                                                  float* input_grad, void* workspace, size_t workspace_bytes,
                                                  void* stream) {
    if (camera_batch == nullptr) return fail(GFT_ERR_INVALID_ARGUMENT, "camera_batch is NULL");
    return multi_grad_impl(input, input_dtype, input_shape, output, output_grad, matrix_m, num_m, matrix_v, matrix_p,
                           frustum, num_cameras, camera_batch, output_shapes, interpolation, boundary, blending_mode,
                           grad_mode, input_grad, workspace, workspace_bytes, stream);
}

static gft_status multi_weights_impl(const int64_t input_shape[5], const float* matrix_m, int32_t num_m,
                                     const float* matrix_v, const float* matrix_p, const float* frustum,
                                     int32_t num_cameras, const int32_t* camera_batch, const int32_t* output_shapes,
                                     int32_t boundary, void* workspace, size_t workspace_bytes, void* stream) {
    std::string why;
    if (!raymarch_grid_ok(input_shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!multi_shapes_ok(output_shapes, num_cameras, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!enum_in(boundary, 0, 2)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid boundary mode");
    gft_status st = check_cameras(matrix_m, num_m, input_shape[0], matrix_v, matrix_p, frustum, num_cameras, 1);
    if (st != GFT_OK) return st;
    if (camera_batch != nullptr && !camera_batch_ok(camera_batch, num_cameras, input_shape[0], why))
        return fail(GFT_ERR_INVALID_ARGUMENT, why);
    const size_t need =
        camera_batch != nullptr
            ? gft_raymarch_grid_transform_views_grad_workspace_size(input_shape, num_cameras, GFT_GRAD_REFERENCE)
            : gft_raymarch_grid_transform_multi_grad_workspace_size(input_shape, num_cameras, GFT_GRAD_REFERENCE);
    if (workspace == nullptr || workspace_bytes < need)
        return fail(GFT_ERR_WORKSPACE, "raymarch gradient workspace too small");
    if ((st = check_workspace_aligned(workspace)) != GFT_OK) return st;
    RaymarchArgs a{};
    a.N = (int)input_shape[0];
    a.C = (int)input_shape[4];
    a.din = dims_of(input_shape);
    a.filter = GFT_FILTER_LINEAR;
    a.boundary = boundary;
    const auto pairs = multi_pairs(matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras, a.N, output_shapes,
                                   camera_batch);
    a.n_slots = (int)pairs.size();
    if (!launch_raymarch_weights(a, pairs, reinterpret_cast<float*>(workspace), as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_raymarch_grid_transform_multi_grad_weights(const int64_t input_shape[5], const float* matrix_m,
                                                          int32_t num_m, const float* matrix_v, const float* matrix_p,
                                                          const float* frustum, int32_t num_cameras,
                                                          const int32_t* output_shapes, int32_t boundary,
                                                          void* workspace, size_t workspace_bytes, void* stream) {
    return multi_weights_impl(input_shape, matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras, nullptr,
                              output_shapes, boundary, workspace, workspace_bytes, stream);
}

gft_status gft_raymarch_grid_transform_views_grad_weights(const int64_t input_shape[5], const float* matrix_m,
                                                          int32_t num_m, const float* matrix_v, const float* matrix_p,
                                                          const float* frustum, int32_t num_cameras,
                                                          const int32_t* camera_batch, const int32_t* output_shapes,
                                                          int32_t boundary, void* workspace, size_t workspace_bytes,
                                                          void* stream) {
    if (camera_batch == nullptr) return fail(GFT_ERR_INVALID_ARGUMENT, "camera_batch is NULL");
    return multi_weights_impl(input_shape, matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras, camera_batch,
                              output_shapes, boundary, workspace, workspace_bytes, stream);
}

// ---------------------------------------------------------------- resample
static size_t mip_ws_bytes(const int64_t* s, int mip, int num) {
    if (mip == GFT_MIP_NONE) return 0;
    const int L = usable_mip_levels(dims_of(s), num);
    return sizeof(float) * mip_workspace_floats(dims_of(s), L, (int)s[4]) * (size_t)s[0];
}
// SampleGridTransform's workspace: the mips, then (with mips) the occupancy
// maps of the N input slices.
static size_t transform_ws_bytes(const int64_t* s, int mip, int num) {
    const size_t m = mip_ws_bytes(s, mip, num);
    return m == 0 ? 0 : align256(m) + occupancy_bytes(dims_of(s)) * (size_t)s[0];
}

size_t gft_sample_grid_transform_workspace_size(const int64_t input_shape[5], int32_t mipmapping, int32_t num_mipmaps) {
    std::string why;
    if (!grid_shape_ok(input_shape, why)) return 0;
    return transform_ws_bytes(input_shape, mipmapping, num_mipmaps);
}

static bool build_batch_mips(const void* input, int dtype, const int64_t* s, int mip, int num, void* ws,
                             std::vector<MipSet>& sets, cudaStream_t st) {
    const int N = (int)s[0], C = (int)s[4];
    const Dims d = dims_of(s);
    const int L = (mip == GFT_MIP_NONE) ? 0 : usable_mip_levels(d, num);
    const size_t per = mip_workspace_floats(d, L, C);
    sets.resize(N);
    const size_t esz = dtype == GFT_DTYPE_BF16 ? 2 : 4;
    for (int b = 0; b < N; ++b) {
        const void* base = reinterpret_cast<const char*>(input) + (size_t)b * voxels(d) * C * esz;
        if (!launch_build_mips(base, dtype, C, d, L, reinterpret_cast<float*>(ws) + per * b, st, &sets[b]))
            return false;
    }
    return true;
}

gft_status gft_sample_grid_transform(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                                     const float* matrix_m, int32_t num_m, const float* matrix_v,
                                     const float* matrix_p, const float* frustum, int32_t num_cameras,
                                     const int32_t output_shape[3], int32_t interpolation, int32_t boundary,
                                     int32_t mipmapping, int32_t num_mipmaps, float mip_bias,
                                     int32_t coordinate_mode, float cell_center_offset,
                                     int32_t separate_camera_batch, float* output, void* workspace,
                                     size_t workspace_bytes, void* stream) {
    std::string why;
    const bool dense = (interpolation & GFT_SAMPLE_DENSE) != 0;
    interpolation &= ~GFT_SAMPLE_DENSE;
    if (!grid_shape_ok(input_shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!channels_ok(input_shape[4])) return fail(GFT_ERR_UNIMPLEMENTED, "Only 1,2 and 4 Channel supported.");
    if (output_shape == nullptr || output_shape[0] < 1 || output_shape[1] < 1 || output_shape[2] < 1)
        return fail(GFT_ERR_INVALID_ARGUMENT, "All shape dimensions must be positive (output_shape)");
    if (!enum_in(interpolation, 0, 3) || !enum_in(boundary, 0, 2) || !enum_in(mipmapping, 0, 2) ||
        !enum_in(input_dtype, 0, 1))
        return fail(GFT_ERR_INVALID_ARGUMENT, "invalid enum");
    if (!(coordinate_mode == 0 || coordinate_mode == 1 || coordinate_mode == 3 || coordinate_mode == 4))
        return fail(GFT_ERR_INVALID_ARGUMENT, "Invalid coordinate_mode");
    if (num_mipmaps <= 0 && mipmapping != GFT_MIP_NONE)
        return fail(GFT_ERR_INVALID_ARGUMENT, "when using mipmaps num_mipmaps must be larger than 0.");
    if (cell_center_offset != 0.5f)
        return fail(GFT_ERR_INVALID_ARGUMENT, "Invalid cell center offset for given coordinate mode.");
    gft_status st = check_cameras(matrix_m, num_m, input_shape[0], matrix_v, matrix_p, frustum, num_cameras,
                                  separate_camera_batch);
    if (st != GFT_OK) return st;
    if (!input || !output) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    const size_t need = transform_ws_bytes(input_shape, mipmapping, num_mipmaps);
    if (need > 0 && (workspace == nullptr || workspace_bytes < need))
        return fail(GFT_ERR_WORKSPACE, "mip workspace too small");
    if ((st = check_aligned({input}, vec_bytes(input_shape[4], input_dtype))) != GFT_OK ||
        (st = check_aligned({output}, vec_bytes(input_shape[4], 0))) != GFT_OK ||
        (st = check_workspace_aligned(workspace)) != GFT_OK)
        return st;
    std::vector<MipSet> sets;
    if (!build_batch_mips(input, input_dtype, input_shape, mipmapping, num_mipmaps, workspace, sets, as_stream(stream)))
        return GFT_ERR_CUDA;
    // Occupancy (forward modes, whose input is a volume, often mostly empty;
    // BORDER / CLAMP with LINEAR or NEAREST filtering): samples reading only
    // zeros skip their LOD and fetches.
    if (need > 0 && !dense && (coordinate_mode == 0 || coordinate_mode == 3) &&
        (boundary == GFT_BOUNDARY_BORDER || boundary == GFT_BOUNDARY_CLAMP) &&
        (interpolation == GFT_FILTER_LINEAR || interpolation == GFT_FILTER_NEAREST)) {
        const Dims d = dims_of(input_shape);
        const size_t esz = input_dtype == GFT_DTYPE_BF16 ? 2 : 4, ob = occupancy_bytes(d);
        uint8_t* occ = reinterpret_cast<uint8_t*>(workspace) + align256(mip_ws_bytes(input_shape, mipmapping, num_mipmaps));
        for (int b = 0; b < (int)input_shape[0]; ++b) {
            const void* base = reinterpret_cast<const char*>(input) + (size_t)b * voxels(d) * input_shape[4] * esz;
            uint8_t* raw = occ + ob * b;
            if (!launch_occupancy(base, input_dtype, (int)input_shape[4], d, sets[b].levels, raw, raw + ob / 2,
                                  as_stream(stream), &sets[b]))
                return GFT_ERR_CUDA;
        }
    }
    SampleArgs a;
    a.input = input;
    a.dtype = input_dtype;
    a.N = (int)input_shape[0];
    a.C = (int)input_shape[4];
    a.din = dims_of(input_shape);
    a.dout = Dims{output_shape[2], output_shape[1], output_shape[0]};
    a.filter = interpolation;
    a.boundary = boundary;
    a.mip_mode = mipmapping;
    a.levels = sets.empty() ? 0 : sets[0].levels;
    a.mip_bias = mip_bias;
    a.cco = cell_center_offset;
    a.coord_mode = coordinate_mode;
    const auto pairs = make_pairs(matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras, a.N,
                                  separate_camera_batch != 0);
    if (!launch_sample_transform_fwd(a, pairs, sets.data(), output, as_stream(stream))) return GFT_ERR_CUDA;
    return GFT_OK;
}

size_t gft_sample_grid_transform_grad_workspace_size(const int64_t input_shape[5]) {
    std::string why;
    if (!grid_shape_ok(input_shape, why)) return 0;
    return align256(sizeof(unsigned int) * (size_t)input_shape[1] * input_shape[2] * input_shape[3]);
}

gft_status gft_sample_grid_transform_grad(const int64_t input_shape[5], const float* output_grad,
                                          const int64_t output_grad_shape[6], const float* matrix_m, int32_t num_m,
                                          const float* matrix_v, const float* matrix_p, const float* frustum,
                                          int32_t num_cameras, int32_t interpolation, int32_t boundary,
                                          int32_t coordinate_mode, float cell_center_offset,
                                          int32_t separate_camera_batch, int32_t grad_mode, float* input_grad,
                                          void* workspace, size_t workspace_bytes, void* stream) {
    std::string why;
    if (!grid_shape_ok(input_shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!channels_ok(input_shape[4])) return fail(GFT_ERR_UNIMPLEMENTED, "Only 1,2 and 4 Channel supported.");
    if (output_grad_shape == nullptr) return fail(GFT_ERR_INVALID_ARGUMENT, "output_grad shape is NULL");
    for (int i = 0; i < 6; ++i)
        if (output_grad_shape[i] <= 0) return fail(GFT_ERR_INVALID_ARGUMENT, "Invalid output_grads shape (NVDHWC)");
    if (output_grad_shape[0] != input_shape[0])
        return fail(GFT_ERR_INVALID_ARGUMENT, "output_grads batch size does not match input batch size.");
    if (output_grad_shape[5] != input_shape[4]) return fail(GFT_ERR_INVALID_ARGUMENT, "channel mismatch");
    if (!enum_in(interpolation, 0, 3) || !enum_in(boundary, 0, 2) || !enum_in(grad_mode, 0, 1))
        return fail(GFT_ERR_INVALID_ARGUMENT, "invalid enum");
    if (!(coordinate_mode == 0 || coordinate_mode == 1 || coordinate_mode == 3 || coordinate_mode == 4))
        return fail(GFT_ERR_INVALID_ARGUMENT, "Invalid coordinate_mode");
    if (cell_center_offset != 0.5f)
        return fail(GFT_ERR_INVALID_ARGUMENT, "Invalid cell center offset for given coordinate mode.");
    gft_status st = check_cameras(matrix_m, num_m, input_shape[0], matrix_v, matrix_p, frustum, num_cameras,
                                  separate_camera_batch);
    if (st != GFT_OK) return st;
    if (output_grad_shape[1] != (separate_camera_batch ? num_cameras : 1))
        return fail(GFT_ERR_INVALID_ARGUMENT, "output_grads views size does not match cameras.");
    if (!output_grad || !input_grad) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    const size_t need = gft_sample_grid_transform_grad_workspace_size(input_shape);
    if (grad_mode == GFT_GRAD_REFERENCE && (workspace == nullptr || workspace_bytes < need))
        return fail(GFT_ERR_WORKSPACE, "sample count workspace too small");
    if ((st = check_aligned({output_grad, input_grad}, vec_bytes(input_shape[4], 0))) != GFT_OK ||
        (st = check_workspace_aligned(workspace)) != GFT_OK)
        return st;
    const auto pairs = make_pairs(matrix_m, num_m, matrix_v, matrix_p, frustum, num_cameras, (int)input_shape[0],
                                  separate_camera_batch != 0);
    const Dims dout{(int)output_grad_shape[4], (int)output_grad_shape[3], (int)output_grad_shape[2]};
    if (!launch_sample_transform_bwd((int)input_shape[0], (int)input_shape[4], dims_of(input_shape), dout, boundary,
                                     coordinate_mode, cell_center_offset, pairs, output_grad,
                                     grad_mode == GFT_GRAD_EXACT, input_grad,
                                     reinterpret_cast<unsigned int*>(workspace), as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

size_t gft_sample_grid_lut_workspace_size(const int64_t input_shape[5], int32_t mipmapping, int32_t num_mipmaps) {
    std::string why;
    if (!grid_shape_ok(input_shape, why)) return 0;
    return mip_ws_bytes(input_shape, mipmapping, num_mipmaps);
}

static gft_status check_lut(const int64_t* input_shape, const int64_t* lookup_shape, int separate) {
    std::string why;
    if (!grid_shape_ok(input_shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!channels_ok(input_shape[4])) return fail(GFT_ERR_UNIMPLEMENTED, "Only 1,2 and 4 Channel supported.");
    if (!grid_shape_ok(lookup_shape, why) || lookup_shape[4] != 4)
        return fail(GFT_ERR_INVALID_ARGUMENT, "Invalid lut shape (NDHWC) with C=4");
    if (!separate && lookup_shape[0] != input_shape[0])
        return fail(GFT_ERR_INVALID_ARGUMENT, "camera batch must match data batch when not using global sampling.");
    return GFT_OK;
}

gft_status gft_sample_grid_lut(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                               const float* lookup, const int64_t lookup_shape[5], int32_t interpolation,
                               int32_t boundary, int32_t mipmapping, int32_t num_mipmaps, float mip_bias,
                               float cell_center_offset, int32_t separate_camera_batch, int32_t relative_coords,
                               int32_t normalized_coords, float* output, void* workspace, size_t workspace_bytes,
                               void* stream) {
    gft_status st = check_lut(input_shape, lookup_shape, separate_camera_batch);
    if (st != GFT_OK) return st;
    if (!enum_in(interpolation, 0, 3) || !enum_in(boundary, 0, 2) || !enum_in(mipmapping, 0, 2) ||
        !enum_in(input_dtype, 0, 1))
        return fail(GFT_ERR_INVALID_ARGUMENT, "invalid enum");
    if (num_mipmaps <= 0 && mipmapping != GFT_MIP_NONE)
        return fail(GFT_ERR_INVALID_ARGUMENT, "when using mipmaps num_mipmaps must be larger than 0.");
    if (normalized_coords && cell_center_offset != 0.5f)
        return fail(GFT_ERR_INVALID_ARGUMENT, "Invalid cell center offset must be 0.5 when using normalized coordinates.");
    if (!input || !lookup || !output) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    const size_t need = mip_ws_bytes(input_shape, mipmapping, num_mipmaps);
    if (need > 0 && (workspace == nullptr || workspace_bytes < need))
        return fail(GFT_ERR_WORKSPACE, "mip workspace too small");
    if ((st = check_aligned({input}, vec_bytes(input_shape[4], input_dtype))) != GFT_OK ||
        (st = check_aligned({output}, vec_bytes(input_shape[4], 0))) != GFT_OK ||
        (st = check_aligned({lookup}, 16)) != GFT_OK || (st = check_workspace_aligned(workspace)) != GFT_OK)
        return st;
    std::vector<MipSet> sets;
    if (!build_batch_mips(input, input_dtype, input_shape, mipmapping, num_mipmaps, workspace, sets, as_stream(stream)))
        return GFT_ERR_CUDA;
    LutArgs a;
    a.input = input;
    a.dtype = input_dtype;
    a.N = (int)input_shape[0];
    a.C = (int)input_shape[4];
    a.din = dims_of(input_shape);
    a.dout = dims_of(lookup_shape);
    a.n_lut = (int)lookup_shape[0];
    a.filter = interpolation;
    a.boundary = boundary;
    a.mip_mode = mipmapping;
    a.levels = sets.empty() ? 0 : sets[0].levels;
    a.mip_bias = mip_bias;
    a.cco = cell_center_offset;
    a.separate = separate_camera_batch;
    a.relative = relative_coords;
    a.normalized = normalized_coords;
    if (!launch_lut_fwd(a, lookup, sets.data(), output, as_stream(stream))) return GFT_ERR_CUDA;
    return GFT_OK;
}

size_t gft_sample_grid_lut_grad_workspace_size(const int64_t input_shape[5]) {
    return gft_sample_grid_transform_grad_workspace_size(input_shape);
}

gft_status gft_sample_grid_lut_grad(const float* input, const int64_t input_shape[5], const float* output_grad,
                                    const float* lookup, const int64_t lookup_shape[5], int32_t interpolation,
                                    int32_t boundary, float cell_center_offset, int32_t separate_camera_batch,
                                    int32_t relative_coords, int32_t normalized_coords, int32_t grad_mode,
                                    float* input_grad, float* lookup_grad, void* workspace, size_t workspace_bytes,
                                    void* stream) {
    gft_status st = check_lut(input_shape, lookup_shape, separate_camera_batch);
    if (st != GFT_OK) return st;
    if (!enum_in(interpolation, 0, 3) || !enum_in(boundary, 0, 2) || !enum_in(grad_mode, 0, 1))
        return fail(GFT_ERR_INVALID_ARGUMENT, "invalid enum");
    if (normalized_coords && cell_center_offset != 0.5f)
        return fail(GFT_ERR_INVALID_ARGUMENT, "Invalid cell center offset must be 0.5 when using normalized coordinates.");
    if (!input || !lookup || !output_grad || !input_grad || !lookup_grad)
        return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    const size_t need = gft_sample_grid_lut_grad_workspace_size(input_shape);
    if (grad_mode == GFT_GRAD_REFERENCE && (workspace == nullptr || workspace_bytes < need))
        return fail(GFT_ERR_WORKSPACE, "sample count workspace too small");
    if ((st = check_aligned({input, output_grad, input_grad}, vec_bytes(input_shape[4], 0))) != GFT_OK ||
        (st = check_aligned({lookup, lookup_grad}, 16)) != GFT_OK || (st = check_workspace_aligned(workspace)) != GFT_OK)
        return st;
    LutArgs a;
    a.input = input;
    a.dtype = 0;
    a.N = (int)input_shape[0];
    a.C = (int)input_shape[4];
    a.din = dims_of(input_shape);
    a.dout = dims_of(lookup_shape);
    a.n_lut = (int)lookup_shape[0];
    a.filter = interpolation;
    a.boundary = boundary;
    a.mip_mode = 0;
    a.levels = 0;
    a.mip_bias = 0.f;
    a.cco = cell_center_offset;
    a.separate = separate_camera_batch;
    a.relative = relative_coords;
    a.normalized = normalized_coords;
    if (!launch_lut_bwd(a, input, lookup, output_grad, grad_mode == GFT_GRAD_EXACT, input_grad, lookup_grad,
                        reinterpret_cast<unsigned int*>(workspace), as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_lod_transform(const int32_t input_shape[3], const float* matrix_mv, const float* matrix_p,
                             const float* frustum, int32_t num, const int32_t output_shape[3],
                             int32_t inverse_transform, float* output, void* stream) {
    if (!input_shape || !output_shape || input_shape[0] < 1 || input_shape[1] < 1 || input_shape[2] < 1 ||
        output_shape[0] < 1 || output_shape[1] < 1 || output_shape[2] < 1)
        return fail(GFT_ERR_INVALID_ARGUMENT, "All shape dimensions must be positive");
    if (!matrix_mv || !matrix_p || !frustum || num <= 0) return fail(GFT_ERR_INVALID_ARGUMENT, "camera batch size mismatch");
    if (!output) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    if (const gft_status st = check_aligned({output}, 16); st != GFT_OK) return st;
    const auto pairs = make_pairs(nullptr, 1, matrix_mv, matrix_p, frustum, num, num, false);
    const Dims din{input_shape[2], input_shape[1], input_shape[0]};
    const Dims dout{output_shape[2], output_shape[1], output_shape[0]};
    if (!launch_lod_transform(din, dout, pairs, inverse_transform != 0, output, as_stream(stream))) return GFT_ERR_CUDA;
    return GFT_OK;
}

// ---------------------------------------------------------------- blend
gft_status gft_reduce_grid_blend(const float* input, const int64_t input_shape[5], int32_t blending_mode,
                                 int32_t keep_dims, float* output, void* stream) {
    std::string why;
    if (!grid_shape_ok(input_shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!channels_ok(input_shape[4])) return fail(GFT_ERR_UNIMPLEMENTED, "Only 1,2 and 4 Channel supported.");
    if (!enum_in(blending_mode, 0, 4) || blending_mode == GFT_BLEND_BEER_LAMBERT_EXCLUSIVE)
        return fail(GFT_ERR_INVALID_ARGUMENT, "invalid blending mode");
    if (!input || !output) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    if (const gft_status st = check_aligned({input, output}, vec_bytes(input_shape[4], 0)); st != GFT_OK) return st;
    if (!launch_blend_fwd(input, (int)input_shape[0], (int)input_shape[4], dims_of(input_shape), blending_mode,
                          keep_dims != 0, output, as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_reduce_grid_blend_grad(const float* output_grad, const float* output, const float* input,
                                      const int64_t input_shape[5], int32_t blending_mode, int32_t keep_dims,
                                      int32_t grad_mode, float* input_grad, void* stream) {
    std::string why;
    if (!grid_shape_ok(input_shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!channels_ok(input_shape[4])) return fail(GFT_ERR_UNIMPLEMENTED, "Only 1,2 and 4 Channel supported.");
    // ReduceGridBlendGrad accepts BEER_LAMBERT, ALPHA and ADDITIVE (reduce_blend.cc:41)
    if (!(blending_mode == GFT_BLEND_BEER_LAMBERT || blending_mode == GFT_BLEND_ALPHA ||
          blending_mode == GFT_BLEND_ADDITIVE))
        return fail(GFT_ERR_INVALID_ARGUMENT, "invalid blending mode");
    if (!enum_in(grad_mode, 0, 1)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid enum");
    if (!output_grad || !output || !input || !input_grad) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    if (const gft_status st = check_aligned({output_grad, output, input, input_grad}, vec_bytes(input_shape[4], 0));
        st != GFT_OK)
        return st;
    if (!launch_blend_bwd(output_grad, output, input, (int)input_shape[0], (int)input_shape[4], dims_of(input_shape),
                          blending_mode, keep_dims != 0, grad_mode == GFT_GRAD_EXACT, input_grad, as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

// ---------------------------------------------------------------- advect
size_t gft_advect_workspace_size(const int64_t density_shape[5], int32_t order) {
    std::string why;
    if (!grid_shape_ok(density_shape, why) || order != 2) return 0;
    return align256(sizeof(float) * (size_t)density_shape[1] * density_shape[2] * density_shape[3] * density_shape[4]);
}

static gft_status check_advect(const int64_t* s, const float* vx, const float* vy, const float* vz, int order,
                               int clamp, int boundary) {
    std::string why;
    if (!grid_shape_ok(s, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!channels_ok(s[4])) return fail(GFT_ERR_UNIMPLEMENTED, "Only 1,2 and 4 Channel supported.");
    if (order != 1 && order != 2) return fail(GFT_ERR_INVALID_ARGUMENT, "Unsupported warp order");
    if (!enum_in(clamp, 0, 2)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid clamp");
    if (!enum_in(boundary, 0, 2)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid boundary mode");
    if (!vx || !vy || !vz) return fail(GFT_ERR_INVALID_ARGUMENT, "velocity pointer is NULL");
    return GFT_OK;
}

gft_status gft_advect(const void* density, int32_t density_dtype, const int64_t density_shape[5], const float* vel_x,
                      const float* vel_y, const float* vel_z, float dt, int32_t order, int32_t clamp,
                      int32_t boundary, float* output, void* workspace, size_t workspace_bytes, void* stream) {
    gft_status st = check_advect(density_shape, vel_x, vel_y, vel_z, order, clamp, boundary);
    if (st != GFT_OK) return st;
    if (!enum_in(density_dtype, 0, 1)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid enum");
    if (!density || !output) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    const size_t need = gft_advect_workspace_size(density_shape, order);
    if (need > 0 && (workspace == nullptr || workspace_bytes < need))
        return fail(GFT_ERR_WORKSPACE, "advect workspace too small");
    if ((st = check_aligned({density}, vec_bytes(density_shape[4], density_dtype))) != GFT_OK ||
        (st = check_aligned({output}, vec_bytes(density_shape[4], 0))) != GFT_OK ||
        (st = check_aligned({vel_x, vel_y, vel_z}, 4)) != GFT_OK || (st = check_workspace_aligned(workspace)) != GFT_OK)
        return st;
    AdvectArgs a;
    a.density = density;
    a.dtype = density_dtype;
    a.N = (int)density_shape[0];
    a.C = (int)density_shape[4];
    a.d = dims_of(density_shape);
    a.vx = vel_x;
    a.vy = vel_y;
    a.vz = vel_z;
    a.dt = dt;
    a.order = order;
    a.clamp = clamp;
    a.boundary = boundary;
    if (!launch_advect_fwd(a, output, reinterpret_cast<float*>(workspace), as_stream(stream))) return GFT_ERR_CUDA;
    return GFT_OK;
}

size_t gft_advect_grad_workspace_size(const int64_t density_shape[5], int32_t order) {
    std::string why;
    if (!grid_shape_ok(density_shape, why)) return 0;
    const size_t nv = (size_t)density_shape[1] * density_shape[2] * density_shape[3];
    const size_t C = (size_t)density_shape[4];
    // + 16 bytes: the single-channel layout pads two regions to even offsets
    return align256(sizeof(float) * (nv * (4 * C + 3)) + sizeof(unsigned int) * 2 * nv + 16);
}

size_t gft_advect_grad_workspace_size_mode(const int64_t density_shape[5], int32_t order, int32_t grad_mode) {
    if ((grad_mode & GFT_GRAD_DETERMINISTIC) == 0) return gft_advect_grad_workspace_size(density_shape, order);
    std::string why;
    if (!grid_shape_ok(density_shape, why)) return 0;
    const size_t nv = (size_t)density_shape[1] * density_shape[2] * density_shape[3];
    return align256(advect_det_ws_bytes(nv, (size_t)density_shape[4]));
}

gft_status gft_advect_grad(const float* density, const int64_t density_shape[5], const float* vel_x,
                           const float* vel_y, const float* vel_z, float dt, int32_t order, int32_t clamp,
                           int32_t boundary, int32_t grad_mode, const float* output_grad, float* density_grad,
                           float* vel_x_grad, float* vel_y_grad, float* vel_z_grad, void* workspace,
                           size_t workspace_bytes, void* stream) {
    gft_status st = check_advect(density_shape, vel_x, vel_y, vel_z, order, clamp, boundary);
    if (st != GFT_OK) return st;
    const size_t need = gft_advect_grad_workspace_size_mode(density_shape, order, grad_mode);
    const bool forward_ready = (grad_mode & GFT_GRAD_FORWARD_READY) != 0;
    const bool det = (grad_mode & GFT_GRAD_DETERMINISTIC) != 0;
    grad_mode &= ~(GFT_GRAD_FORWARD_READY | GFT_GRAD_DETERMINISTIC);
    if (!enum_in(grad_mode, 0, 1)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid enum");
    if (forward_ready && (order != 2 || density_shape[0] != 1))
        return fail(GFT_ERR_INVALID_ARGUMENT, "GFT_GRAD_FORWARD_READY needs order 2 and one batch slice");
    if (!density || !output_grad || !density_grad || !vel_x_grad || !vel_y_grad || !vel_z_grad)
        return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    if (workspace == nullptr || workspace_bytes < need) return fail(GFT_ERR_WORKSPACE, "advect gradient workspace too small");
    if ((st = check_aligned({density, output_grad, density_grad}, vec_bytes(density_shape[4], 0))) != GFT_OK ||
        (st = check_aligned({vel_x, vel_y, vel_z, vel_x_grad, vel_y_grad, vel_z_grad}, 4)) != GFT_OK ||
        (st = check_workspace_aligned(workspace)) != GFT_OK)
        return st;
    AdvectArgs a;
    a.density = density;
    a.dtype = 0;
    a.N = (int)density_shape[0];
    a.C = (int)density_shape[4];
    a.d = dims_of(density_shape);
    a.vx = vel_x;
    a.vy = vel_y;
    a.vz = vel_z;
    a.dt = dt;
    a.order = order;
    a.clamp = clamp;
    a.boundary = boundary;
    a.det = det;
    if (!launch_advect_bwd(a, grad_mode == GFT_GRAD_EXACT, forward_ready, output_grad, density_grad, vel_x_grad,
                           vel_y_grad, vel_z_grad, reinterpret_cast<float*>(workspace), as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

// ---------------------------------------------------------------- pipeline fusions
static bool single_channel_grid(const int64_t* shape, std::string& why) {
    if (!grid_shape_ok(shape, why)) return false;
    if (shape[4] != 1) {
        why = "expected a single-channel grid [N, D, H, W, 1]";
        return false;
    }
    return true;
}

gft_status gft_transmittance(const float* input, const int64_t shape[5], float* output, void* stream) {
    std::string why;
    if (!single_channel_grid(shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!input || !output) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    if (const gft_status st = check_aligned({input, output}, 4); st != GFT_OK) return st;
    if (!launch_transmittance(input, (int)shape[0], dims_of(shape), output, as_stream(stream))) return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_transmittance_grad(const float* output, const float* output_grad, const int64_t shape[5],
                                  float* input_grad, void* stream) {
    std::string why;
    if (!single_channel_grid(shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!output || !output_grad || !input_grad) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    if (const gft_status st = check_aligned({output, output_grad, input_grad}, 4); st != GFT_OK) return st;
    if (!launch_transmittance_grad(output, output_grad, (int)shape[0], dims_of(shape), input_grad, as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

static bool layout_ok(int32_t layout) { return layout == 0 || layout == GFT_LAYOUT_BRICK; }

// ---------------------------------------------------------------- FP64 checks
gft_status gft_transmittance_check(const float* input, const float* output, const int64_t shape[5],
                                   int32_t column_stride, double* result, void* stream) {
    std::string why;
    if (!single_channel_grid(shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (column_stride < 1) return fail(GFT_ERR_INVALID_ARGUMENT, "column stride must be positive");
    if (!input || !output || !result) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    gft_status st;
    if ((st = check_aligned({input, output}, 4)) != GFT_OK || (st = check_aligned({result}, 16)) != GFT_OK) return st;
    if (!launch_transmittance_check(input, output, (int)shape[0], dims_of(shape), column_stride, result,
                                    as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_raymarch_check(const void* input, int32_t input_dtype, const int64_t input_shape[5],
                              const float* matrix_m, int32_t num_m, const float* matrix_v, const float* matrix_p,
                              const float* frustum, int32_t num_cameras, const int32_t output_shape[3],
                              const float* output, int32_t ray_stride, double* result, void* stream) {
    std::string why;
    const int32_t layout = input_dtype & GFT_LAYOUT_BRICK;
    const int32_t dtype = input_dtype & ~GFT_LAYOUT_BRICK;
    if (!raymarch_grid_ok(input_shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!channels_ok(input_shape[4])) return fail(GFT_ERR_UNIMPLEMENTED, "Only 1,2 and 4 Channel supported.");
    if (!enum_in(dtype, 0, 1)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid enum");
    if (output_shape == nullptr || output_shape[0] <= 0 || output_shape[1] <= 0 || output_shape[2] <= 0)
        return fail(GFT_ERR_INVALID_ARGUMENT, "invalid output shape");
    if (ray_stride < 1) return fail(GFT_ERR_INVALID_ARGUMENT, "ray stride must be positive");
    if (!input || !output || !result) return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    gft_status st = check_cameras(matrix_m, num_m, input_shape[0], matrix_v, matrix_p, frustum, num_cameras, 1);
    if (st != GFT_OK) return st;
    if ((st = check_aligned({input}, vec_bytes(input_shape[4], dtype))) != GFT_OK ||
        (st = check_aligned({output}, vec_bytes(input_shape[4], 0))) != GFT_OK ||
        (st = check_aligned({result}, 16)) != GFT_OK)
        return st;
    // every (batch, camera) pair with the camera inverses in double
    std::vector<CheckTable> tabs;
    const int N = (int)input_shape[0];
    for (int b = 0; b < N; ++b)
        for (int c = 0; c < num_cameras; ++c) {
            if (tabs.empty() || tabs.back().n == MAX_PAIRS) {
                tabs.emplace_back();
                std::memset(&tabs.back(), 0, sizeof(CheckTable));
            }
            CheckTable& t = tabs.back();
            double m[4][4], v[4][4], p[4][4], mv[4][4], mvi[4][4], pi[4][4];
            mat_from_flat(matrix_m + 16 * (num_m == 1 ? 0 : b), m);
            mat_from_flat(matrix_v + 16 * c, v);
            mat_from_flat(matrix_p + 16 * c, p);
            matmul4(v, m, mv);
            inverse4(mv, mvi);
            inverse4(p, pi);
            for (int r = 0; r < 4; ++r)
                for (int k = 0; k < 4; ++k) {
                    t.cam[t.n].mvi[4 * r + k] = mvi[r][k];
                    t.cam[t.n].pi[4 * r + k] = pi[r][k];
                }
            t.in_batch[t.n] = b;
            t.out_slot[t.n] = b * num_cameras + c;
            ++t.n;
        }
    if (!launch_raymarch_check(input, dtype, layout ? LAYOUT_BRICK : LAYOUT_FLAT, (int)input_shape[4],
                               dims_of(input_shape), tabs, output_shape[2], output_shape[1], output_shape[0], output,
                               ray_stride, result, as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_light_compose(const float* density, const float* transmittance, const float* light_color,
                             const int64_t shape[5], float ambient, float scale, int32_t output_layout, void* output,
                             void* stream) {
    std::string why;
    if (!single_channel_grid(shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    const bool bf16 = (output_layout & ~GFT_LAYOUT_BRICK) == GFT_DTYPE_BF16;
    if (bf16) output_layout &= GFT_LAYOUT_BRICK;
    if (!layout_ok(output_layout)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid layout");
    if (voxels(dims_of(shape)) >= MAX_SLICE_CELLS) return fail(GFT_ERR_INVALID_ARGUMENT, "grid slice too large");
    if (!density || !transmittance || !light_color || !output)
        return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    gft_status st;
    if ((st = check_aligned({density, transmittance, light_color}, 4)) != GFT_OK ||
        (st = check_aligned({output}, bf16 ? 8 : 16)) != GFT_OK)
        return st;
    if (!launch_light_compose(density, transmittance, light_color, nullptr, (int)shape[0], dims_of(shape), ambient,
                              scale, output_layout ? LAYOUT_BRICK : LAYOUT_FLAT, bf16, output, as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_light_compose_factored(const float* density, const float* transmittance, const float* falloff,
                                      const float light_rgb[3], const int64_t shape[5], float ambient, float scale,
                                      int32_t output_layout, void* output, void* stream) {
    std::string why;
    if (!single_channel_grid(shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    const bool bf16 = (output_layout & ~GFT_LAYOUT_BRICK) == GFT_DTYPE_BF16;
    if (bf16) output_layout &= GFT_LAYOUT_BRICK;
    if (!layout_ok(output_layout)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid layout");
    if (voxels(dims_of(shape)) >= MAX_SLICE_CELLS) return fail(GFT_ERR_INVALID_ARGUMENT, "grid slice too large");
    if (!density || !transmittance || !falloff || !light_rgb || !output)
        return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    gft_status st;
    if ((st = check_aligned({density, transmittance, falloff}, 4)) != GFT_OK ||
        (st = check_aligned({output}, bf16 ? 8 : 16)) != GFT_OK)
        return st;
    if (!launch_light_compose(density, transmittance, falloff, light_rgb, (int)shape[0], dims_of(shape), ambient,
                              scale, output_layout ? LAYOUT_BRICK : LAYOUT_FLAT, bf16, output, as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_light_compose_projection(const float light_rgb[3], float ambient, float scale, float projection[8]) {
    if (light_rgb == nullptr || projection == nullptr) return fail(GFT_ERR_INVALID_ARGUMENT, "pointer is NULL");
    for (int c = 0; c < 3; ++c) {
        projection[c] = scale * light_rgb[c];
        projection[4 + c] = scale * ambient;
    }
    projection[3] = 0.f;
    projection[7] = scale;
    return GFT_OK;
}

gft_status gft_light_compose_factored_grad_cameras(const float* density, const float* transmittance,
                                                   const float* falloff, const int64_t shape[5], int32_t num_cameras,
                                                   const float* camera_sums, const float* weight_sums,
                                                   float* density_grad, float* transmittance_grad, void* stream) {
    std::string why;
    if (!single_channel_grid(shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (num_cameras < 1) return fail(GFT_ERR_INVALID_ARGUMENT, "num_cameras must be positive");
    if (voxels(dims_of(shape)) >= MAX_SLICE_CELLS) return fail(GFT_ERR_INVALID_ARGUMENT, "grid slice too large");
    if (!density || !transmittance || !falloff || !camera_sums || !weight_sums || !density_grad ||
        !transmittance_grad)
        return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    gft_status st;
    if ((st = check_aligned({density, transmittance, falloff, weight_sums, density_grad, transmittance_grad}, 4)) !=
            GFT_OK ||
        (st = check_aligned({camera_sums}, 8)) != GFT_OK)
        return st;
    if (!launch_light_compose_factored_grad_cameras(density, transmittance, falloff, camera_sums, weight_sums,
                                                    num_cameras, (int)shape[0], dims_of(shape), density_grad,
                                                    transmittance_grad, as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_light_compose_factored_grad(const float* density, const float* transmittance, const float* falloff,
                                           const int64_t shape[5], int32_t output_layout,
                                           const float* projected_grad, float* density_grad,
                                           float* transmittance_grad, void* stream) {
    std::string why;
    if (!single_channel_grid(shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!layout_ok(output_layout)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid layout");
    if (voxels(dims_of(shape)) >= MAX_SLICE_CELLS) return fail(GFT_ERR_INVALID_ARGUMENT, "grid slice too large");
    if (!density || !transmittance || !falloff || !projected_grad || !density_grad || !transmittance_grad)
        return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    gft_status st;
    if ((st = check_aligned({density, transmittance, falloff, density_grad, transmittance_grad}, 4)) != GFT_OK ||
        (st = check_aligned({projected_grad}, 8)) != GFT_OK)
        return st;
    if (!launch_light_compose_factored_grad(density, transmittance, falloff, projected_grad, (int)shape[0],
                                            dims_of(shape), output_layout ? LAYOUT_BRICK : LAYOUT_FLAT, density_grad,
                                            transmittance_grad, as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_light_compose_grad(const float* density, const float* transmittance, const float* light_color,
                                  const int64_t shape[5], float ambient, float scale, int32_t output_layout,
                                  const float* output_grad, float* density_grad, float* transmittance_grad,
                                  void* stream) {
    std::string why;
    if (!single_channel_grid(shape, why)) return fail(GFT_ERR_INVALID_ARGUMENT, why);
    if (!layout_ok(output_layout)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid layout");
    if (voxels(dims_of(shape)) >= MAX_SLICE_CELLS) return fail(GFT_ERR_INVALID_ARGUMENT, "grid slice too large");
    if (!density || !transmittance || !light_color || !output_grad || !density_grad || !transmittance_grad)
        return fail(GFT_ERR_INVALID_ARGUMENT, "tensor pointer is NULL");
    gft_status st;
    if ((st = check_aligned({density, transmittance, light_color, density_grad, transmittance_grad}, 4)) != GFT_OK ||
        (st = check_aligned({output_grad}, 16)) != GFT_OK)
        return st;
    if (!launch_light_compose_grad(density, transmittance, light_color, output_grad, (int)shape[0], dims_of(shape),
                                   ambient, scale, output_layout ? LAYOUT_BRICK : LAYOUT_FLAT, density_grad,
                                   transmittance_grad, as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

size_t gft_image_loss_workspace_size(int64_t pixels) {
    if (pixels <= 0) return 0;
    return align256(sizeof(float) * image_loss_ws_floats(pixels));
}

static gft_status image_loss_args(const float* image, const float* target, const float background[3], int64_t pixels,
                                  int32_t tonemap, const void* out) {
    if (pixels <= 0) return fail(GFT_ERR_INVALID_ARGUMENT, "pixel count must be positive");
    if (pixels > (int64_t(1) << 40)) return fail(GFT_ERR_INVALID_ARGUMENT, "pixel count too large");
    if (!enum_in(tonemap, GFT_TONEMAP_NONE, GFT_TONEMAP_NORMALIZE)) return fail(GFT_ERR_INVALID_ARGUMENT, "invalid tonemap");
    if (!image || !target || !background || !out) return fail(GFT_ERR_INVALID_ARGUMENT, "pointer is NULL");
    return GFT_OK;
}

gft_status gft_image_loss_tonemap(const float* image, const float* target, const float background[3], int64_t pixels,
                                  int32_t tonemap, float* loss, void* workspace, size_t workspace_bytes,
                                  void* stream) {
    gft_status st = image_loss_args(image, target, background, pixels, tonemap, loss);
    if (st != GFT_OK) return st;
    if (workspace == nullptr || workspace_bytes < gft_image_loss_workspace_size(pixels))
        return fail(GFT_ERR_WORKSPACE, "image loss workspace too small");
    if ((st = check_aligned({image}, 16)) != GFT_OK || (st = check_aligned({target, loss}, 4)) != GFT_OK ||
        (st = check_workspace_aligned(workspace)) != GFT_OK)
        return st;
    if (!launch_image_loss(image, target, pixels, background, tonemap, reinterpret_cast<float*>(workspace), loss,
                           as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_image_loss(const float* image, const float* target, const float background[3], int64_t pixels,
                          float* loss, void* workspace, size_t workspace_bytes, void* stream) {
    return gft_image_loss_tonemap(image, target, background, pixels, GFT_TONEMAP_NONE, loss, workspace,
                                  workspace_bytes, stream);
}

gft_status gft_image_loss_tonemap_grad(const float* image, const float* target, const float background[3],
                                       int64_t pixels, int32_t tonemap, const float* loss_grad, float* image_grad,
                                       void* workspace, size_t workspace_bytes, void* stream) {
    gft_status st = image_loss_args(image, target, background, pixels, tonemap, image_grad);
    if (st != GFT_OK) return st;
    if (!loss_grad) return fail(GFT_ERR_INVALID_ARGUMENT, "pointer is NULL");
    if (tonemap == GFT_TONEMAP_NORMALIZE) {
        if (workspace == nullptr || workspace_bytes < gft_image_loss_workspace_size(pixels))
            return fail(GFT_ERR_WORKSPACE, "image loss workspace too small");
        if ((st = check_workspace_aligned(workspace)) != GFT_OK) return st;
    }
    if ((st = check_aligned({image, image_grad}, 16)) != GFT_OK || (st = check_aligned({target, loss_grad}, 4)) != GFT_OK)
        return st;
    if (!launch_image_loss_grad(image, target, pixels, background, tonemap, reinterpret_cast<float*>(workspace),
                                loss_grad, image_grad, as_stream(stream)))
        return GFT_ERR_CUDA;
    return GFT_OK;
}

gft_status gft_image_loss_grad(const float* image, const float* target, const float background[3], int64_t pixels,
                               const float* loss_grad, float* image_grad, void* stream) {
    return gft_image_loss_tonemap_grad(image, target, background, pixels, GFT_TONEMAP_NONE, loss_grad, image_grad,
                                       nullptr, 0, stream);
}

}  // extern "C"
