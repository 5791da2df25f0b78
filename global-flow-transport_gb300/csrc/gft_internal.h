// Host-side declarations shared by the kernel translation units and the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "gft.h"
#include "gft_common.cuh"

namespace gft {

// Up to this many (input batch, camera) pairs travel by value in one launch's
// parameter block; more pairs are split into several launches.
constexpr int MAX_PAIRS = 16;

struct PairTable {
    CamX cam[MAX_PAIRS];
    int in_batch[MAX_PAIRS];  // batch slice of the input grid
    int out_slot[MAX_PAIRS];  // slot in the output's [N * V] leading dims
    // raymarch only: each pair's image (width, height, depth samples), its first
    // output pixel, and the first block of its pixel tiles in this launch
    // (tile0[n] = blocks of the launch), so that cameras of different image
    // sizes share one launch
    int rw[MAX_PAIRS], rh[MAX_PAIRS], rd[MAX_PAIRS];
    int64_t pix0[MAX_PAIRS];
    int64_t smp0[MAX_PAIRS];  // raymarch sample store: first float of each pair
    int tile0[MAX_PAIRS + 1];
    int pair_base;            // global index of pair 0 of this launch
    int n;                    // pairs in this launch
};

// One (input batch, camera) pair of a launcher loop (e.g. raymarch_grid.cu.cc:262-291).
struct Pair {
    CamX cam;
    int in_batch;
    int out_slot;
    int camera;
    int W = 0, H = 0, D = 0;  // raymarch image of the pair
    int64_t pix0 = 0;         // raymarch: first output pixel of the pair
};

// Builds the (batch, camera) pairs with MV = V*M and the inverses computed in
// double on the host.  separate_camera_batch=false pairs batch b with camera b.
std::vector<Pair> make_pairs(const float* M, int num_m, const float* V, const float* P, const float* F,
                             int num_cameras, int batch, bool separate_camera_batch);
std::vector<PairTable> make_tables(const std::vector<Pair>& pairs);

// Mip pyramid of one batch slice: level 0 is the input, levels 1..L live in a
// workspace as fp32 (dims >> m per level).
constexpr int MAX_MIPS = 15;
struct MipSet {
    const float* lvl[MAX_MIPS + 1];
    Dims dims[MAX_MIPS + 1];
    int levels;  // L
    // Optional occupancy of level 0 per 8^3-voxel block, grown by the
    // footprint of every level's fetch (occupancy_radius): 0 = every sample
    // whose (clamped) floor position lies in the block reads only zeros.
    const uint8_t* occ = nullptr;
    Dims occ_dims{0, 0, 0};
};
int usable_mip_levels(Dims d, int num_mips);
size_t mip_workspace_floats(Dims d, int levels, int C);
// Occupancy map of a sampled grid (SampleGridTransform, forward coordinate
// modes): bytes per batch slice, and the map build (raw blocks into `raw`,
// grown into set->occ) for one slice.
constexpr int OCC_BLOCK_SHIFT = 3;
size_t occupancy_bytes(Dims d);
bool launch_occupancy(const void* input, int dtype, int C, Dims d, int levels, uint8_t* raw, uint8_t* grown,
                      cudaStream_t s, MipSet* set);

// Launch-configuration knobs (gft_set_knob; values checked there): read when
// a launch is issued, so a captured graph keeps the values of its capture.
int knob_value(int knob);
int sm_count();  // SMs of the current device
// Blocks of a raymarch launch over `tiles` pixel tiles under
// GFT_KNOB_RAYMARCH_BLOCKS_PER_SM.
unsigned raymarch_blocks(int tiles);
// ... of the weight pass (GFT_KNOB_WEIGHTS_BLOCKS_PER_SM; 0: raymarch_blocks)
unsigned weights_blocks(int tiles);
// Creates the library's side stream of the current device (the pipelined
// weight pass) ahead of any stream capture.
bool prepare_side_stream();

// error helpers
void set_error(const std::string& msg);
bool cuda_ok(cudaError_t e, const char* what);
// Records n kernel launches in the process-wide launch counter and checks the
// launch status.
bool launched(int n, const char* what);

// launchers ------------------------------------------------------------------
// Two projections of a 4-channel gradient: (a . g, b . g).
struct ChanProj {
    float a[4], b[4];
};

struct RaymarchArgs {
    const void* input;
    int dtype;
    int N, C;
    Dims din;
    int D, H, W;
    int filter, boundary, blend;
    int layout = LAYOUT_FLAT;  // cell layout of the input and its gradient
    int n_slots;  // output slots = N * (separate ? V : 1)
    // Sample store (LINEAR only): the forward writes the samples it blends, the
    // adjoint reads them instead of re-sampling (store.samples != nullptr).
    struct Store {
        float* samples = nullptr;     // the pool: cells of C floats
        uint32_t capacity = 0;        // cells of the pool
        unsigned long long* count = nullptr;  // pool cells handed out (in chunks)
        uint32_t* words = nullptr;    // per pair, tile, step and warp: the lanes with a non-zero sample
        uint32_t* first = nullptr;    // per pair, tile, step and warp: the step's first pool cell, or
                                      // 0xffffffff where the pool was full
        uint8_t* occ = nullptr;       // per input slice and 4^3-voxel block: 0 = no non-zero voxel in
                                      // the block grown by one voxel at its upper faces
        uint8_t* dist = nullptr;      // per slice and block: Chebyshev distance (in blocks, capped) to the
                                      // nearest occupied block; 0 = occupied
        uint8_t* dist_tmp = nullptr;  // scratch of the distance passes
        int nbx = 0, nby = 0, nbz = 0;
    } store;
    // Deterministic adjoint (GFT_GRAD_DETERMINISTIC): integer accumulation in
    // the workspace after the reciprocal weight sums (raymarch_det_bytes).
    bool det = false;
    unsigned long long* det_acc = nullptr;  // set by launch_raymarch_bwd
    const float* det_scale = nullptr;
    // Projected adjoint (C == 4, brick layout; float or deterministic): the gradient
    // holds (proj.a . g, proj.b . g) per cell instead of the 4 channels of g.
    bool project = false;
    ChanProj proj = {};
    // With project, GFT_GRAD_REFERENCE: per pair the unnormalised projected
    // sums (the gradient, [pairs][cells][2]) and the weight sums (the
    // workspace) from one pass; the caller divides.
    bool camera_sums = false;
};
// Workspace bytes of the deterministic adjoint for `pairs` (batch, camera) pairs.
size_t raymarch_det_bytes(int N, int C, Dims din, size_t pairs);
// Bytes of the sample store of these pairs (samples, ballot words,
// occupancy map of the N input slices), and its parts at `base`.
// a store whose pool holds every sample the launch could store, and the part
// before the pool (a store of that size keeps no samples)
size_t raymarch_store_bytes(const std::vector<Pair>& pairs, int C, int N, Dims din);
size_t raymarch_store_min_bytes(const std::vector<Pair>& pairs, int N, Dims din);
RaymarchArgs::Store raymarch_store_layout(void* base, size_t bytes, const std::vector<Pair>& pairs, int C, int N,
                                          Dims din);
// Fills a.store.occ from the input (before the storing forward).
bool launch_raymarch_occupancy(const RaymarchArgs& a, cudaStream_t s);
bool launch_raymarch_fwd(const RaymarchArgs& a, const std::vector<Pair>& pairs, float* out, cudaStream_t s);
// Per-pair reciprocal weight sums of the reference-normalised adjoint (pass 1).
bool launch_raymarch_weights(const RaymarchArgs& a, const std::vector<Pair>& pairs, float* ws_cnt, cudaStream_t s);
// The deterministic adjoint's weight sums into its workspace layout (integer
// sums, their largest value and the reciprocals), for a later gradient call
// with GFT_GRAD_WEIGHTS_READY | GFT_GRAD_DETERMINISTIC.
bool launch_raymarch_weights_det(const RaymarchArgs& a, const std::vector<Pair>& pairs, float* ws_cnt,
                                 cudaStream_t s);
// weights_ready: ws_cnt already holds the pass-1 reciprocals of the same geometry.
bool launch_raymarch_bwd(const RaymarchArgs& a, const std::vector<Pair>& pairs, const float* out,
                         const float* dout, bool exact, bool weights_ready, float* grad, float* ws_cnt,
                         cudaStream_t s);

bool launch_build_mips(const void* input, int dtype, int C, Dims d, int levels, float* ws, cudaStream_t s,
                       MipSet* set_out);

struct SampleArgs {
    const void* input;
    int dtype;
    int N, C;
    Dims din, dout;
    int filter, boundary, mip_mode, levels;
    float mip_bias, cco;
    int coord_mode;
};
bool launch_sample_transform_fwd(const SampleArgs& a, const std::vector<Pair>& pairs, const MipSet* mips_per_batch,
                                 float* out, cudaStream_t s);
bool launch_sample_transform_bwd(int N, int C, Dims din, Dims dout, int boundary, int coord_mode, float cco,
                                 const std::vector<Pair>& pairs, const float* dy, bool exact, float* grad,
                                 unsigned int* count, cudaStream_t s);

struct LutArgs {
    const void* input;
    int dtype;
    int N, C;
    Dims din, dout;
    int n_lut;  // V
    int filter, boundary, mip_mode, levels;
    float mip_bias, cco;
    int separate, relative, normalized;
};
bool launch_lut_fwd(const LutArgs& a, const float* lut, const MipSet* mips_per_batch, float* out, cudaStream_t s);
bool launch_lut_bwd(const LutArgs& a, const float* input, const float* lut, const float* dy, bool exact,
                    float* grad, float* lut_grad, unsigned int* count, cudaStream_t s);
bool launch_lod_transform(Dims din, Dims dout, const std::vector<Pair>& pairs, bool inverse, float* out,
                          cudaStream_t s);

bool launch_blend_fwd(const float* in, int N, int C, Dims d, int mode, bool keep_dims, float* out, cudaStream_t s);
bool launch_blend_bwd(const float* dy, const float* y, const float* x, int N, int C, Dims d, int mode,
                      bool keep_dims, bool exact, float* gx, cudaStream_t s);

struct AdvectArgs {
    const void* density;
    int dtype;
    int N, C;
    Dims d;
    const float *vx, *vy, *vz;
    float dt;
    int order, clamp, boundary;
    bool det = false;  // deterministic adjoint: int64 scatters, workspace advect_det_ws_bytes
};
size_t advect_det_ws_bytes(size_t voxels, size_t channels);
bool launch_advect_fwd(const AdvectArgs& a, float* out, float* ws, cudaStream_t s);
// forward_ready: ws starts with the semi-Lagrangian grid of launch_advect_fwd
// (order 2, N == 1), which is then not recomputed.
bool launch_advect_bwd(const AdvectArgs& a, bool exact, bool forward_ready, const float* dy, float* gd, float* gvx,
                       float* gvy, float* gvz, float* ws, cudaStream_t s);

// pipeline fusions (compose.cu)
bool launch_transmittance(const float* s, int N, Dims d, float* out, cudaStream_t st);
bool launch_transmittance_grad(const float* tr, const float* g, int N, Dims d, float* gs, cudaStream_t st);
// rgb3 != nullptr: color is the per-voxel falloff [V] of a factored light
// (colour = falloff x rgb3), else the colour grid [V, 3].
bool launch_light_compose(const float* dens, const float* tr, const float* color, const float* rgb3, int N, Dims d,
                          float ambient, float scale, int layout, bool bf16, void* out, cudaStream_t st);
// g2: the projected raymarch gradient (P, Q) per cell of layout `layout`.
bool launch_light_compose_factored_grad(const float* dens, const float* tr, const float* fall, const float* g2,
                                        int N, Dims d, int layout, float* gd, float* gt, cudaStream_t st);
// From per-camera sums (ncam pairs per batch slice): g2 [N*ncam][cells][2],
// wsum [N*ncam][cells], brick layout.
bool launch_light_compose_factored_grad_cameras(const float* dens, const float* tr, const float* fall,
                                                const float* g2, const float* wsum, int ncam, int N, Dims d,
                                                float* gd, float* gt, cudaStream_t st);
bool launch_light_compose_grad(const float* dens, const float* tr, const float* color, const float* g, int N, Dims d,
                               float ambient, float scale, int layout, float* gd, float* gt, cudaStream_t st);
int image_loss_blocks(int64_t npix);
size_t image_loss_ws_floats(int64_t npix);
bool launch_image_loss(const float* img, const float* tgt, int64_t npix, const float bkg[3], int tonemap, float* ws,
                       float* loss, cudaStream_t st);
// ws: the workspace of the forward's size (only NORMALIZE uses it)
bool launch_image_loss_grad(const float* img, const float* tgt, int64_t npix, const float bkg[3], int tonemap,
                            float* ws, const float* gloss, float* gimg, cudaStream_t st);

// FP64 check step (check.cu): double-precision camera inverses per pair
struct CamD {
    double mvi[16], pi[16];  // (V M)^-1 and P^-1, row-major
};
struct CheckTable {
    CamD cam[MAX_PAIRS];
    int in_batch[MAX_PAIRS];
    int out_slot[MAX_PAIRS];
    int n;
};
bool launch_transmittance_check(const float* x, const float* tr, int N, Dims d, int stride, double* result,
                                cudaStream_t s);
bool launch_raymarch_check(const void* in, int dtype, int layout, int C, Dims din, const std::vector<CheckTable>& tabs,
                           int W, int H, int D, const float* img, int stride, double* result, cudaStream_t s);

}  // namespace gft
