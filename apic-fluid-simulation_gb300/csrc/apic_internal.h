// apic_internal.h — device state of one scene and the launchers of each stage.
//
// Layout in HBM (one scene):
//   particles   9 SoA float arrays of npad = 8*ceil(N/8) lanes (+ a second set
//               for the Morton permutation), i.e. the reference's AoSoA-8
//               `Vec2x8` chunks (src/apic.rs:757-767) unrolled to SoA so that a
//               warp reads 128 contiguous bytes per field;
//   MAC faces   u: (W+1)*H, v: W*(H+1) floats, valid flags as bytes;
//   cells       density / smoothed / pressure: W*H floats;
//   bit masks   u32 words (count rounded to even so a u64 view matches the
//               reference's Vec<u64> masks bit for bit);
//   levels      per multigrid level: fluid mask words, the ascending list of
//               non-zero mask words ("segments": 32 consecutive cells each,
//               one warp per segment), and the pressure system in the
//               reference's padded layout (index = cell + width, size
//               cells + 2*width) so +-1 / +-width stencil reads stay in bounds.
// All per-substep scalars (dt, time, PCG coefficients, counts) live in a
// device-resident `Ctl` block so kernels never need host round trips.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/apic_gpu.h"

namespace apic {

constexpr int kMaxLevels = 20;        // base + coarse levels
#ifndef APIC_SEG_BLOCK
#define APIC_SEG_BLOCK 256
#endif
constexpr int kSegBlock = APIC_SEG_BLOCK;  // threads per block of segment kernels
constexpr int kSegWarps = kSegBlock / 32;
constexpr int kMaxRedBlocks = 152 * (2048 / kSegBlock);  // one full wave on 152 SMs: grid of reduction kernels
constexpr int kSortTile = 2048;       // keys per block in the radix sort
constexpr int kSortThreads = 256;
constexpr int kMaxDigitBits = 10;     // widest radix-sort digit (1024 buckets)

// Device-resident control block of one scene.
struct Ctl {
    // substep loop (src/apic.rs:2429-2474)
    float frame_dt;
    float t;
    float dt;
    float prev_dt;
    float cfl_cs;           // cfl * cell_size (src/apic.rs:2436)
    uint32_t timestamp;
    uint32_t substeps;
    uint32_t go;            // 1 while another substep is due
    uint32_t sort_now;      // sort on this substep
    uint32_t flags;         // APIC_UPDATE_* of the running update
    uint32_t vmax_bits;     // max |v| over all lanes, as float bits
    uint32_t status;        // error bits (kStatus*)
    uint32_t nonfinite;     // non-finite particle lanes after G2P
    uint32_t has_ext;       // external force fields may be non-zero
    uint32_t has_post;      // post force fields may be non-zero
    // pressure solve
    float gamma;            // r.z of the current iteration (FP32, as the reference)
    float alpha;
    float beta;
    uint32_t beta_valid;    // beta belongs to this solve (the search direction is z + beta s)
    uint32_t delta_stop;    // k_pcg_update found s.Ap unusable; the next kernel turns it into pcg_done
    unsigned long long solve_t0;  // %globaltimer at the start of the running solve (ns)
    unsigned long long solve_ns;  // summed solve time of this update (ns)
    uint32_t max_r_bits;    // max |r| (float bits)
    uint32_t pcg_done;
    uint32_t pcg_iters;
    uint32_t pcg_iters_total;
    uint32_t not_converged;
    uint32_t refinements;
    uint32_t inner_cap;     // iteration cap of the running (inner) solve
    uint32_t used_iters;    // iterations used by the refinement loop so far
    uint32_t refinements_total;  // refinements summed over the substeps of an update
    uint32_t cond;          // last loop decision of a control kernel (eager runs read it)
    uint32_t sorted;        // the update ran the Morton sort
    double dgamma;          // FP64 copies for the relative-tolerance modes
    double bnorm2;          // ||b||^2 of the running solve
    double rnorm2;          // ||r||^2 of the recursive residual
    double true_rel;        // ||b - A p|| / ||b|| (FP64)
    double target_rel;      // tolerance of the running inner solve
    // fluid bookkeeping, per level (0 = base)
    uint32_t seg_count[kMaxLevels];
    uint32_t fluid_cells;   // base fluid cells (src/apic.rs:1461-1485)
    uint32_t last_fluid;    // padded index of the last base fluid cell
    uint32_t pad_count;     // duplicates padding the base list to a multiple of 8
    uint32_t red_counter;   // last-block-done counter of the reductions
    uint32_t pcg_on;        // the PCG loop goes on (a batched solve gates its phases on it)
    float b_rz;             // batched solve: the iteration's r.z sum (from the last V-cycle's parts)
    float b_sap;            // batched solve: the iteration's s.Ap sum
};

enum : uint32_t {
    kStatusNonfinite = 1u,
    kStatusBadStep = 2u,
    kStatusP2gLayout = 8u,  // a particle's staggered stencil left the bins P2G searches (never expected)
    kStatusBounds = 16u,    // checked build (APIC_BOUNDS_CHECK): an index left its buffer
};

struct Level {
    uint32_t w = 0, h = 0, cells = 0;
    int wshift = -1;        // log2 w, or -1 when w is not a power of two
    uint32_t words = 0;     // u32 mask words (even)
    uint32_t padded = 0;    // cells + 2w rounded up to 8
    uint32_t* fluid = nullptr;
    uint32_t* seg = nullptr;
    float* diag = nullptr;
    float* inv_diag = nullptr;
    float* px = nullptr;
    float* py = nullptr;
    float* res = nullptr;
    float* err = nullptr;
};

// Particle field order, matching apic_field ids 0..8.
enum { PX = 0, PY, VX, VY, CUX, CUY, CVX, CVY, TR, NPF };

// Device-resident table of the particle arrays.  The Morton permutation
// gathers `f` into `alt` and then swaps the two tables on the device, so a
// captured CUDA graph never holds a stale particle pointer.
struct PartPtrs {
    float* f[NPF];
    float* alt[NPF];
};

struct RenderBuffers;  // render.cu

// Splatting parameters as the kernels use them (render.cu).
struct RenderParamsDev {
    uint32_t width, height;     // frame in pixels
    uint32_t ntx, nty, ntiles;  // 16 x 16 pixel tiles
    float fw, fh;               // width, height as floats
    float scale, margin, radius, size;  // pixels per unit, out-of-bounds margin, disc radius, 2 * radius
    float tex_scale;                    // texels per pixel: 32 / size
    float pick_x, pick_y, pick_r2;      // pick centre and squared radius (< 0: no pick)
    uint32_t bg;                // clear colour, RGBA8 little-endian
};

struct RenderResult {
    uint32_t valid, nan, oob;
    int64_t picked;
    uint32_t kernels;
};

struct Scene {
    uint32_t W = 0, H = 0, cells = 0;
    float dx = 0;
    apic_world_props props{};
    uint32_t n = 0, nchunks = 0, npad = 0;
    uint32_t part_cap = 0;                 // allocated lanes
    float* part[NPF] = {};                 // allocation A of each field
    float* part_alt[NPF] = {};             // allocation B of each field
    PartPtrs* pp = nullptr;                // device table: which allocation is current
    float* vec_stage = nullptr;            // Vec2x8 staging for host reads (allocated on first use)
    uint32_t vec_stage_floats = 0;
    // pipelined host I/O (apic_stage_field / apic_read_vec2x8_async): an
    // upload and a download stream; two device buffers per staged force
    // field (ext u, ext v, post u, post v) and per Vec2x8 field pair, each
    // with an event when filled and one when its contents were used
    cudaStream_t up_stream = nullptr, down_stream = nullptr;
    float* stage_buf[4][2] = {};
    cudaEvent_t stage_ready[4][2] = {}, stage_used[4][2] = {};
    int stage_next[4] = {};
    int stage_pending[4] = {-1, -1, -1, -1};
    float* read_buf[4][2] = {};
    uint64_t read_floats[4][2] = {};
    cudaEvent_t read_packed[4][2] = {}, read_done[4][2] = {};
    int read_next[4] = {};
    uint32_t* keys = nullptr;
    uint32_t* vals = nullptr;
    uint32_t* keys_alt = nullptr;
    uint32_t* vals_alt = nullptr;
    uint32_t* sort_hist = nullptr;         // sort_hist_words(n)
    uint32_t* sort_scan_tmp = nullptr;
    // P2G binning: (cell of the density stencil's base, slot) pairs sorted by
    // cell, and each cell's run [bin_lo, bin_hi) in the sorted pairs
    uint32_t *bin_keys = nullptr, *bin_vals = nullptr, *bin_keys_alt = nullptr, *bin_vals_alt = nullptr;
    uint32_t *bin_lo = nullptr, *bin_hi = nullptr;

    uint32_t uf = 0, vf = 0;               // face counts
    float *u = nullptr, *v = nullptr, *u_alt = nullptr, *v_alt = nullptr;
    uint8_t *valid_u = nullptr, *valid_v = nullptr, *valid_u_alt = nullptr, *valid_v_alt = nullptr;
    float *acc_u = nullptr, *acc_uw = nullptr, *acc_v = nullptr, *acc_vw = nullptr;
    float *ext_u = nullptr, *ext_v = nullptr, *post_u = nullptr, *post_v = nullptr;
    uint32_t *u_open = nullptr, *v_open = nullptr;
    uint32_t u_open_words = 0, v_open_words = 0;

    float *density = nullptr, *sm_a = nullptr, *sm_b = nullptr, *pressure = nullptr;
    uint32_t* obstacle = nullptr;
    float *search = nullptr, *ap = nullptr;   // base, padded layout
    float* corr = nullptr;                    // correction of an inner solve (padded)
    double* p64 = nullptr;                    // FP64 pressure of the refinement loop (padded)
    double* b64 = nullptr;                    // FP64 right-hand side (padded)
    bool p64_valid = false;                   // p64 holds the refined pressure (mixed mode)
    bool warm_start = true;                   // mixed mode: start from the previous solve's FP64 pressure
    int p2g_order = 0;                        // APIC_OPT_P2G_ORDER (0: follow the solver mode)

    int nlevels = 0;                          // including the base (levels[0])
    int tail_first = 0;                       // first level of the shared-memory tail (nlevels: none)
    size_t tail_smem = 0;
    Level lv[kMaxLevels];
    float *cg_s = nullptr, *cg_ap = nullptr, *cg_r = nullptr;  // coarsest level CG

    Ctl* ctl = nullptr;                       // device
    Ctl* ctl_host = nullptr;                  // pinned mirror
    double* partials = nullptr;               // kPartialDoubles doubles (block partials of reductions)
    float* exact_parts = nullptr;             // chunk sums of the reference-order s.Ap (cells / 8192 + 1)
    uint32_t* seg_pre = nullptr;              // fluid cells before each base segment (words + 1)
    uint32_t* scan_tmp = nullptr;             // compaction block counts
    uint32_t scan_tmp_len = 0;

    cudaStream_t stream = nullptr;
    int priority = 0;                         // stream priority: levels above the lowest
    cudaStream_t cap_stream = nullptr;        // stream used to record graphs
    cudaGraphExec_t update_exec = nullptr;    // whole Apic::update as one graph
    uint64_t graph_version = 0;               // bumped whenever recorded graphs go stale
    int device = 0;                           // the CUDA device the scene lives on
    bool batched = false;                     // the last update ran inside a joint batch
    uint32_t kn_bsort = 0, kn_bstep = 0;      // ... its own kernels there: sort, one substep
    bool use_pdl = true;                      // programmatic dependent launch inside the PCG loop
    // levels [dsm_first, dsm_tail) of the V-cycle held in a cluster's
    // distributed shared memory, dsm_tail.. in CTA 0 (dsm_first == nlevels: none)
    bool use_dsm = true;
    int dsm_first = 0, dsm_tail = 0;
    size_t dsm_smem = 0;
    uint32_t dsm_off = 0;
    // kernel nodes per execution of each graph body (launch accounting)
    uint32_t kn_top = 0, kn_sort = 0, kn_loop = 0, kn_pcg = 0, kn_refine = 0;
    int solver_mode = APIC_SOLVER_REFERENCE;
    // WHILE node of the PCG loop being recorded: the kernel that runs the
    // residual's exit test also sets the loop condition (pcg_set_cond false:
    // host-driven loops of profiling runs)
    cudaGraphConditionalHandle pcg_h = 0;
    uint32_t pcg_cap = 0;
    int pcg_dyn_cap = 0;
    bool pcg_set_cond = false;
    float rel_tol = 1e-6f;
    uint32_t max_iter = 500;
    bool vmax_valid = false;
    bool world_ready = false;
    bool has_ext = false, has_post = false;

    // measurement
    bool profiling = false;
    double stage_ms[APIC_STAGE_COUNT] = {};
    uint64_t stage_launches[APIC_STAGE_COUNT] = {};
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;

    apic_step_stats stats{};
    RenderBuffers* render = nullptr;          // splatting buffers (allocated on the first frame)
};

// ---- launchers (each enqueues on s.stream) --------------------------------
// sort.cu
cudaError_t launch_sort(Scene& s);
// Exclusive scan of data[0..n) in place; tmp holds div_up(n, 1024) words.
cudaError_t exclusive_scan_u32(uint32_t* data, uint32_t n, uint32_t* tmp, cudaStream_t st);
// Block partials of the PCG loop's split reductions, in Scene::partials after
// the 2 * kMaxRedBlocks doubles of the single-kernel reductions: s.Ap (one
// float2 per block), the residual's sum of squares and max (one float4) and
// r.z (one float2).
constexpr int kPartialDoubles = 6 * kMaxRedBlocks;
inline float2* part_sap(const Scene& s) { return reinterpret_cast<float2*>(s.partials + 2 * kMaxRedBlocks); }
inline float4* part_res(const Scene& s) { return reinterpret_cast<float4*>(s.partials + 3 * kMaxRedBlocks); }
inline float2* part_rz(const Scene& s) { return reinterpret_cast<float2*>(s.partials + 5 * kMaxRedBlocks); }

// The mixed-precision solve starts from the FP64 pressure that the previous
// solve left in p64 (zeroed whenever the particle set is replaced).
inline int warm_start(const Scene& s) { return s.warm_start && s.solver_mode == APIC_SOLVER_REL_MIXED ? 1 : 0; }
// P2G adds each face's contributions in the reference's order (else in cell order).
inline bool p2g_reference_order(const Scene& s) {
    return s.p2g_order == 1 || (s.p2g_order == 0 && s.solver_mode == APIC_SOLVER_REFERENCE);
}
// The reference solver mode reproduces the reference's FP32 reduction orders
// (dot_product's eight lane sums, apply_matrix_and_dot's 8192-cell chunks,
// the coarsest CG's serial sums), so its pressure is bit-identical to the
// oracle's; the relative modes reduce in FP64 / double-float instead.
inline bool coarse_cg_exact(const Scene& s) { return s.solver_mode == APIC_SOLVER_REFERENCE; }
// render.cu: splat the particles into the scene's frame and wait for it
cudaError_t render_frame(Scene& s, const RenderParamsDev& p, RenderResult* out);
const uint32_t* render_frame_ptr(const Scene& s, uint32_t* width, uint32_t* height);
void free_render(Scene& s);
cudaError_t radix_sort_pairs_in(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, uint32_t* hist,
                                uint32_t* scan_tmp, uint32_t n, int bits, cudaStream_t st);
// Stable LSD sort with digits of up to kMaxDigitBits bits; the sorted pairs
// stay where the last pass wrote them (*keys_out / *vals_out: keys/vals or
// keys_alt/vals_alt).  hist: sort_hist_words(n), scan_tmp: sort_scan_words(n).
// status: where the checked build (APIC_BOUNDS_CHECK) records an index outside
// its buffer (may be null).
cudaError_t radix_sort_pairs(uint32_t* keys, uint32_t* vals, uint32_t* keys_alt, uint32_t* vals_alt, uint32_t* hist,
                             uint32_t* scan_tmp, uint32_t n, int bits, cudaStream_t st, bool pdl,
                             uint32_t** keys_out, uint32_t** vals_out, uint32_t* status = nullptr);
bool radix_sort_in_alt(int bits);     // radix_sort_pairs over `bits` bits ends in the alt buffers
uint32_t sort_hist_words(uint32_t n);
uint32_t sort_scan_words(uint32_t n);
bool sort_result_in_alt(const Scene& s);  // where launch_sort leaves the Morton-sorted pairs
int morton_key_bits(uint32_t width, uint32_t height);
// runtime.cu: record the calling thread's last error text (apic_last_error)
void set_last_error(const char* msg);
// runtime.cu: unique id of the CUDA context current on the calling thread
// (the runtime's primary context is made current first if none is).  Ids are
// never reused within a process, so caches of device addresses keyed by it
// cannot outlive their context (cudaDeviceReset, a caller's own context).
cudaError_t current_context_key(unsigned long long* key);
// particles.cu
cudaError_t launch_p2g(Scene& s);
cudaError_t launch_g2p(Scene& s);
cudaError_t launch_vmax(Scene& s);
cudaError_t launch_permute(Scene& s, const uint32_t* sorted_vals);
cudaError_t launch_pack_vec2x8(Scene& s, int which, float* out);  // which: 0 pos, 1 vel, 2 C_u, 3 C_v
// grid.cu
cudaError_t launch_finalize_faces(Scene& s, bool forces, bool gravity);
cudaError_t launch_base_lists(Scene& s);
cudaError_t launch_external_forces(Scene& s);
cudaError_t launch_build_pressure(Scene& s);
cudaError_t launch_multilevel(Scene& s);
cudaError_t launch_gradient(Scene& s, bool post);
cudaError_t launch_post_forces(Scene& s);
cudaError_t launch_extrapolate(Scene& s);
cudaError_t launch_smoothed_view(Scene& s, float* out);
cudaError_t launch_level_lists(Scene& s, int level);
// solver.cu: the solve is recorded into graphs (apic_graph.h: build_solve)
// solver.cu: the same solve launched kernel by kernel with host loop control
// (profiling runs, so every kernel is a separate launch)
cudaError_t run_solve_eager(Scene& s);
// vcycle.cu
void plan_vcycle(Scene& s);     // pick the coarse levels that run in one CTA / one cluster
// vcycle_dsm.cu
void plan_vcycle_dsm(Scene& s);
void launch_vcycle_dsm(Scene& s, cudaStream_t st);
// z = M^-1 r on s.stream; base_red_done: the base level's first red sweep
// was already written (by k_pcg_update); rz_mode >= 0: the last kernel also
// reduces r.z and finishes the PCG iteration for that solver mode (returns
// false when this V-cycle form cannot, and the caller must).
// residual_exit: the first kernel also runs the PCG residual's exit test
// (k_smooth_exit; with base_red_done, rz_mode = the solver mode).
bool enqueue_vcycle(Scene& s, bool base_red_done = false, int rz_mode = -1, bool residual_exit = false);
// runtime.cu
cudaError_t launch_plan_first(Scene& s);
cudaError_t launch_advance(Scene& s);

// runtime.cu: Apic::update split in two, so several scenes can be enqueued
// before any is waited on (apic_update_batch, the request server)
int update_launch(apic_handle* h, uint32_t flags, float frame_dt);
int update_begin(apic_handle* h, uint32_t flags, float frame_dt);  // update_launch before the substep loop
int update_end(apic_handle* h);                                    // ... and after it
Scene& scene_of(apic_handle* h);
cudaError_t scene_pre_solve(Scene& s);   // the substep's stages before the pressure solve
cudaError_t scene_post_solve(Scene& s);  // ... and after it
// batch.cu: apic_update_batch with the solves as one launch per phase
struct BatchShape {
    uint32_t chunk_segs, block_group;
};
// The form of one apic_update_batch call, as the batch tuner planned it.
struct BatchTicket {
    uint64_t key = 0;   // makeup of the batch
    int step = -1;      // the tuner's step this call measures (-1: none)
    int joint = 0;      // 1: joint form with `shape`; 0: a stream per scene
    BatchShape shape{64, 4};
};
bool batch_eligible(apic_handle* const* handles, uint32_t count);
int update_batch_joint(apic_handle* const* handles, uint32_t count, uint32_t flags, float frame_dt, BatchShape shape,
                       int* rc);
void batch_note_streams(uint32_t count);
void batch_choose(apic_handle* const* handles, uint32_t count, bool force_joint, BatchTicket* tk);
void batch_record(const BatchTicket& tk, double wall_ms, uint64_t iterations);
void batch_release_scene(const Scene* s);
int create_scene(uint32_t width, uint32_t height, float cell_size, const apic_world_props* props,
                 bool default_particles, apic_handle** out);
int update_finish(apic_handle* h);
int update_prepare(apic_handle* h);       // build the update graph ahead of the first update
cudaStream_t scene_stream(apic_handle* h);

// helpers shared by the launchers
inline uint32_t div_up(uint64_t a, uint64_t b) { return uint32_t((a + b - 1) / b); }

// Launch kern on st.  pdl: programmatic dependent launch, so the kernel's
// CTAs are scheduled while the previous kernel on the stream drains instead
// of after it; the kernel must call pdl_wait() (apic_device.cuh) before it
// reads anything the previous kernel writes.  Only for a launch whose
// predecessor on the stream (within the same capture) is a kernel.
template <typename... KArgs, typename... Args>
inline cudaError_t launch(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                          Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}
uint32_t seg_grid(uint32_t words);     // blocks for a segment kernel over `words` words

}  // namespace apic
