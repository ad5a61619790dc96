/*
 * apic_gpu.h — C-ABI of the GB300 (sm_103a) APIC/FLIP time step.
 *
 * This is the drop-in boundary for the reference crate's simulation API
 * (fireblade2534/APIC-Fluid-Simulation, `src/apic.rs`).  Every entry point
 * names the reference item it replaces.  A Rust caller binds these with an
 * `extern "C"` block; Python binds them with ctypes.  Only plain pointers,
 * sizes and PODs cross the boundary.
 *
 * Ownership: a handle owns all device memory of one scene.  Host buffers are
 * caller-owned and only copied in or out.  Calls on one handle must be
 * serialised by the caller (the reference's methods take `&mut self`);
 * distinct handles may be driven from different threads.  Each handle runs on
 * its own CUDA stream.
 *
 * Errors: every call returns an `int` status (APIC_OK == 0).  The reference
 * has no error path (it panics; `Cargo.toml:18` sets panic = "abort"); a Rust
 * shim turns a non-zero status into `panic!` to keep the reference signatures.
 */
#ifndef APIC_GPU_H
#define APIC_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define APIC_OK                 0
#define APIC_ERR_INVALID_ARG    1  /* bad size or pointer; odd or <=4 side with particles (src/apic.rs:910 panics there) */
#define APIC_ERR_OOM            2  /* device allocation failed */
#define APIC_ERR_CUDA           3  /* a CUDA runtime call failed; see apic_last_error() */
#define APIC_ERR_TIMEOUT        4  /* a bounded device wait gave up */
#define APIC_ERR_NONFINITE      5  /* non-finite particle state detected */
#define APIC_ERR_NOT_CONVERGED  6  /* warning: a pressure solve hit its iteration cap */
#define APIC_ERR_NO_DEVICE      7  /* no CUDA device visible */
#define APIC_ERR_UNSUPPORTED    8

/* ---- update flags (DebugOptions, src/apic.rs:397-400) ------------------ */
#define APIC_UPDATE_DISABLE_SORT  0x1u  /* DebugOptions::disable_particle_sort */
/* apic_update_batch only: run each scene's whole update on its own stream
 * even where the pressure solves could run as one launch per phase ... */
#define APIC_UPDATE_BATCH_STREAMS 0x2u
/* ... or run the joint form whenever it applies, whatever the batch tuner
 * has found (see apic_batch_info). */
#define APIC_UPDATE_BATCH_JOINT   0x4u

/* ---- pressure-solver modes --------------------------------------------- */
/* Reference semantics (src/apic.rs:1865-1956): absolute max-norm exit at
 * solve_error, 100-iteration cap, 1e-5 early exits on gamma and delta. */
#define APIC_SOLVER_REFERENCE   0
/* FP32 PCG with the same V-cycle preconditioner, run to
 * ||r||_2 <= rel_tol * ||b||_2 (recursively updated residual). */
#define APIC_SOLVER_REL_FP32    1
/* FP64 outer iterative refinement around an FP32 inner PCG; converged on the
 * true residual ||b - A p||_2 <= rel_tol * ||b||_2 evaluated in FP64. */
#define APIC_SOLVER_REL_MIXED   2

/* WorldProperties (src/apic.rs:707-713). */
typedef struct apic_world_props {
    float gravity;
    float border_damping;
    float cfl;          /* the reference recommends 5.0 */
    float solve_error;  /* the reference recommends 1e-5 */
} apic_world_props;

/* Scalars among the reference's public `Apic` fields (src/apic.rs:716-776). */
typedef struct apic_info {
    uint32_t width, height, cells;
    float    cell_size;
    uint32_t num_chunks;      /* ceil(num_particles / 8): AoSoA-8 chunks */
    uint32_t num_particles;
    uint32_t fluid_cells;     /* base-grid fluid cells of the last substep */
    uint32_t timestamp;       /* substeps taken so far (src/apic.rs:2467) */
    float    prev_deltatime;  /* last substep dt (src/apic.rs:2465) */
    uint32_t mg_levels;       /* coarse multigrid levels (src/apic.rs:900-908) */
} apic_info;

/* Statistics of the last apic_update (the reference only shows HUD text,
 * src/main.rs:514-583). */
typedef struct apic_step_stats {
    uint32_t substeps;             /* substeps taken by the last apic_update */
    uint32_t pcg_iterations;       /* PCG iterations of the last substep */
    uint32_t pcg_iterations_total; /* summed over the substeps of the last update */
    uint32_t refinement_steps;     /* outer FP64 refinements of the last substep */
    float    residual_max;         /* max |r| of the recursive residual, last substep */
    float    residual_rel;         /* ||r||_2 / ||b||_2 of the recursive residual */
    double   true_residual_rel;    /* ||b - A p||_2 / ||b||_2 in FP64 (solver modes 1, 2) */
    uint32_t not_converged;        /* substeps whose solve hit its iteration cap */
    uint32_t nonfinite_lanes;      /* NaN/Inf particle lanes after the last G2P */
    uint64_t kernel_launches;      /* kernels the last update's graph launched (0 when profiling) */
    double   solve_ms;             /* device time of the last update's pressure solves, read from
                                      the GPU's global nanosecond timer by the solve's first and
                                      last kernels (0 for the persistent solver) */
} apic_step_stats;

/* ---- field identifiers for apic_read_field / apic_write_field ---------- */
/* Particle fields are SoA float arrays of num_chunks*8 lanes; lanes at and
 * beyond num_particles are the reference's AoSoA padding lanes
 * (src/apic.rs:857-898). */
enum apic_field {
    APIC_F_POS_X = 0, APIC_F_POS_Y, APIC_F_VEL_X, APIC_F_VEL_Y,
    APIC_F_CU_X, APIC_F_CU_Y, APIC_F_CV_X, APIC_F_CV_Y, APIC_F_TRES,
    /* MAC faces (src/apic.rs:736-751): u has (W+1)*H, v has W*(H+1) */
    APIC_F_U = 16, APIC_F_V, APIC_F_VALID_U /* u8 */, APIC_F_VALID_V /* u8 */,
    /* cell arrays, W*H floats */
    APIC_F_DENSITY = 24, APIC_F_SMOOTHED_DENSITY, APIC_F_PRESSURE,
    /* bit masks as u64 words: bit (i % 64) of word i / 64 is cell or face i */
    APIC_F_FLUID_BITS = 32, APIC_F_OBSTACLE_BITS, APIC_F_U_OPEN_BITS, APIC_F_V_OPEN_BITS,
    /* base pressure system in the reference's padded layout (index = cell + W,
     * W*H + 2W floats); only entries at fluid cells are defined */
    APIC_F_RESIDUAL = 40, APIC_F_DIAG, APIC_F_INV_DIAG, APIC_F_PLUS_X, APIC_F_PLUS_Y,
    APIC_F_ERROR /* base multigrid error (preconditioned residual z) */,
    /* (key, val) pairs of the last Morton sort, num_particles u32 each */
    APIC_F_SORT_KEYS = 48, APIC_F_SORT_VALS,
    /* base fluid cell list: padded indices, ascending, fluid_cells u32 */
    APIC_F_FLUID_LIST = 52,
    /* force fields (src/apic.rs:725-728), face-sized floats */
    APIC_F_EXT_FORCE_U = 56, APIC_F_EXT_FORCE_V, APIC_F_POST_FORCE_U, APIC_F_POST_FORCE_V,
    /* coarse multigrid level l (0-based): id + APIC_F_MG_LEVEL_STRIDE * l.
     * Coefficients use the padded layout of that level (Wl*Hl + 2Wl). */
    APIC_F_MG_FLUID_BITS = 64, APIC_F_MG_DIAG, APIC_F_MG_INV_DIAG, APIC_F_MG_PLUS_X,
    APIC_F_MG_PLUS_Y
};
#define APIC_F_MG_LEVEL_STRIDE 256

/* ---- stages, for apic_debug_run_stage (order of src/apic.rs:2429-2474) - */
enum apic_stage {
    APIC_STAGE_SORT = 0, /* update_spatial_lookup                 :1043-1111 */
    APIC_STAGE_P2G,      /* transfer_particles_to_grid            :1218-1497 */
    APIC_STAGE_FORCES,   /* apply_external_forces                 :1604-1626 */
    APIC_STAGE_BUILD,    /* build_pressure_system                 :1640-1785 */
    APIC_STAGE_MG,       /* update_multilevel_grid                :1499-1602 */
    APIC_STAGE_PCG,      /* solve_pcg                             :1865-1956 */
    APIC_STAGE_GRAD,     /* apply_pressure_gradient               :1958-2055 */
    APIC_STAGE_POST,     /* post-force add                        :2453-2458 */
    APIC_STAGE_EXTRAP,   /* extrapolate_velocity                  :2266-2350 */
    APIC_STAGE_G2P,      /* transfer_grid_to_particles_and_advect :2057-2264 */
    APIC_STAGE_VMAX,     /* get_max_particle_velocity             :2412-2427 */
    APIC_STAGE_VCYCLE,   /* apply_preconditioner alone            :1788-1821 */
    APIC_STAGE_COUNT
};

/* ---- scene generators (host code only; no GPU needed) ------------------ */
#define APIC_SCENE_REFERENCE_DEFAULT 0 /* Apic::new's 3x3-per-cell block, src/apic.rs:831-849 */
#define APIC_SCENE_DAM_BREAK         1 /* fluid where x < fluid_x and y < fluid_y */
#define APIC_SCENE_DAM_BREAK_DISK    2 /* dam break plus a disk with its own velocity */
#define APIC_SCENE_NOISE             3 /* value-noise mask > threshold, N(0, sigma^2) velocities */
typedef struct apic_scene_params {
    uint32_t kind;
    uint32_t width, height;   /* grid cells */
    float    cell_size;       /* domain units per cell */
    uint32_t sub;             /* sub x sub particles per cell, jittered per sub-cell */
    uint32_t seed;
    float    fluid_x, fluid_y;          /* dam-break extent (domain units) */
    float    disk_x, disk_y, disk_r;    /* disk centre and radius */
    float    disk_vx, disk_vy;          /* disk initial velocity */
    float    noise_period;              /* value-noise lattice period (domain units) */
    float    noise_threshold;
    float    vel_sigma;                 /* per-component velocity std-dev (NOISE) */
} apic_scene_params;

/* Number of particles the scene holds. */
int apic_scene_count(const apic_scene_params* p, uint64_t* n_out);
/* Fill n particles; n must equal apic_scene_count's result. */
int apic_scene_fill(const apic_scene_params* p, uint64_t n,
                    float* pos_x, float* pos_y, float* vel_x, float* vel_y);

/* ---- lifecycle --------------------------------------------------------- */
typedef struct apic_handle apic_handle;

/* Apic::new (src/apic.rs:779-916): grid, 1-cell solid border, the reference's
 * default dam-break particles, multigrid hierarchy, open-face masks. */
int apic_create(uint32_t width, uint32_t height, float cell_size,
                const apic_world_props* props, apic_handle** out);
int apic_destroy(apic_handle* h);
/* Text of the last error on this thread (static storage, never NULL). */
const char* apic_last_error(void);
/* Number of CUDA devices visible (0 without a GPU). */
int apic_device_count(int* n_out);

/* ---- the step ---------------------------------------------------------- */
/* Apic::update (src/apic.rs:2429-2474).  flags: APIC_UPDATE_*. */
int apic_update(apic_handle* h, uint32_t flags, float frame_deltatime);
/* Apic::add_radial_force (src/apic.rs:2352-2410). */
int apic_add_radial_force(apic_handle* h, float world_x, float world_y,
                          float radius, float strength);
/* Apic::get_max_particle_velocity (src/apic.rs:2412-2427). */
int apic_max_particle_velocity(apic_handle* h, float* out);
/* Apic::is_fluid (src/apic.rs:1015-1022). */
int apic_is_fluid(apic_handle* h, int32_t i, int32_t j, uint64_t* out);
/* Apic::update_world (src/apic.rs:918-944): recompute the open-face masks
 * from the obstacle mask (call after writing APIC_F_OBSTACLE_BITS). */
int apic_update_world(apic_handle* h);

/* ---- state access (the reference's public fields) ---------------------- */
int apic_get_info(apic_handle* h, apic_info* out);
int apic_get_stats(apic_handle* h, apic_step_stats* out);
/* Element count and element size in bytes of a field. */
int apic_field_shape(apic_handle* h, int field, uint64_t* count, uint32_t* elem_bytes);
/* Copy a whole field device->host / host->device; bytes must equal
 * count*elem_bytes.  Both synchronise the handle's stream. */
int apic_read_field(apic_handle* h, int field, void* dst, uint64_t bytes);
int apic_write_field(apic_handle* h, int field, const void* src, uint64_t bytes);
/* Particle pair field in the reference's AoSoA-8 `Vec2x8` layout: per chunk
 * 8 x-lanes then 8 y-lanes (num_chunks*16 floats).  which: 0 positions,
 * 1 velocities, 2 c_u, 3 c_v.  Fills `Vec<Vec2x8>` mirrors directly. */
int apic_read_vec2x8(apic_handle* h, int which, float* dst, uint64_t floats);

/* ---- pipelined host I/O (no counterpart in the reference) -------------------
 * Stream-ordered forms of apic_update, apic_write_field (force fields) and
 * apic_read_vec2x8 for callers that overlap their host <-> device copies with
 * the next update, e.g. a GUI or server that uploads each frame's forces and
 * reads each frame's particles.  Host buffers should be pinned
 * (cudaHostAlloc / cudaHostRegister) for the copies to be asynchronous.
 * Results are those of the synchronous calls, bit for bit.
 *
 * apic_update_async enqueues Apic::update (src/apic.rs:2429) and returns;
 * apic_update_wait waits for it and publishes its statistics (apic_get_stats)
 * and status.  apic_update = apic_update_async + apic_update_wait. */
int apic_update_async(apic_handle* h, uint32_t flags, float frame_deltatime);
int apic_update_wait(apic_handle* h);
/* Starts copying one external or post force field (APIC_F_EXT_FORCE_U/V,
 * APIC_F_POST_FORCE_U/V; u: (W+1)*H floats, v: W*(H+1)) from host memory
 * into a device staging buffer on the handle's upload stream and returns.
 * The next update applies it to the field before it starts, as if
 * apic_write_field had been called just before (after any apic_write_field
 * of the same field); a field staged twice before an update applies the
 * second.  Staged, not yet applied fields are not part of a snapshot. */
int apic_stage_field(apic_handle* h, int field, const void* src, uint64_t bytes);
/* Enqueues the Vec2x8 packing of `which` (as apic_read_vec2x8) after the
 * work already enqueued on the handle (so after an apic_update_async) and its
 * copy into dst on the handle's download stream; returns at once.  dst holds
 * the values after apic_read_wait.  Two reads of the same pair may be in
 * flight; the caller keeps their destinations apart. */
int apic_read_vec2x8_async(apic_handle* h, int which, float* dst, uint64_t floats);
int apic_read_wait(apic_handle* h);
/* Replace the particle set (scene injection): n particles, C = 0, time
 * residual = 0; the last AoSoA chunk is padded with the last position and
 * zero velocity as in src/apic.rs:887-898. */
int apic_set_particles(apic_handle* h, uint32_t n, const float* pos_x, const float* pos_y,
                       const float* vel_x, const float* vel_y);

/* ---- pressure solver configuration ------------------------------------- */
int apic_set_solver(apic_handle* h, int mode, float rel_tol, uint32_t max_iterations);

/* ---- execution options --------------------------------------------------- */
/* Options 1-3 and 6 (a persistent cooperative solve, a fused V-cycle, a
 * cluster of middle levels reading global memory, a one-cluster solve for
 * small scenes) were measured slower than the defaults on GB300 and are no
 * longer offered; their ids are rejected as unknown options. */
/* 1 (default): kernels inside the PCG loop use programmatic dependent launch
 * (each is scheduled while its predecessor drains and waits on the device
 * for its results); 0: plain stream order.  Same results bit for bit. */
#define APIC_OPT_PDL 4
/* 1 (default where the level sizes allow): the multigrid levels from the
 * largest that fits down to 64 rows live in the distributed shared memory of
 * one 16-CTA thread-block cluster (each CTA owns a band of rows) and the
 * coarser ones in its first CTA.  0: every level above the shared-memory
 * tail runs as separate sweep and transfer kernels.
 * apic_get_option reports 0 where no level qualifies.  Same results bit for
 * bit. */
#define APIC_OPT_DSM_VCYCLE 5
/* No counterpart in the reference (whose PCG starts from zero).  Value 1
 * (default): in APIC_SOLVER_REL_MIXED each solve starts from the FP64
 * pressure of the previous solve (zero after apic_set_particles or
 * apic_restore) instead of zero; the exit test, true residual <= rel_tol of
 * ||b||, is unchanged, so only the iteration count differs.  0: start from
 * zero.  Other solver modes always start from zero. */
#define APIC_OPT_WARM_START 7
/* No counterpart in the reference.  Priority of the scene's stream, in
 * levels above the lowest (0, the default); clamped to the device's range
 * (apic_get_option reports the level used).  When several scenes share the
 * GPU, the block scheduler starts the kernels of higher-priority streams
 * first.  Results do not change. */
#define APIC_OPT_STREAM_PRIORITY 8
/* Order in which P2G adds each face's contributions.  Every order is
 * deterministic (two runs give the same bits).
 *   1: the reference's single-thread order (transfer_particles_to_grid,
 *      src/apic.rs:1218-1426, with add_to_mac's in-chunk merging): per chunk
 *      of 8 slots and per corner the lanes' group sum, groups added in
 *      (chunk, corner) order; bit-identical to the oracle.
 *   2: cell order: the face's contributions by the cell of the particle's
 *      density-stencil base (a fixed list of up to six cells per face), and
 *      by slot within a cell; the same terms as order 1 in another order, so
 *      the sums differ only in rounding.  About twice as fast.
 *   0 (default): order 1 in APIC_SOLVER_REFERENCE, order 2 in the relative
 *      solver modes (which have no counterpart in the reference).
 * apic_get_option reports the order in use (1 or 2). */
#define APIC_OPT_P2G_ORDER 9
int apic_set_option(apic_handle* h, int option, int value);
int apic_get_option(apic_handle* h, int option, int* value);

/* ---- measurement -------------------------------------------------------- */
/* When enabled, each stage of each substep is bracketed by CUDA events on the
 * handle's stream; apic_get_stage_times returns the summed milliseconds per
 * apic_stage and the number of launches of each since the last reset. */
int apic_set_profiling(apic_handle* h, int enabled);
int apic_get_stage_times(apic_handle* h, double* ms, uint64_t* launches, int n);
int apic_reset_stage_times(apic_handle* h);
/* Wait for all work of the handle's stream. */
int apic_synchronize(apic_handle* h);
/* The handle's cudaStream_t, for callers that interleave their own work. */
int apic_get_stream(apic_handle* h, void** stream_out);

/* ---- Morton sort without device allocation ------------------------------ */
/* No counterpart in the reference.  Computes the same Morton keys and stable
 * sort permutation as the handle's sort stage, for callers that cannot
 * allocate device memory: code recording work into a stream capture (where
 * cudaMalloc is not allowed) and applications whose device memory belongs to
 * another runtime or a fixed budget.  pos_x/pos_y: n device floats;
 * keys_out/vals_out: n device u32 (sorted keys; original slot of each).
 * Every intermediate buffer lives in one fixed device array inside the
 * library (about 8.5 MiB, held by every GPU that loads it until exit), so n is
 * limited to 1,048,576; larger n, or a width or height above 65536 (the
 * Morton code interleaves 16 bits per axis), returns APIC_ERR_INVALID_ARG.
 * The first call in a CUDA context (normally: the first on a device) looks up
 * that array's device address; make it before any stream capture.  A context
 * created later (after cudaDeviceReset, or the caller's own) gets a fresh
 * lookup.  Work is enqueued on `stream` (NULL: default stream); calls whose
 * work overlaps on the GPU share the array and race.  Nothing in the array has
 * to start at zero: every word is written before it is read. */
int apic_morton_sort_noalloc(const float* pos_x, const float* pos_y, uint32_t n, uint32_t width, uint32_t height,
                             float cell_size, uint32_t* keys_out, uint32_t* vals_out, void* stream);

/* ---- batched and served scenes ------------------------------------------ */
/* No counterpart in the reference, which simulates one scene per process.
 * One Apic::update of each of `count` distinct scenes; each scene computes
 * exactly what apic_update computes for it, bit for bit.  When every scene
 * uses a relative solver mode (all the same one), has a multigrid level and
 * a shared-memory coarse tail, lives on the calling thread's current device,
 * and no scene is in profiling mode, the whole
 * batch runs as one CUDA graph: each scene's stages before and after the
 * pressure solve are its own kernels (side by side, each under a
 * device-side condition for its substeps), and the pressure solves of all
 * scenes run as ONE launch per solve phase over a table of scenes.  The
 * graph is built on the first call for a given list of scenes and reused
 * while the list and the scenes' settings stay the same.  Otherwise, or with
 * APIC_UPDATE_BATCH_STREAMS in flags, every scene's update is enqueued on its
 * own stream before any is waited on, so the GPU runs the scenes' kernels
 * side by side.  Calls are serialised inside the library.  status (may be
 * NULL): per-scene result; the return value is the first failure. */
int apic_update_batch(apic_handle* const* handles, uint32_t count, uint32_t flags, float frame_deltatime,
                      int* status);

/* Estimated device bytes of a scene (upper bound used for admission). */
int apic_scene_bytes(uint32_t width, uint32_t height, uint64_t particles, uint64_t* bytes_out);

/* The last apic_update_batch call in this process: scenes, whether the
 * solves ran as one launch per phase (joint 1) or on the scenes' streams
 * (joint 0), and, for a joint batch, the kernels the batch itself launched
 * (the solve phases and the substep control: every scene's own kernels are
 * in its apic_step_stats.kernel_launches) and how many times the batch's
 * substep, refinement and PCG loop bodies ran.  The library tunes how it
 * runs a batch of a given makeup (every scene's sides and solver mode, in
 * order) over the first calls for that makeup, trying the stream-per-scene
 * form and the joint form with several work shapes on the caller's own
 * updates (the results are the same bits whichever runs); tuned is 1 once
 * the choice is made, and chunk_segs / block_group give the joint shape
 * used (segments per item of the sweeps and transfers, blocks per item of
 * the PCG iteration's reductions). */
typedef struct apic_batch_info {
    uint32_t scenes;
    uint32_t joint;
    uint64_t batch_kernel_launches;
    uint32_t substep_rounds;
    uint32_t refine_rounds;
    uint32_t pcg_rounds;
    uint32_t tuned;
    uint32_t chunk_segs;
    uint32_t block_group;
} apic_batch_info;
int apic_batch_last_info(apic_batch_info* out);

/* Placement of independent scenes on several GPUs (no counterpart in the
 * reference, which runs one scene in one process).  Scenes share nothing, so
 * a multi-GPU batch needs no collective: each GPU runs the scenes placed on it
 * and the results are gathered on the host.  Scenes are taken largest first
 * (by bytes, ties by index) and each goes to the device with the least work
 * placed so far among those whose remaining budget holds it (ties: lowest
 * device).  bytes / work: per scene (work e.g. particles x steps); budgets:
 * per device.  device_out[i] = the device of scene i, or -1 when no device
 * can hold it.  Deterministic: the same inputs give the same placement on
 * every rank. */
int apic_place_scenes(const uint64_t* bytes, const uint64_t* work, uint32_t count, const uint64_t* budgets,
                      uint32_t devices, int32_t* device_out);

/* Continuous-batching request server (no counterpart in the reference,
 * which runs one scene per process): requests (scene, step count, dt) are
 * queued on submission and admitted in arrival order while the scenes in the
 * server are fewer than max_active and their estimated memory fits
 * memory_budget_bytes; a scene's state stays on the device until it reached
 * its step count.  keep_results: copy each finished scene's positions
 * (Vec2x8 layout) to the host before its device memory is released.
 *
 * APIC_SERVER_CONTINUOUS (default): every scene is relaunched on its own
 * stream as soon as its update completes; admitted scenes are prepared
 * (particles generated, device state allocated and uploaded, update graph
 * built) on `prepare_threads` host threads while the GPU runs the others.
 * apic_server_step returns once at least one update has completed (or the
 * server is empty).  APIC_SERVER_ROUNDS: apic_server_step admits on the
 * calling thread, runs one update of every active scene (as
 * apic_update_batch) and returns when all are done; max_active = 1 gives
 * the plain path, one scene at a time.  Calls on one server must not
 * overlap.  An update that does not complete within 120 s makes
 * apic_server_step return APIC_ERR_TIMEOUT. */
enum { APIC_SERVER_ROUNDS = 0, APIC_SERVER_CONTINUOUS = 1 };
typedef struct apic_server apic_server;
typedef struct apic_server_round {
    uint32_t admitted, stepped, completed, active, queued;  /* active: running or being prepared */
    double   round_ms;       /* wall time of this call's updates */
    uint64_t memory_used;    /* estimated bytes of the admitted scenes */
} apic_server_round;
typedef struct apic_request_info {
    int      status;         /* APIC_OK, or why the request failed */
    uint32_t finished;
    uint32_t steps_done;
    uint64_t particles, substeps, pcg_iterations;
    double   max_true_residual;           /* over its updates (mixed / FP32 relative modes) */
    double   submit_ms, admit_ms, done_ms; /* since server creation; -1 when not yet */
    uint64_t bytes;          /* admission estimate */
    uint64_t result_floats;  /* kept positions (0: none) */
} apic_request_info;
typedef struct apic_server_stats {
    uint64_t submitted, completed, failed, active, queued, rounds;
    uint64_t particle_substeps, particle_updates;
    double   busy_ms, elapsed_ms;
    double   step_p50_ms, step_p99_ms;        /* per update: launch to completion (rounds: the round) */
    double   request_p50_ms, request_p99_ms;  /* completion minus submission */
    uint64_t memory_used, memory_peak;
    uint64_t updates;                         /* completed scene updates */
    double   prepare_ms;                      /* host time spent preparing scenes (all threads) */
    double   host_ms;                         /* step calls' time outside the update loop */
    int32_t  mode;                            /* APIC_SERVER_* */
    uint32_t prepare_threads;
    uint64_t kernel_launches;                 /* kernels the completed updates launched */
} apic_server_stats;
int apic_server_create(uint64_t memory_budget_bytes, uint32_t max_active, uint32_t keep_results,
                       apic_server** out);
/* Mode and preparation threads (0: prepare on the calling thread); only
 * while no scene is admitted. */
int apic_server_set_mode(apic_server* sv, int mode, uint32_t prepare_threads);
/* apic_set_option(option, value) on every scene the server creates whose
 * cell count lies in [min_cells, max_cells] (rules apply in the order given;
 * only while no scene is admitted). */
int apic_server_scene_option(apic_server* sv, int option, int value, uint64_t min_cells, uint64_t max_cells);
/* Work limit: a queued request is admitted only while the grid cells of the
 * admitted scenes plus its own stay within max_active_cells (a request that
 * would be alone is always admitted); 0 (default) removes the limit.  Small
 * scenes need many scenes in flight to fill the GPU, large ones few. */
int apic_server_set_work_limit(apic_server* sv, uint64_t max_active_cells);
int apic_server_destroy(apic_server* sv);
int apic_server_submit(apic_server* sv, const apic_scene_params* scene, const apic_world_props* props,
                       uint32_t steps, float frame_deltatime, int solver_mode, float rel_tol,
                       uint32_t max_iterations, uint64_t* id_out);
int apic_server_step(apic_server* sv, apic_server_round* out);
int apic_server_request(apic_server* sv, uint64_t id, apic_request_info* out);
int apic_server_result_positions(apic_server* sv, uint64_t id, float* dst, uint64_t floats);
int apic_server_get_stats(apic_server* sv, apic_server_stats* out);

/* ---- snapshot / restore ------------------------------------------------ */
/* No counterpart in the reference (its state lives in the Apic struct's pub
 * fields, src/apic.rs:716-775).  A snapshot is a host byte blob of the state
 * that a later apic_update reads: the nine particle arrays with their padding
 * lanes, the obstacle mask, pending external and post forces, timestamp and
 * prev_deltatime, the solver settings, and (APIC_OPT_WARM_START in the mixed
 * mode) the last solve's FP64 pressure that the next solve starts from.
 * apic_restore loads it into a handle created with the same width, height,
 * cell size and world properties; the next updates of both handles then
 * compute the same thing. */
int apic_snapshot_bytes(apic_handle* h, uint64_t* bytes);
int apic_snapshot(apic_handle* h, void* dst, uint64_t bytes);
int apic_restore(apic_handle* h, const void* src, uint64_t bytes);

/* ---- headless particle view -------------------------------------------- */
/* Replaces the GUI's particle drawing (render_particles, src/main.rs:207-277,
 * with make_circle_texture, :73-101) by a frame in device memory: each
 * particle with finite coordinates inside the frame plus `margin` is splatted,
 * in particle order, as a 2*draw_radius pixel quad textured with the 32 x 32
 * anti-aliased disc, tinted r = min(0.01 |v|^2, 1), g = 0.5, b = 1 - r/2, and
 * alpha blended into an RGBA8 frame cleared to `background`.  Pixel (px, py)
 * has its centre at (px + 0.5, py + 0.5); row 0 is the top of the view:
 * draw_x = x * scale, draw_y = height - y * scale (the GUI's default camera,
 * :222-235).  The GL window, its camera zoom/pan and the text HUD are not
 * rendered (no graphics stack is used). */
typedef struct apic_render_params {
    uint32_t width, height;  /* frame in pixels (1920 x 1080 in the GUI, src/main.rs:26-27); 1..16384 */
    float scale;             /* pixels per world unit (SIM_SCALE, :34) */
    float draw_radius;       /* disc radius in pixels (DRAW_RADIUS = 3, :35); (0, 7] */
    float margin;            /* out-of-bounds margin in pixels (50, :237-240); [0, 65536] */
    float pick_x, pick_y;    /* pick centre in pixels (:247-256) */
    float pick_radius;       /* pick radius in pixels; < 0: no pick */
    uint32_t background;     /* clear colour, RGBA8 little-endian (0xFF000000: clear_background(BLACK)) */
} apic_render_params;

typedef struct apic_render_stats {
    uint32_t valid, nan, out_of_bounds;  /* RenderStats (:39-43) */
    uint32_t fluid_cells;                /* base fluid cells of the last substep */
    int64_t picked;                      /* nearest particle within pick_radius (first on ties); -1: none */
    float volume;                        /* fluid_cells * cell_size^2 (:461-468) */
    uint32_t kernels;                    /* kernels launched for the frame */
} apic_render_stats;

/* Render the particles into the scene's frame (device memory, allocated on
 * first use and kept until the handle is destroyed) and wait for it. */
int apic_render(apic_handle* h, const apic_render_params* params, apic_render_stats* stats);
/* Copy the last frame to host memory: width * height * 4 bytes, rows top to
 * bottom, bytes R, G, B, A per pixel. */
int apic_read_frame(apic_handle* h, uint8_t* dst, uint64_t bytes);
/* Device address and size of the last frame (valid until the next apic_render
 * or apic_destroy), for consumers that keep it on the GPU. */
int apic_frame_device_ptr(apic_handle* h, void** ptr, uint32_t* width, uint32_t* height);

/* ---- testing hook ------------------------------------------------------ */
/* Run one stage of the substep on the current device state with substep dt.
 * Derived device structures (fluid lists, segment lists) are rebuilt from the
 * written fields first.  Used by the stage-by-stage parity tests. */
int apic_debug_run_stage(apic_handle* h, int stage, float dt);
/* End-of-substep bookkeeping after stage-by-stage runs: prev_deltatime = dt,
 * timestamp += 1 (src/apic.rs:2465-2467). */
int apic_debug_finish_substep(apic_handle* h, float dt);

#ifdef __cplusplus
}
#endif
#endif /* APIC_GPU_H */
