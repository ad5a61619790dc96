/*
 * apic_oracle.h — C API of the CPU oracle (test infrastructure only).
 *
 * The oracle is a C++ restatement of the reference APIC/FLIP step
 * (fireblade2534/APIC-Fluid-Simulation, src/apic.rs).  Only the tests, the
 * smoke check and bench.py's CPU-baseline leg may load it; the product never
 * does.  Parity is UNPINNED: the reference ships no tests, fixtures or golden
 * vectors, and its Rust toolchain and crates are absent, so the restatement
 * could not be checked against the reference's own outputs.
 *
 * Field and stage identifiers are the ones of include/apic_gpu.h.  A sim
 * created with fp64 != 0 runs every floating-point operation in double (the
 * FP64 shadow); its float fields are then read and written as doubles.
 */
#ifndef APIC_ORACLE_H
#define APIC_ORACLE_H
#include <stdint.h>
#include "../include/apic_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_sim oracle_sim;

/* threads <= 1: serial, in the reference's RAYON_NUM_THREADS=1 order.
 * threads > 1: OpenMP, with the reference's parallel/serial split. */
oracle_sim* oracle_create(uint32_t width, uint32_t height, float cell_size,
                          const apic_world_props* props, int fp64, int threads);
void oracle_destroy(oracle_sim* o);
int  oracle_set_threads(oracle_sim* o, int threads);
int  oracle_set_particles(oracle_sim* o, uint32_t n, const float* px, const float* py,
                          const float* vx, const float* vy);
int  oracle_set_solver(oracle_sim* o, int mode, float rel_tol, uint32_t max_iterations);
/* Mixed mode: start each solve from the previous one's FP64 pressure (1, the
 * default, as the GPU library's APIC_OPT_WARM_START) or from zero (0). */
int  oracle_set_warm_start(oracle_sim* o, int enabled);
int  oracle_update(oracle_sim* o, uint32_t flags, float frame_dt);
int  oracle_run_stage(oracle_sim* o, int stage, float dt);
/* End-of-substep bookkeeping (prev_deltatime, timestamp), src/apic.rs:2463-2467. */
int  oracle_finish_substep(oracle_sim* o, float dt);
int  oracle_max_particle_velocity(oracle_sim* o, float* out);
int  oracle_add_radial_force(oracle_sim* o, float x, float y, float radius, float strength);
int  oracle_get_info(oracle_sim* o, apic_info* out);
int  oracle_get_stats(oracle_sim* o, apic_step_stats* out);
int  oracle_field_shape(oracle_sim* o, int field, uint64_t* count, uint32_t* elem_bytes);
int  oracle_read_field(oracle_sim* o, int field, void* dst, uint64_t bytes);
int  oracle_write_field(oracle_sim* o, int field, const void* src, uint64_t bytes);
/* Headless particle view (src/main.rs:73-101, :207-277): RGBA8 frame of
 * width * height * 4 bytes into rgba, stats as apic_render returns them. */
int  oracle_render(uint32_t n, const float* px, const float* py, const float* vx, const float* vy,
                   const apic_render_params* params, uint32_t fluid_cells, float cell_size, uint8_t* rgba,
                   apic_render_stats* stats);
/* Stand-alone helpers for known-answer tests. */
uint32_t oracle_morton(uint32_t x, uint32_t y);
float    oracle_random_lane(uint32_t slot, uint32_t seed);
float    oracle_temporal_weight(float tau);

#ifdef __cplusplus
}
#endif
#endif
