/* polarism_gb300 -- C ABI of the GB300 (sm_103a) GPE time-stepping library.
 *
 * Plain C types only: pointers, sizes and status codes.  Every entry point returns
 * PG_OK (0) on success or a PG_ERR_* code; pg_last_error() then holds a message
 * for the calling thread.  Complex arrays are interleaved (re, im) in the
 * reference's canonical layout (B, C, ny, nx); reservoir arrays are (B, C_res, ny, nx).
 *
 * A pg_solver owns its device buffers, one non-blocking CUDA stream and the CUDA
 * graphs it captures.  Host buffers passed in are read/written synchronously
 * before the call returns unless stated otherwise; "on_device" flags say whether
 * a pointer is a device address (1) or host memory (0).
 *
 * Each solver entry point replaces the launch path of one reference solver
 * (paths relative to the Polarism source tree):
 *   pg_rk4_advance     <- polarism/solver/rk4_cuda_solver.py:3451-3642 (RK4CudaSolver.advance)
 *                         and _step_gpu :3251-3350 (tiled whole-step kernel :1296-1479)
 *   pg_philox_words    <- polarism/noise/philox.py:59-109 (philox_words kernel, test hook)
 *   pg_ifrk_advance    <- polarism/solver/ifrk_fft_cuda_solver.py:148-241, ifrk_cuda_fused.py:851-1141
 *   pg_ifrk_trial      <- polarism/solver/ifrk_fft_cuda_solver.py:243-311 (adaptive DP5 trial)
 *   pg_set_noise       <- polarism/noise/stochastic.py:15-37 (NoiseApplier member arrays)
 *   pg_split_advance   <- polarism/solver/split_step_fft_solver.py:97-159 (ordering 0) and
 *                         polarism/solver/split_step_fft_cuda_solver.py:1144-1325 (ordering 1)
 *   pg_set_pump        <- polarism/laser/pump_field.py:71-79 (separable envelope) and
 *                         rk4_cuda_solver.py:3564-3578 (per-stage pump scales)
 *   pg_sweep_*         <- polarism/sweep.py:98-324 (Sweep.run over groups of grid sizes) with
 *                         rk4_cuda_solver.py:1482-1536 (batched per-member constants)
 */
#ifndef POLARISM_GB300_H
#define POLARISM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PG_OK 0
#define PG_ERR_INVALID 1     /* bad argument or unsupported configuration */
#define PG_ERR_CUDA 2        /* a CUDA runtime call failed */
#define PG_ERR_UNSUPPORTED 3 /* configuration the kernels do not support */
#define PG_ERR_TIMEOUT 4     /* a bounded device wait gave up */

#define PG_SINGLE 0
#define PG_DOUBLE 1

#define PG_RES_NONE 0
#define PG_RES_SINGLE 1
#define PG_RES_DOUBLE 2      /* active + inactive reservoirs (RK4 tiled kernel and IFRK) */
#define PG_RES_QDOUBLE 3     /* quadratic-double: n_R fed by kappa n_I^2 (RK4 tiled kernel and IFRK) */

#define PG_POT_NONE 0
#define PG_POT_REAL 1
#define PG_POT_COMPLEX 2

/* Physics constants of one sweep member; names and meaning follow
 * polarism/config/simulation_parameters.py:43-67 (PhysicsConstants). */
typedef struct pg_physics {
  double hbar, m_eff, g_C, g_R, g_I, R, gamma_C, gamma_R;
  double kinetic_relaxation_eta;
  /* Double reservoir (polarism/reservoir/double_reservoir.py:106-130). */
  double gamma_I, gamma_A, R_IA, R_AI;
  /* Two-component fields: cross-spin interaction, Zeeman splitting and TE-TM coefficient
   * (polarism/model.py:129-173, polarism/dispersion.py:34-63), and the pump share of each
   * component, (1 +- circular_polarization) / 2 (polarism/simulation_controller.py:974-979). */
  double alpha_2, zeeman, te_tm;
  double pump_weight_plus, pump_weight_minus;
  /* Quadratic inactive-to-active transfer rate (polarism/reservoir/quadratic_double_reservoir.py). */
  double kappa;
} pg_physics;

typedef struct pg_config {
  int32_t nx, ny;          /* periodic grid */
  int32_t members;         /* batch size B */
  int32_t precision;       /* PG_SINGLE (complex64) or PG_DOUBLE (complex128) */
  int32_t reservoir;       /* PG_RES_NONE, PG_RES_SINGLE, PG_RES_DOUBLE or PG_RES_QDOUBLE */
  int32_t potential;       /* PG_POT_* */
  int32_t pump_per_member; /* 0: one envelope shared by all members; 1: one per member */
  int32_t potential_per_member;
  double dx, dy, dt;
  int32_t components;           /* 1 scalar field, 2 circular-basis spinor (0 means 1) */
  int32_t reservoir_components; /* reservoir fields per component set: 1 shared or = components
                                   (0 means = components) */
  /* Separable pump terms L (lasers, polarism/laser/pump_field.py:81-89; 0 means 1):
   * P(x, t) = sum_l c_l(t) E_l(x), each product and each partial sum rounded separately as in
   * the reference's combiner (polarism/solver/cuda_pump.py:7-19).  With L > 1 pg_set_pump
   * takes L envelopes one after another and every coefficient array below gains a term axis
   * before the member axis ([step][stage][term][member]); the full-width RK4 kernel then gives
   * way to the general one. */
  int32_t pump_terms;
  int32_t reserved_;
} pg_config;

typedef struct pg_solver pg_solver;

/* Library status. */
const char* pg_last_error(void);
int pg_device_count(void);
int pg_version(void);

/* Lifecycle. physics points at cfg->members entries. */
int pg_create(const pg_config* cfg, const pg_physics* physics, pg_solver** out);
void pg_destroy(pg_solver* s);
/* The solver's CUDA stream (a cudaStream_t) for event timing by the caller. */
void* pg_stream(pg_solver* s);
int pg_synchronize(pg_solver* s);

/* State transfer: psi is B*nx*ny complex values, res is B*nx*ny reals (or NULL
 * without a reservoir).  pg_set_state clamps nothing; the reference clamps in
 * reservoir.set_state after each step, and so does the step kernel. */
int pg_set_state(pg_solver* s, const void* psi, const void* res, int on_device);
int pg_get_state(pg_solver* s, void* psi, void* res, int on_device);
/* Device addresses of the current state buffers (valid until the next advance). */
int pg_state_pointers(pg_solver* s, void** psi, void** res);

/* Pump envelopes (L times nx*ny reals, or L times B*nx*ny with pump_per_member) and potential
 * (nx*ny reals or complex, or B*nx*ny with potential_per_member). */
int pg_set_pump(pg_solver* s, const void* envelope, int on_device);
int pg_set_potential(pg_solver* s, const void* potential, int on_device);

/* Truncated-Wigner noise: per member seed, gamma_C, R and strength, and the common
 * dt / (4 dV).  seeds == NULL turns the noise off. */
int pg_set_noise(pg_solver* s, const uint64_t* seeds, const double* gamma,
                 const double* scattering, const double* strength, double dt_over_4dv);

/* Advance n_steps fused RK4 steps starting at global step index start_step.
 * stage_scales holds 3 * members coefficients per step, laid out
 * [step][stage (t, t+dt/2, t+dt)][member], on the host.  use_graphs captures
 * chunks of up to 64 steps into CUDA graphs. */
int pg_rk4_advance(pg_solver* s, int64_t start_step, int32_t n_steps, const double* stage_scales,
                   int use_graphs);
/* Build, without launching anything, the CUDA graphs an n_steps pg_rk4_advance uses (for
 * either buffer parity), so that the first such advance replays them instead of capturing (no
 * counterpart in the reference, which captures on first use; rk4_cuda_solver.py:3564-3602). */
int pg_rk4_prepare(pg_solver* s, int32_t n_steps);

/* Override the RK4 launch geometry (the autotuner's knobs): tile_w useful columns per
 * block (tile_w >= nx selects one full-width block per row strip) and strip_h output
 * rows per block (a positive multiple of 4). */
int pg_rk4_set_geometry(pg_solver* s, int32_t tile_w, int32_t strip_h);
int pg_rk4_get_geometry(pg_solver* s, int32_t* tile_w, int32_t* strip_h);

/* Advance n_steps split-step Fourier steps (nx, ny powers of two up to 4096).
 * ordering 0: R(dt/2) K(dt/2) N(dt) K(dt/2) R(dt/2) with psi in real space before and after
 *             (replaces polarism/solver/split_step_fft_solver.py:97-159, "split-step-fft");
 * ordering 1: K(dt/2) [R(dt/2) N(dt) R(dt/2)] K(dt/2) with the state left as the
 *             unnormalised 2-D spectrum (replaces polarism/solver/split_step_fft_cuda_solver.py:
 *             1144-1325, "split-step-fft-cuda").
 * half_scales holds 2 * members pump coefficients per step, [step][(t+dt/4, t+3dt/4)][member].
 * The Wigner increment is drawn after N (ordering 0, with n_R after the first half step) or after
 * the second reservoir half step (ordering 1), with counter step = start_step + k. */
int pg_split_advance(pg_solver* s, int32_t ordering, int64_t start_step, int32_t n_steps,
                     const double* half_scales, int use_graphs);
/* The same for pg_split_advance of the ordering (see pg_rk4_prepare). */
int pg_split_prepare(pg_solver* s, int32_t ordering, int32_t n_steps);
/* Whether the state buffer holds psi(x, y) (0) or its unnormalised spectrum (1). */
int pg_set_state_kind(pg_solver* s, int32_t spectral);
int pg_get_state_kind(pg_solver* s, int32_t* spectral);

/* Lawson integrating-factor RK steps (nx, ny powers of two up to 4096; psi in real space
 * before and after).  tableau 0 = classic RK4, 1 = Dormand-Prince 5(4).  Replaces the fixed-step
 * path of polarism/solver/ifrk_fft_cuda_solver.py:148-241 and polarism/solver/ifrk_cuda_fused.py:
 * 851-1141.  stage_scales holds stages * members pump coefficients per step,
 * [step][stage (t + c_i dt)][member]; the Wigner increment follows each step (counter step =
 * start_step + k, post-step clamped n_R). */
int pg_ifrk_advance(pg_solver* s, int32_t tableau, int64_t start_step, int32_t n_steps,
                    const double* stage_scales);
/* One adaptive Dormand-Prince trial of size h (tableau must be 1): computes the embedded error
 * norm of polarism/solver/ifrk_fft_cuda_solver.py:243-293 (accumulated in FP64) into err_out
 * and commits the step when err <= 1 (accepted = 1); otherwise the state is unchanged.
 * stage_scales holds 7 * members coefficients [stage (t + c_i h)][member]. */
int pg_ifrk_trial(pg_solver* s, int32_t tableau, double h, const double* stage_scales, double rtol,
                  double atol, double* err_out, int32_t* accepted);

/* FP64 observables of the current (real-space) state.
 * pg_accumulate adds one sample: kinds bit 1 = per-site sum |psi|^2 and sum |psi|^4
 * (polarism/results/accumulators.py:134-172, G2Accumulator), bit 2 = per-mode sum |FFT2 psi|^2
 * (accumulators.py:95-131, MomentumDistribution; nx, ny powers of two).
 * pg_accumulator_sums copies B*nx*ny sums of kind 0 (rho), 1 (rho^2) or 2 (|psi_k|^2) to the host
 * with their sample count; pg_accumulator_reset clears them. */
int pg_accumulate(pg_solver* s, int32_t kinds);
int pg_accumulator_sums(pg_solver* s, int32_t kind, double* out, int64_t* samples);
int pg_accumulator_reset(pg_solver* s);
/* Zero the observable sums and their sample counts, stream ordered (no host wait; the
 * steady-state monitor is left alone): a fresh MomentumDistribution / G2Accumulator
 * (polarism/results/accumulators.py:95-172) for a run whose samples are queued on the device.  Samples queued while the solver's halt word is set
 * (after the steady-state check that stopped every member) add nothing. */
int pg_accumulator_zero(pg_solver* s);
/* Restore one accumulator (kind as pg_accumulator_sums) and its sample count, as
 * Accumulator.load_state_dict does on a checkpoint resume (polarism/results/accumulators.py:
 * 83-87,117-119,155-158). */
int pg_accumulator_load(pg_solver* s, int32_t kind, const double* sums, int64_t samples);
/* Per-member norm sum |psi|^2 dx dy in FP64 (polarism/simulation_controller.py:92-103). */
int pg_norms(pg_solver* s, double* out);
/* Steady-state comparison against the previous call (polarism/simulation_controller.py:710-734):
 * per member ||rho - rho_prev|| / ||rho_prev||, |N - N_prev| / N_prev (infinite on the first call)
 * and the norms N; the current density becomes the reference for the next call. */
int pg_steady_check(pg_solver* s, double* rel_density, double* rel_norm, double* norms);
/* Device-resident steady-state monitor: the sampling path of SimulationController.run
 * (polarism/simulation_controller.py:1063-1130 with _check_steady_state and _record_stops,
 * :698-734) without a host round trip per check.
 * pg_steady_update enqueues one check on the solver's stream and returns at once: the
 * comparison of pg_steady_check, and, when `record` is non-zero (the caller's t >= min_time),
 * `step` becomes the stop step of every member not yet stopped whose norm is below 1e-30 or
 * whose relative density and norm changes are both below rtol (no decision on the first check
 * after a reset).  With halt_when_all_stopped, the check that finds every member stopped sets
 * the solver's halt word: RK4 steps queued after it return without changing the state.
 * pg_steady_poll reads, without waiting for the device, the number of stopped members and the
 * index (1, 2, ...) of the newest check the device has finished.
 * pg_steady_results waits for the stream and copies the newest check's values and the stop
 * steps (-1: not stopped; any output may be NULL); if the run halted it returns the halt step
 * (else -1), makes the state of that step the current one and clears the halt.
 * pg_steady_reset forgets the previous density, the stop steps and the halt.
 * pg_steady_check shares the previous density with these calls. */
int pg_steady_update(pg_solver* s, int64_t step, int32_t record, double rtol,
                     int32_t halt_when_all_stopped);
int pg_steady_poll(pg_solver* s, int32_t* stopped, int64_t* updates_done);
int pg_steady_results(pg_solver* s, double* rel_density, double* rel_norm, double* norms,
                      int64_t* stop_steps, int64_t* halt_step);
int pg_steady_reset(pg_solver* s);
/* The monitor's state in checkpoint form (the steady_density / steady_norm / stop_time entries
 * of checkpoint format 2, polarism/simulation_controller.py:771-774,851-864): the previous
 * check's density (members * nx * ny reals of the solver's precision, summed over components),
 * its norms and the stop steps (-1: not stopped).  have_reference is 0 before the first check
 * (density and norms are then left untouched).  pg_steady_import restores them (a reset
 * first); any of density / norms / stop_steps may be NULL on export, stop_steps on import. */
int pg_steady_export(pg_solver* s, void* density, double* norms, int64_t* stop_steps,
                     int32_t* have_reference);
int pg_steady_import(pg_solver* s, const void* density, const double* norms,
                     const int64_t* stop_steps, int32_t have_reference);
/* FP64 norms (sum |psi|^2 * cell per member) of caller-owned device fields psi
 * (members * sites_per_member complex values of the given precision) into the device array
 * norms_out, on `stream` (a cudaStream_t, NULL for the default stream); per-block partial sums
 * live in scratch memory allocated for the call. */
int pg_field_norms(const void* psi, int32_t precision, int32_t members, int64_t sites_per_member,
                   double cell, double* norms_out, void* stream);

/* Allocation-free variant of pg_field_norms (no counterpart in the reference).  For callers
 * that must not allocate device memory -- an application whose device memory is owned by another
 * framework's pooling allocator, or a stepping loop that cannot afford the device-wide
 * synchronisation of cudaMalloc/cudaFree.  The per-block partial sums use a fixed 64 KiB device
 * array (8192 doubles) that every GPU loading the library holds until the process exits; at most
 * 8192 members per call (PG_ERR_INVALID beyond).  All calls share the array: calls whose kernels
 * overlap on the GPU race and must be serialised by the caller.  The call is asynchronous on
 * `stream`; the first call on each device looks up the array's address and should come before
 * any stream capture.  That address is cached per device for the process's lifetime and is not
 * valid after cudaDeviceReset: do not call this entry point on a device that was reset. */
int pg_field_norms_noalloc(const void* psi, int32_t precision, int32_t members,
                           int64_t sites_per_member, double cell, double* norms_out, void* stream);

/* Choose the RK4 kernel: 0 automatic, 1 the tiled streaming kernel (any size, FP32/FP64,
 * potential and relaxation terms), 2 the full-width FP32 kernel (nx in {128, 256, 512, 1024},
 * or a multiple of 1024 up to 16384 in 1024-site bands; single reservoir, one laser, or two on
 * rows of at most 1024 sites; real or complex potential and kinetic relaxation in its general
 * variant), 3 the full-width kernel
 * with four sites a thread (rows of 512 or 1024 sites, no potential or relaxation; bitwise the
 * same results as 2).  pg_rk4_get_kernel reports the one in use (1, 2 or 3). */
int pg_rk4_set_kernel(pg_solver* s, int32_t kind);
int pg_rk4_get_kernel(pg_solver* s, int32_t* kind);

/* Failure detection of the TMA-fed RK4 kernels (full-width, four-sites-a-thread, cluster
 * form; no counterpart in the reference, whose kernels wait on nothing).  Every wait of these
 * kernels on an mbarrier -- a row copy, the block's row exchange, a neighbouring CTA's edge
 * values -- gives up after 100000 polls, a bound compiled into the kernels.  Once a wait of
 * the thread that feeds a block's row ring has given up, it completes later ring slots without
 * copying into them, so the block's remaining waits pass at once and the kernel ends in about
 * the time of one full wait; copies still in flight are waited for before the block exits.
 * The next pg_synchronize or pg_get_state then returns PG_ERR_TIMEOUT, and the state is
 * invalid until set again.  `polls` is 100000 (the default) or 0, the give-up setting: the
 * kernels withhold each block's first row copy, so that a wait runs out on a healthy GPU and
 * the failure path can be exercised (PG_ERR_INVALID for other values).  Changing it drops the
 * captured CUDA graphs. */
int pg_set_wait_limit(pg_solver* s, int32_t polls);

/* CUDA graph capture failures (rk4_cuda_solver.py:3591-3602 restores the pre-chunk state and
 * re-runs the chunk with plain launches when a capture fails).  Here a capture only records, so
 * nothing of a chunk has run when its capture or instantiation fails: pg_rk4_advance and
 * pg_split_advance run that chunk as plain launches from the same state and count it in
 * pg_graph_fallbacks.  pg_test_fail_next_graph is a test hook: the next graph this solver
 * builds fails at capture (1) or instantiation (2) as a failing CUDA call would (0 clears it);
 * it drops the solver's cached graphs. */
int pg_test_fail_next_graph(pg_solver* s, int32_t what);
int64_t pg_graph_fallbacks(pg_solver* s);

/* No counterpart in the reference (whose NumPy/CuPy loop waits whenever it reads a value).
 * Host waits the library has made for this solver: host_syncs counts every wait for the
 * solver's stream to drain (each synchronising entry point: state and input copies, results,
 * set-up), throttle_waits the advance calls that found their pinned staging slot still in
 * use (the host had queued four chunks ahead of the device) and waited for it.  An advance
 * and a pg_steady_update make no host wait of the first kind. */
int pg_sync_counts(pg_solver* s, int64_t* host_syncs, int64_t* throttle_waits);

/* Number of kernel launches the last advance call issued (graph nodes included). */
int64_t pg_last_launch_count(pg_solver* s);

/* Philox-4x32-10 words for n counters (4 words each) under a 64-bit key, computed on
 * the device; counters/out are host arrays of 4*n uint32. */
int pg_philox_words(const uint32_t* counters, uint64_t key, uint32_t* out, int64_t n);

/* The two Box-Muller normals (re, im) the step kernels draw from each counter's Philox words,
 * with unit variance; out holds 2*n floats (PG_SINGLE) or doubles (PG_DOUBLE).  Test hook for
 * polarism/noise/philox.py:41-56 (normal_pair). */
int pg_wigner_normals(const uint32_t* counters, uint64_t key, int32_t precision, void* out,
                      int64_t n);

/* Uneven-size sweep.  Polarism runs each grid size of a sweep as its own batch
 * (polarism/sweep.py:98-324: grid.* overrides are non-batchable, so members are grouped and each
 * group runs through its own SimulationController and rk4-cuda launches, rk4_cuda_solver.py:
 * 1482-1536 for the per-member constants).  A pg_sweep steps members of different power-of-two
 * grids (nx in [64, 1024]) with one persistent kernel launch per RK4 step: FP32 (complex64),
 * single reservoir, no potential, a pump envelope per member.  Member m's sites occupy
 * [offset_m, offset_m + nx_m * ny_m) of the packed arrays (pg_sweep_offsets, members + 1
 * entries); psi (interleaved complex64), n_R and the envelopes all use that packing. */
typedef struct pg_sweep pg_sweep;
typedef struct pg_sweep_grid {
  int32_t nx, ny;
  double dx, dy;
} pg_sweep_grid;

int pg_sweep_create(int32_t members, const pg_sweep_grid* grids, const pg_physics* physics,
                    double dt, pg_sweep** out);
void pg_sweep_destroy(pg_sweep* w);
void* pg_sweep_stream(pg_sweep* w);
int64_t pg_sweep_total_sites(pg_sweep* w);
int pg_sweep_offsets(pg_sweep* w, int64_t* offsets);
int pg_sweep_set_state(pg_sweep* w, const void* psi, const void* res, int on_device);
int pg_sweep_get_state(pg_sweep* w, void* psi, void* res, int on_device);
int pg_sweep_state_pointers(pg_sweep* w, void** psi, void** res);
int pg_sweep_set_pump(pg_sweep* w, const void* envelope, int on_device);
/* Wigner noise per member (NoiseApplier arrays, polarism/noise/stochastic.py:15-37) with each
 * member's own cell volume dx*dy; seeds == NULL turns the noise off. */
int pg_sweep_set_noise(pg_sweep* w, const uint64_t* seeds, const double* gamma,
                       const double* scattering, const double* strength);
/* Tile shape of the persistent launch: `lanes` columns per block (512 or 1024; a block stacks
 * lanes / nx strips of equally wide members side by side, so every member needs
 * lanes / 8 <= nx <= lanes) and `strip_rows` rows per work item (>= 8).  The choice changes
 * speed only, never results.  pg_sweep_get_tiling also reports the work items and the grid. */
int pg_sweep_set_tiling(pg_sweep* w, int32_t lanes, int32_t strip_rows);
int pg_sweep_get_tiling(pg_sweep* w, int32_t* lanes, int32_t* strip_rows, int32_t* items,
                        int32_t* blocks);
/* Leave members whose entry is 0 out of the launch (their state is kept); NULL = all active. */
/* The same give-up setting for the uneven sweep's kernel (0 or 100000; see
 * pg_set_wait_limit).  Its waits are bounded the same way, but after a failure it keeps
 * copying into its ring (each later wait still bounded): completing the ring without copies
 * measured 4-6% slower on this kernel. */
int pg_sweep_set_wait_limit(pg_sweep* w, int32_t polls);
int pg_sweep_set_active(pg_sweep* w, const uint8_t* active);
/* n_steps RK4 steps (rk4_cuda_solver.py:3451-3642 semantics per member); stage_scales holds
 * [n_steps][3][members] pump coefficients at t, t + dt/2, t + dt. */
int pg_sweep_advance(pg_sweep* w, int64_t start_step, int32_t n_steps, const double* stage_scales,
                     int use_graphs);
/* Device time of the last pg_sweep_advance (CUDA events on the sweep's stream), in ms. */
int pg_sweep_last_time_ms(pg_sweep* w, float* ms);
int64_t pg_sweep_last_launch_count(pg_sweep* w);
int pg_sweep_synchronize(pg_sweep* w);
/* Per-member steady-state comparison with the previous call, as pg_steady_check. */
int pg_sweep_steady_check(pg_sweep* w, double* rel_density, double* rel_norm, double* norms);
/* The device steady-state monitor for the sweep, as pg_steady_reset / _update / _poll /
 * _results for a solver (each member's norm uses its own cell area dx * dy): no host wait
 * from reset to results, and with halt_when_all_stopped every sweep launch after the check
 * that finds every member stopped returns at once.  A run uses either these or
 * pg_sweep_steady_check.  Replaces the per-group steady-state stop of Sweep.run
 * (polarism/sweep.py:98-324 running SimulationController.run, simulation_controller.py:698-734,
 * 1063-1130). */
int pg_sweep_steady_reset(pg_sweep* w);
int pg_sweep_steady_update(pg_sweep* w, int64_t step, int32_t record, double rtol,
                           int32_t halt_when_all_stopped);
int pg_sweep_steady_poll(pg_sweep* w, int32_t* stopped, int64_t* updates_done);
int pg_sweep_steady_results(pg_sweep* w, double* rel_density, double* rel_norm, double* norms,
                            int64_t* stop_steps, int64_t* halt_step);
/* Host waits of the sweep handle, as pg_sync_counts. */
int pg_sweep_sync_counts(pg_sweep* w, int64_t* host_syncs, int64_t* throttle_waits);

/* Learned warm start (no counterpart in the reference: Polarism has no learned component).
 * Kernels of a Fourier neural operator trained on solver-made steady states.  All run
 * asynchronously on `stream` (a cudaStream_t) on caller-owned device arrays.
 *
 * pg_gemm_bf16: C = alpha op(A) op(B) + beta C for `batch` matrices (element strides
 * strideA/B/C), A, B row-major BF16 (op = transpose when transA/transB: A stored K x M, B stored
 * N x K), C row-major FP32, FP32 accumulation on the tensor cores. */
int pg_gemm_bf16(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, int32_t lda,
                 int32_t ldb, int32_t ldc, int32_t transA, int32_t transB, float alpha, float beta,
                 int32_t batch, int64_t strideA, int64_t strideB, int64_t strideC, void* stream);
/* Two-level batch: `batch` outer x `inner` inner matrices, operand offsets
 * outer * stride + inner * stride2 (a split-K reduction writes its K slices through the inner
 * level, then pg_fno_sum_slices adds them in a fixed order). */
int pg_gemm_bf16_2d(const void* A, const void* B, float* C, int32_t M, int32_t N, int32_t K, int32_t lda,
                    int32_t ldb, int32_t ldc, int32_t transA, int32_t transB, float alpha, float beta,
                    int32_t batch, int64_t strideA, int64_t strideB, int64_t strideC, int32_t inner,
                    int64_t strideA2, int64_t strideB2, int64_t strideC2, void* stream);
/* out (+)= sum of `count` consecutive slices of n floats. */
int pg_fno_sum_slices(const float* parts, float* out, int64_t n, int32_t count, int32_t accumulate,
                      void* stream);
/* GEMM engine: 0 = tcgen05.mma with FP32 accumulators in tensor memory (default), 1 = mma.sync
 * (the pre-Blackwell tensor-core path, kept as the cross-check).  pg_gemm_timeouts reports
 * (and optionally clears) whether a tcgen05 GEMM's bounded completion wait gave up; its
 * results are then invalid. */
int pg_gemm_set_engine(int32_t engine);
int pg_gemm_timeouts(int32_t* count, int32_t clear);
/* y = bf16(x) (round to nearest even). */
int pg_fno_to_bf16(const float* x, void* y, int64_t n, void* stream);
/* u[b, c, :] += bias[c] (bias may be NULL); act = GELU(u) (tanh form) if gelu else u, written to
 * act (FP32) and/or act_bf16 when not NULL.  C channels of `plane` values. */
int pg_fno_bias_act(float* u, const float* bias, float* act, void* act_bf16, int32_t C, int64_t plane,
                    int64_t n, int32_t gelu, void* stream);
/* grad_pre = grad_act * GELU'(pre) (FP32 and/or BF16 outputs). */
int pg_fno_gelu_backward(const float* pre, const float* grad_act, float* grad_pre, void* grad_bf16,
                         int64_t n, void* stream);
/* out[c] (+)= sum over b and the plane of x[b, c, :]. */
int pg_fno_channel_sum(const float* x, float* out, int32_t B, int32_t C, int64_t plane, int32_t accumulate,
                       void* stream);
/* Per-mode complex mixing of the kept spectrum: out[b, o, k] = sum_i y[b, i, k] w[k, i, o].
 * Spectra are [b][channel][ky (2 modes)][kx re (modes) | kx im (modes)]; BF16 weights
 * [ky][kx][in][out] as separate real and imaginary arrays. */
int pg_fno_mode_mix(const float* y, const void* wre, const void* wim, float* out, int32_t B, int32_t cin,
                    int32_t cout, int32_t modes, void* stream);
/* Adjoints: dy = dout conj(w) (if dy != NULL), dw = conj(y) dout summed over b (if dwre/dwim). */
int pg_fno_mode_mix_backward(const float* y, const float* dout, const void* wre, const void* wim, float* dy,
                             float* dwre, float* dwim, int32_t B, int32_t cin, int32_t cout, int32_t modes,
                             void* stream);
/* Adam on FP32 weights (bias-corrected, optional L2 decay), refreshing the BF16 copy. */
int pg_fno_adam(float* w, const float* g, float* m1, float* m2, void* w_bf16, int64_t n, float lr,
                float beta1, float beta2, float eps, int64_t step, float decay, void* stream);
/* Weighted squared error over C channels of `plane` values: grad = 2 w_c (pred - target) scale;
 * per-block FP64 partial sums of w_c (pred - target)^2 in partials (blocks_used entries). */
int pg_fno_mse(const float* pred, const float* target, const float* weight, int32_t C, int64_t plane,
               float* grad, void* grad_bf16, double* partials, int32_t max_partials, int64_t n, float scale,
               int32_t* blocks_used, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* POLARISM_GB300_H */
