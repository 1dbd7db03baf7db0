/*
 * amx -- GB300-native MHD step of astronomix, C ABI.
 *
 * Plain C: integers, doubles, opaque handles and raw device pointers.  No
 * torch, JAX or C++ types cross this boundary and nothing here throws.
 *
 * Every entry point returns 0 on success or a bitwise OR of AMX_ERR_* codes.
 * Device-side numerical conditions (NaN, fixed-point cap, barrier timeout)
 * are accumulated in the plan's status word and read with amx_status().
 * Entry points are stream-ordered on the caller's stream (a cudaStream_t
 * passed as void*); none of them synchronises the stream unless its comment
 * says so.
 *
 * State arrays are the reference's layout: state[var][x][y][z], C order,
 * without ghost cells, in float32 or float64 (amx_config.dtype), with the
 * row order of astronomix/variable_registry/registered_variables.py:116-238.
 */
#ifndef AMX_H_
#define AMX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status / error bits ------------------------------------------------ */
#define AMX_OK 0
#define AMX_ERR_INVALID_ARG (1 << 0)   /* bad pointer, size or option      */
#define AMX_ERR_CUDA (1 << 1)          /* a CUDA runtime call failed       */
#define AMX_ERR_NAN (1 << 2)           /* non-finite value met on device   */
#define AMX_ERR_NEGATIVE (1 << 3)      /* negative density or pressure     */
#define AMX_ERR_NOT_CONVERGED (1 << 4) /* magnetic fixed point hit its cap */
#define AMX_ERR_TIMEOUT (1 << 5)       /* bounded grid barrier gave up     */
#define AMX_ERR_BOUNDS (1 << 6)        /* index check failed               */
#define AMX_ERR_UNSUPPORTED (1 << 7)   /* option outside the kernels       */
#define AMX_ERR_TOO_LARGE (1 << 8)     /* size above a fixed limit         */

/* ---- enumerations (values equal the reference's constants,
 *      astronomix/option_classes/simulation_config.py:20-93) --------------- */
#define AMX_F32 0
#define AMX_F64 1

#define AMX_FINITE_VOLUME 0
#define AMX_FINITE_DIFFERENCE 1

#define AMX_HLL 0
#define AMX_HLLC 1
#define AMX_HLLC_LM 2
#define AMX_LAX_FRIEDRICHS 3
#define AMX_HYBRID_HLLC 4  /* HLLC-LM where the cell right of a face is compressed, HLLC elsewhere */
#define AMX_AM_HLLC 5      /* HYBRID_HLLC with the low-Mach dissipation control */

#define AMX_MINMOD 0
#define AMX_OSHER 1
#define AMX_DOUBLE_MINMOD 2
#define AMX_SUPERBEE 3
#define AMX_VAN_ALBADA 4
#define AMX_VAN_ALBADA_PP 5  /* positivity-preserving multidimensional (unsplit, 2D / 3D) */

#define AMX_BC_OPEN 0
#define AMX_BC_REFLECTIVE 1
#define AMX_BC_PERIODIC 2

#define AMX_GHOST_CELLS 0
#define AMX_PERIODIC_ROLL 1

#define AMX_IMPLICIT_MIDPOINT 0
#define AMX_IMPLICIT_EULER 1

/* self-gravity source-term versions (simulation_config.py, self_gravity_version) */
#define AMX_SIMPLE_SOURCE_TERM 0
#define AMX_DONOR_ACCOUNTING 1
#define AMX_RIEMANN_SPLIT 2
#define AMX_RIEMANN_SPLIT_UNSTABLE 3
#define AMX_HALF_SPLIT 4

/* Static configuration: the fields of SimulationConfig that select kernels
 * (astronomix/option_classes/simulation_config.py:160-342). */
typedef struct amx_config {
  int32_t solver_mode;            /* AMX_FINITE_VOLUME / AMX_FINITE_DIFFERENCE  */
  int32_t dtype;                  /* AMX_F32 / AMX_F64 (storage and arithmetic) */
  int32_t dimensionality;         /* 1, 2 or 3                                  */
  int32_t num_cells;              /* cells per axis (square / cubic grids)      */
  int32_t num_vars;               /* rows of the state array                    */
  int32_t mhd;                    /* 0 / 1                                      */
  int32_t riemann_solver;         /* AMX_HLL .. AMX_AM_HLLC                     */
  int32_t limiter;                /* AMX_MINMOD .. AMX_VAN_ALBADA_PP            */
  int32_t fv_magnetic_integrator; /* AMX_IMPLICIT_MIDPOINT / _EULER             */
  int32_t numerical_precision;    /* 0: fixed-point tol 1e-5, 1: 1e-10          */
  int32_t boundary_handling;      /* AMX_GHOST_CELLS / AMX_PERIODIC_ROLL        */
  int32_t bc_lo[3];               /* per axis AMX_BC_*                          */
  int32_t bc_hi[3];
  int32_t enforce_positivity;     /* FD floors                                  */
  int32_t exact_end_time;
  int32_t fixed_timestep;
  int32_t num_timesteps;
  double box_size;
  double grid_spacing;            /* box_size / num_cells                       */
  int32_t split;                  /* FV: 0 unsplit (SSP-RK2), 1 split (MUSCL-Hancock sweeps) */
  int32_t first_order_fallback;   /* split: piecewise-constant interface states */
  int32_t use_max_adaptive_timestep; /* split: dt = min(dt, dt_max)            */
  int32_t self_gravity;           /* FV: 0 / 1, the source term after every gas update */
  int32_t self_gravity_version;   /* AMX_SIMPLE_SOURCE_TERM .. AMX_HALF_SPLIT  */
  int32_t stellar_wind;           /* FD (3D): the EI wind source in every stage's right-hand side */
  int32_t num_injection_cells;    /* wind injection radius in cells            */
  int32_t turbulent_forcing;      /* 3D: solenoidal forcing before every step  */
  int32_t reserved;
} amx_config;

/* Traced parameters (astronomix/option_classes/simulation_params.py:11-66). */
typedef struct amx_params {
  double C_cfl;
  double gamma;
  double minimum_density;
  double minimum_pressure;
  double dt_max;
  double t_end;
  double gravitational_constant;  /* self-gravity G                        */
  double wind_mass_loss_rate;     /* stellar wind (WindParams)             */
  double wind_final_velocity;
  double energy_injection_rate;   /* turbulent forcing (TurbulentForcingParams) */
  int64_t forcing_seed;           /* key of the forcing's random stream    */
} amx_params;

/* Result of a time-integration call. */
typedef struct amx_run_info {
  double t;                       /* simulation time reached              */
  double last_dt;                 /* dt of the last step                  */
  int64_t steps;                  /* total steps taken by this plan       */
  int64_t magnetic_iterations;    /* total FV fixed-point iterations      */
  int32_t last_magnetic_iterations;
  int32_t status;                 /* AMX_ERR_* bits seen on the device    */
} amx_run_info;

typedef struct amx_plan amx_plan;

/* ---- plan lifecycle ----------------------------------------------------- */

/* Validates `cfg` (the checks of finalize_config,
 * astronomix/option_classes/simulation_config.py:345-470, that concern the
 * kernels) and allocates the plan's device workspace on the current device.
 * `max_history` (>= 0) sizes the per-step dt / iteration record. */
int amx_plan_create(const amx_config* cfg, int64_t max_history, amx_plan** out);
int amx_plan_destroy(amx_plan* plan);
/* No counterpart in the reference.  Limits of the FV persistent kernel:
 * the cap on magnetic fixed-point iterations per update (the reference's
 * 1000, _magnetic_field_update.py:141; reaching it sets
 * AMX_ERR_NOT_CONVERGED) and the polls a block makes at a grid barrier
 * before it gives up with AMX_ERR_TIMEOUT (2^24).  0 restores a default.
 * For tests of the failure paths and for callers that want an earlier
 * timeout; AMX_ERR_UNSUPPORTED for an FD plan (no fixed point, no barrier). */
int amx_plan_set_limits(amx_plan* plan, int32_t max_fixed_point_iterations, int64_t barrier_spin_limit);
/* No counterpart in the reference.  Per-kernel timing of the FD step: with
 * amx_plan_profile(plan, 1), every amx_run / amx_run_until / amx_run_async
 * step of an FD plan records a CUDA event after each of its launches on the
 * caller's stream and waits for the step's last event (so steps no longer
 * overlap host work); amx_plan_profile_read copies, per kernel kind, the
 * summed milliseconds and the launch counts since the last reset into
 * ms[n] / launches[n] (either may be null): 0 CFL, 1 stage prep, 2-4 WENO
 * x / y / z, 5 edge EMF, 6 EMF averages, 7 wind source, 8 stage update,
 * 9 finalize, 10 turbulent forcing, 11 time advance.  AMX_ERR_UNSUPPORTED for an FV plan
 * (one persistent launch per step). */
int amx_plan_profile(amx_plan* plan, int32_t enable);
int amx_plan_profile_read(amx_plan* plan, double* ms, int64_t* launches, int32_t n, int32_t reset);
/* Bytes of device workspace the plan holds. */
int amx_plan_workspace_bytes(const amx_plan* plan, size_t* bytes);
/* Resets time, step counters, history and status to zero (stream-ordered). */
int amx_plan_reset(amx_plan* plan, void* stream);
/* Sets the time accumulator (used by drivers that restart a run). */
int amx_plan_set_time(amx_plan* plan, double t, void* stream);

/* ---- step-level seams ---------------------------------------------------- */

/* Replaces _cfl_time_step, astronomix/_finite_volume/_timestep_estimation/
 * _timestep_estimator.py:95-218 (UNSPLIT branch), and _cfl_time_step_fd,
 * astronomix/_finite_difference/_timestep_estimation/_timestep_estimator.py:26-91.
 * Writes the FP64 dt to *dt_host (synchronises the stream). */
int amx_cfl_dt(amx_plan* plan, const void* state, const amx_params* prm, double* dt_host,
               void* stream);

/* Replaces _evolve_gas_state_unsplit (one SSP-RK2 update of the gas rows),
 * astronomix/_finite_volume/_state_evolution/evolve_state.py:419-488, with
 * time step dt (with split = 1 the Strang sweeps of _evolve_gas_state_split,
 * :167-336; with self_gravity followed by the gravitational source term).
 * `state` holds the full state; only gas rows change. */
int amx_fv_hydro_rk2(amx_plan* plan, void* state, const amx_params* prm, double dt, void* stream);

/* Replaces magnetic_update,
 * astronomix/_finite_volume/_magnetic_update/_magnetic_field_update.py:37-242.
 * Updates B rows, gas velocity and pressure in place. */
int amx_fv_magnetic_update(amx_plan* plan, void* state, const amx_params* prm, double dt,
                           void* stream);

/* Replaces _evolve_state_fv,
 * astronomix/_finite_volume/_state_evolution/evolve_state.py:497-600, and
 * _evolve_state_fd, astronomix/_finite_difference/_state_evolution/
 * _evolve_state.py:25-73: one step of size dt, in place. */
int amx_evolve_state(amx_plan* plan, void* state, const amx_params* prm, double dt, void* stream);

/* ---- time driver --------------------------------------------------------- */

/* Replaces the loop of _time_integration,
 * astronomix/time_stepping/time_integration.py:386-801 (adaptive dt with
 * exact end time, or the fixed-step loop): advances `state` in place until
 * t >= prm->t_end or `max_steps` more steps were taken, without a host round
 * trip per step.  Synchronises the stream and fills *info when non-null.
 * With self_gravity a step is a stream-ordered sequence of launches (the
 * Poisson solve sits between the persistent kernel's phases) with dt, t and
 * the decision to step on the device; the host checks t after 1, 2, 4 ..
 * 32 steps. */
int amx_run(amx_plan* plan, void* state, const amx_params* prm, int64_t max_steps,
            amx_run_info* info, void* stream);

/* amx_run that also stops before the first step starting at t >= t_pause
 * (the snapshot points of time_integration.py:556-566). */
int amx_run_until(amx_plan* plan, void* state, const amx_params* prm, int64_t max_steps, double t_pause,
                  amx_run_info* info, void* stream);

/* Like amx_run but does not synchronise: launches exactly the work of
 * `max_steps` steps (steps after t_end are skipped on the device).  For
 * timing and for callers that overlap host work.  With self_gravity at most
 * 2^20 steps per call (AMX_ERR_TOO_LARGE above). */
int amx_run_async(amx_plan* plan, void* state, const amx_params* prm, int64_t max_steps,
                  void* stream);

/* Copies the per-step dt record (FP64) and fixed-point iteration counts of
 * the steps taken since the last reset into host arrays of length `n`
 * (synchronises).  Either pointer may be null. */
int amx_history(amx_plan* plan, double* dt_host, int32_t* iters_host, int64_t n, void* stream);

/* ---- diagnostics ---------------------------------------------------------- */

/* FP64 global sums of the state (astronomix/_fluid_equations/total_quantities.py:
 * 31-176): out[0] = total mass, out[1] = total energy, out[2] = kinetic
 * energy, out[3] = internal energy, out[4] = max |div B| (0 without MHD).
 * Synchronises the stream. */
int amx_conservation_sums(amx_plan* plan, const void* state, const amx_params* prm,
                          double out_host[5], void* stream);

/* Reads (and with clear != 0 resets) the plan's device status bits.
 * Synchronises the stream. */
int amx_status(amx_plan* plan, int32_t* status_host, int32_t clear, void* stream);

/* ---- allocation-free variant ----------------------------------------------- */

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory: a framework that owns the GPU's memory and forbids allocations
 * behind its back (XLA preallocates most of the device; a JAX custom call
 * must not take more), a process held to a fixed device-memory budget, or a
 * loop that cannot afford an allocation's implicit synchronisation.  Runs
 * `max_steps` FV time steps of `state` in place, like amx_run_async, without
 * a plan.  Its scratch is a fixed 8 MiB __device__ array inside the library,
 * shared by every call on a device (calls that overlap on the GPU race on
 * it; each call clears what must start at zero); configurations that need
 * more return AMX_ERR_TOO_LARGE (2D MHD fits up to 362^2 cells in FP32 and
 * 255^2 in FP64; 3D MHD up to 49^3 / 39^3).  The first call on each device
 * resolves the array's device address; make it before any stream capture.
 * Fills *info (and synchronises) when info is non-null; since a stream that
 * is being captured may not be synchronised, such a call on a capturing
 * stream returns AMX_ERR_INVALID_ARG without launching anything.  Accepts what amx_plan_create accepts for the FV
 * scheme (including VAN_ALBADA_PP), except self_gravity, turbulent_forcing
 * and stellar_wind (AMX_ERR_UNSUPPORTED: they need cuFFT work between the
 * kernel's phases) and FD configurations. */
int amx_fv_run_noalloc(const amx_config* cfg, void* state, const amx_params* prm, int64_t max_steps,
                       amx_run_info* info, void* stream);

/* ---- batched ensemble ----------------------------------------------------- */

/* No counterpart in the reference, which integrates one simulation per
 * time_integration call (astronomix/time_stepping/time_integration.py:61-236);
 * an ensemble there is a Python loop over that call.  A batch advances up to
 * 256 independent 2D FV runs of uneven grid sizes with one persistent
 * cooperative launch.  Every run follows amx_run exactly (bit-identical
 * results) with its own dt, time, end time and fixed-point iteration count.
 * The runs share the template configuration `tmpl` (dtype, MHD, HLL / HLLC /
 * HLLC-LM, limiter, boundaries, magnetic integrator; adaptive dt only) and
 * the parameters other than t_end; run r has num_cells[r]^2 cells on a box of
 * side box_size[r] (tmpl->num_cells and tmpl->grid_spacing are ignored). */
typedef struct amx_batch amx_batch;
int amx_batch_create(const amx_config* tmpl, int32_t num_runs, const int32_t* num_cells, const double* box_size,
                     amx_batch** out);
int amx_batch_destroy(amx_batch* batch);
int amx_batch_workspace_bytes(const amx_batch* batch, size_t* bytes);
/* Time, step counters and status of every run back to zero (stream-ordered). */
int amx_batch_reset(amx_batch* batch, void* stream);
/* Advances every run r (states[r]: device state of run r, in place) until
 * t_r >= t_end[r], or for at most `max_steps` lock-step steps, in one
 * cooperative launch.  With use_graph != 0 the launch is captured once into
 * a CUDA graph and replayed while the arguments and the tiling stay the same.
 * Does not synchronise. */
int amx_batch_run(amx_batch* batch, void* const* states, const amx_params* prm, const double* t_end,
                  int64_t max_steps, int32_t use_graph, void* stream);
/* Per-run progress (infos[num_runs]) and the lock-step steps taken so far
 * (synchronises). */
int amx_batch_info(amx_batch* batch, amx_run_info* infos, int64_t* lock_steps, void* stream);
/* Autotuner: times `steps` lock-step steps of copies of the states under
 * every compiled tile shape and resident-block count and keeps the fastest
 * (the states and counters are left as they were; *best_ms, if non-null,
 * gets the winning time).  Synchronises. */
int amx_batch_tune(amx_batch* batch, void* const* states, const amx_params* prm, const double* t_end,
                   int32_t steps, double* best_ms, void* stream);
/* Current tiling: shape variant, resident blocks per SM, tile extent. */
int amx_batch_tiling(const amx_batch* batch, int32_t* variant, int32_t* blocks_per_sm, int32_t* tile0,
                     int32_t* tile1);
/* Forces a tiling (blocks_per_sm <= 0 picks the default). */
int amx_batch_set_tiling(amx_batch* batch, int32_t variant, int32_t blocks_per_sm);

/* ---- discrete adjoint --------------------------------------------------------- */

/* Reverse-mode gradient of the FV time integration (2D / 3D, HLL, MINMOD,
 * periodic; MHD or hydro).  The reference differentiates time_integration
 * with jax.grad (tests/mhd_tests/mhd_correct.py:237-264): dt is held fixed
 * (stop_gradient, astronomix/time_stepping/time_integration.py:632-661) and
 * the magnetic fixed point is differentiated through the iterations it took
 * (its while loop, _magnetic_field_update.py:127-171).  This is the
 * hand-written discrete adjoint of the same program.  amx_adjoint_forward runs
 * the ordinary kernel to t_end, keeping the state every `checkpoint_every`
 * steps and the dt / iteration schedule; amx_adjoint_backward maps the
 * cotangent of the final state (full state layout) to the cotangent of the
 * initial state, replaying one segment at a time from its checkpoint.
 * `max_steps` bounds the schedule. */
typedef struct amx_adjoint amx_adjoint;
int amx_adjoint_create(const amx_config* cfg, int32_t checkpoint_every, int64_t max_steps, amx_adjoint** out);
int amx_adjoint_destroy(amx_adjoint* adj);
/* Advances `state` in place to prm->t_end, recording checkpoints and the
 * schedule (synchronises; fills *info when non-null). */
int amx_adjoint_forward(amx_adjoint* adj, void* state, const amx_params* prm, amx_run_info* info, void* stream);
/* grad_initial = (d final / d initial)^T grad_final for the last forward
 * (device buffers in the state layout; synchronises). */
int amx_adjoint_backward(amx_adjoint* adj, const void* grad_final, void* grad_initial, void* stream);
/* Advances `state` in place with the recorded schedule (fixed dt and
 * iteration counts): the program the gradient is exact for (synchronises). */
int amx_adjoint_replay(amx_adjoint* adj, void* state, void* stream);
/* Device bytes the forward may use to store the whole tape (every
 * intermediate state of every step, written by the forward kernel itself).
 * When the run fits, the backward reads the stored tape and recomputes
 * nothing; otherwise (and with 0, the default) the forward keeps
 * checkpoints and the backward replays one segment at a time. */
int amx_adjoint_set_tape_budget(amx_adjoint* adj, size_t bytes);
/* *yes = 1 when the last forward stored the whole tape. */
int amx_adjoint_uses_stored_tape(const amx_adjoint* adj, int32_t* yes);
/* Steps of the last forward, and the first n dt / iteration counts. */
int amx_adjoint_schedule(amx_adjoint* adj, double* dt_host, int32_t* iters_host, int64_t n, int64_t* steps);
/* Device bytes held for checkpoints and for the tape and cotangents. */
int amx_adjoint_memory(const amx_adjoint* adj, size_t* checkpoint_bytes, size_t* tape_bytes);

/* ---- self-gravity: the Poisson solve -------------------------------------
 *
 * Replaces _compute_gravitational_potential
 * (astronomix/_physics_modules/_self_gravity/_poisson_solver.py:17-151):
 * with `periodic` the FFT solve of lap(phi) = 4 pi G (rho - mean(rho)) with
 * the reference's Green's function (-4 pi G / k^2, -1 / (4 pi) at k = 0);
 * otherwise the Hockney-Eastwood convolution with the isolated kernel
 * (-2 pi G r, -2 G log r, -G / r; r = 0 replaced by dx) on the grid padded
 * to twice its size, scaled by dx^d.  cuFFT transforms (R2C / C2R) on the
 * device.  Runs with amx_config.self_gravity use the same solver on the
 * grid the reference solves on (the padded grid with ghost-cell handling). */
typedef struct amx_poisson amx_poisson;
int amx_poisson_create(int32_t dimensionality, int32_t num_cells, double grid_spacing, int32_t periodic,
                       int32_t dtype, amx_poisson** out);
int amx_poisson_destroy(amx_poisson* solver);
/* density, potential: device arrays of num_cells^d values (C order). */
int amx_poisson_solve(amx_poisson* solver, const void* density, void* potential, double G, void* stream);

/* ---- measurement ---------------------------------------------------------- */

/* No counterpart in the reference: the FP32 FMA throughput of the current GPU
 * in TFLOP/s (a timed kernel of independent FMA chains), the compute roof of
 * the FD WENO kernel.  Synchronises. */
int amx_probe_fp32_fma(double* tflops, void* stream);

/* Library version string. */
const char* amx_version(void);

#ifdef __cplusplus
}
#endif

#endif /* AMX_H_ */
