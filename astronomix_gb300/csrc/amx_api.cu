// C-ABI implementation: plans, workspace and launches (host code).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>

#include "../../include/amx.h"
#include "amx_common.cuh"
#include "fd_api.h"
#include "fv_kernels.cuh"
#include "fv_registry.h"
#include "forcing.h"
#include "gravity.h"
#include "validate.h"

extern "C" int amx_diag_sums_raw(const amx_config* cfg, const void* state, double gamma, double* out_dev,
                                 void* stream);

using amx::FVControl;
using amx::FVKernelInfo;

struct amx_plan {
  amx_config cfg;
  int device = 0;
  int num_sms = 0;
  size_t elem = 4;          // bytes per value
  long long ncells = 0;
  size_t ws_bytes = 0;
  unsigned char* ws = nullptr;
  // FV
  void* p1 = nullptr;
  void* mag0 = nullptr;
  void* mag1 = nullptr;
  FVControl* ctl = nullptr;
  double* dt_hist = nullptr;
  int* it_hist = nullptr;
  int64_t max_hist = 0;
  FVKernelInfo fv{};
  int fv_grid = 0;
  double* diag = nullptr;   // 8 doubles of reduction scratch for amx_conservation_sums
  // FD
  amx::FDPlan* fd = nullptr;
  // limits of the persistent kernel (amx_plan_set_limits)
  int max_iters = 1000;                                    // the reference's fixed-point cap
  unsigned long long spin_limit = AMX_BARRIER_SPIN_LIMIT;  // polls per grid barrier
  // FV self-gravity and turbulent forcing (null without)
  amx::GravPlan* grav = nullptr;
  amx::ForcingPlan* force = nullptr;
};

namespace {

inline int cuda_ok(cudaError_t e) { return e == cudaSuccess ? AMX_OK : AMX_ERR_CUDA; }

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

long long ipow(long long b, int e) {
  long long r = 1;
  while (e-- > 0) r *= b;
  return r;
}

template <typename T>
amx::FVArgs<T> make_fv_args(amx_plan* p, void* state, const amx_params* prm, int mode) {
  amx::FVArgs<T> a{};
  const amx_config& c = p->cfg;
  a.state = static_cast<T*>(state);
  a.p1 = static_cast<T*>(p->p1);
  a.mag0 = static_cast<T*>(p->mag0);
  a.mag1 = static_cast<T*>(p->mag1);
  a.ctl = p->ctl;
  a.dt_hist = p->dt_hist;
  a.it_hist = p->it_hist;
  a.max_hist = p->max_hist;
  a.n = c.num_cells;
  a.ncells = p->ncells;
  for (int k = 0; k < 3; ++k) a.bc[k] = amx::AxisBC{c.bc_lo[k], c.bc_hi[k]};
  a.periodic_roll = (c.boundary_handling == AMX_PERIODIC_ROLL);
  a.limiter = c.limiter;
  a.integrator = c.fv_magnetic_integrator;
  a.lm = (c.riemann_solver == AMX_HLLC_LM);
  a.am = (c.riemann_solver == AMX_AM_HLLC) ? 1 : (c.riemann_solver == AMX_HYBRID_HLLC ? 2 : 0);
  a.exact_end_time = c.exact_end_time;
  a.fixed_timestep = c.fixed_timestep;
  a.mode = mode;
  a.dx = c.grid_spacing;
  a.inv_dx = 1.0 / c.grid_spacing;
  a.gamma = prm->gamma;
  a.C_cfl = prm->C_cfl;
  a.t_end = prm->t_end;
  a.dt_fixed = c.num_timesteps > 0 ? prm->t_end / c.num_timesteps : 0.0;
  a.dt_in = 0.0;
  a.dt_scale = 1.0;
  a.tol = (c.numerical_precision == 1) ? 1e-10 : 1e-5;
  a.max_iters = p->max_iters;
  a.spin_limit = p->spin_limit;
  a.mhd = c.mhd;
  a.split = c.split;
  a.first_order = c.first_order_fallback;
  a.use_dt_max = c.use_max_adaptive_timestep;
  a.dt_max = prm->dt_max;
  a.p2 = static_cast<T*>(p->mag0);  // the split sweeps' third buffer (free outside the magnetic update)
  a.max_steps = 0;
  a.t_pause = INFINITY;
  return a;
}

// zero the reduction slots and the barrier before a cooperative launch (the
// leading members of FVControl, up to dt)
int fv_prepare(amx_plan* p, cudaStream_t s) {
  return cuda_ok(cudaMemsetAsync(p->ctl, 0, offsetof(FVControl, dt), s));
}

template <typename T>
int fv_launch(amx_plan* p, amx::FVArgs<T>& a, cudaStream_t s) {
  int rc = fv_prepare(p, s);
  if (rc) return rc;
  void* args[] = {&a};
  cudaError_t e = cudaLaunchCooperativeKernel(p->fv.fn, dim3(p->fv_grid), dim3(amx::kFVThreads), args,
                                              p->fv.smem, s);
  return cuda_ok(e);
}

int fv_run_mode(amx_plan* p, void* state, const amx_params* prm, int mode, double dt_in, double dt_scale,
                long long max_steps, bool with_hist, cudaStream_t s) {
  if (p->cfg.dtype == AMX_F32) {
    auto a = make_fv_args<float>(p, state, prm, mode);
    a.dt_in = dt_in;
    a.dt_scale = dt_scale;
    a.max_steps = max_steps;
    return fv_launch(p, a, s);
  }
  auto a = make_fv_args<double>(p, state, prm, mode);
  a.dt_in = dt_in;
  a.dt_scale = dt_scale;
  a.max_steps = max_steps;
  (void)with_hist;
  return fv_launch(p, a, s);
}

// The end of a device-driven step: t += dt, the step count and the history
// records (when ctl->active).
__global__ void k_step_advance(FVControl* ctl, double* dt_hist, int* it_hist, long long max_hist, int mhd) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (!ctl->active) return;
  const double dt = ctl->dt;
  ctl->t = ctl->t + dt;
  const long long idx = ctl->steps;
  ctl->steps = idx + 1;
  const int it = mhd ? ctl->mag_iters : 0;
  ctl->mag_iters_total += it;
  if (dt_hist && idx < max_hist) dt_hist[idx] = dt;
  if (it_hist && idx < max_hist) it_hist[idx] = it;
}

// A device-driven seam (dt from ctl->dt times dt_scale; skipped unless ctl->active).
int fv_seam(amx_plan* p, void* state, const amx_params* prm, int mode, double dt_scale, double t_pause,
            cudaStream_t s) {
  if (p->cfg.dtype == AMX_F32) {
    auto a = make_fv_args<float>(p, state, prm, mode);
    a.dt_dev = 1;
    a.dt_scale = dt_scale;
    a.t_pause = t_pause;
    return fv_launch(p, a, s);
  }
  auto a = make_fv_args<double>(p, state, prm, mode);
  a.dt_dev = 1;
  a.dt_scale = dt_scale;
  a.t_pause = t_pause;
  return fv_launch(p, a, s);
}

// One device-driven step (time_integration.py:626-762) for runs whose step
// needs work between the persistent kernel's phases: self-gravity (the
// Poisson solve after each gas update, evolve_state.py:178-322, 429-487) and
// turbulent forcing (before the evolve, :700-711), both cuFFT-based.  The
// step is a stream-ordered sequence of launches with dt, t and the decision
// to step kept on the device: dt (FV_MODE_DT), the forcing, then with
// gravity per gas update a copy of the gas rows, the hydro seam and the
// source term (the magnetic seam between the two half updates with MHD),
// without gravity the evolve seam; and the time advance.  `evolve_only`: one
// _evolve_state_fv with the dt already in ctl->dt (no dt, no forcing, no
// advance).
int fv_device_step(amx_plan* p, void* state, const amx_params* prm, double t_pause, bool evolve_only,
                   cudaStream_t s) {
  int rc = AMX_OK;
  if (!evolve_only) {
    rc = fv_seam(p, state, prm, amx::FV_MODE_DT, 1.0, t_pause, s);
    if (!rc && p->force)
      rc = amx::forcing_apply(p->force, state, &p->ctl->dt, &p->ctl->active, &p->ctl->steps, *prm, s);
    if (rc) return rc;
  }
  if (!p->grav) {
    rc = fv_seam(p, state, prm, amx::FV_MODE_EVOLVE, 1.0, INFINITY, s);
  } else {
    const size_t gas_bytes = (size_t)(p->cfg.dimensionality + 2) * (size_t)p->ncells * p->elem;
    void* old = amx::grav_old_state(p->grav);
    const double h = p->cfg.mhd ? 0.5 : 1.0;
    rc |= cuda_ok(cudaMemcpyAsync(old, state, gas_bytes, cudaMemcpyDeviceToDevice, s));
    rc |= fv_seam(p, state, prm, amx::FV_MODE_HYDRO_RK2, h, INFINITY, s);
    rc |= amx::grav_apply(p->grav, old, state, p->ctl, h, *prm, s);
    if (rc) return rc;
    if (p->cfg.mhd) {
      rc |= fv_seam(p, state, prm, amx::FV_MODE_MAGNETIC, 1.0, INFINITY, s);
      rc |= cuda_ok(cudaMemcpyAsync(old, state, gas_bytes, cudaMemcpyDeviceToDevice, s));
      rc |= fv_seam(p, state, prm, amx::FV_MODE_HYDRO_RK2, h, INFINITY, s);
      rc |= amx::grav_apply(p->grav, old, state, p->ctl, h, *prm, s);
    }
  }
  if (rc) return rc;
  if (!evolve_only) {
    k_step_advance<<<1, 32, 0, s>>>(p->ctl, p->dt_hist, p->it_hist, p->max_hist, p->cfg.mhd);
    rc = cuda_ok(cudaGetLastError());
  }
  return rc;
}

}  // namespace

// ====================================================================== ABI

extern "C" {

const char* amx_version(void) { return "amx 0.1.0 (sm_103a)"; }

int amx_plan_create(const amx_config* cfg, int64_t max_history, amx_plan** out) {
  if (!out) return AMX_ERR_INVALID_ARG;
  *out = nullptr;
  int rc = amx::validate_config(cfg);
  if (rc) return rc;
  if (max_history < 0) return AMX_ERR_INVALID_ARG;
  amx_plan* p = new (std::nothrow) amx_plan();
  if (!p) return AMX_ERR_INVALID_ARG;
  p->cfg = *cfg;
  p->elem = cfg->dtype == AMX_F32 ? 4 : 8;
  p->ncells = ipow(cfg->num_cells, cfg->dimensionality);
  if (cudaGetDevice(&p->device) != cudaSuccess) { delete p; return AMX_ERR_CUDA; }
  cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, p->device);
  if (cudaMalloc(&p->diag, 8 * sizeof(double)) != cudaSuccess) { delete p; return AMX_ERR_CUDA; }

  if (cfg->solver_mode == AMX_FINITE_DIFFERENCE) {
    rc = amx::fd_plan_create(*cfg, max_history, &p->fd);
    if (rc) { cudaFree(p->diag); delete p; return rc; }
    *out = p;
    return AMX_OK;
  }

  // ---- FV kernel selection
  const int rs = amx::fv_riemann_family(cfg->riemann_solver);
  const int scheme = cfg->split ? amx::FV_SPLIT
                                 : (cfg->limiter == AMX_VAN_ALBADA_PP ? amx::FV_UNSPLIT_PP : amx::FV_UNSPLIT);
  const bool ok = (cfg->dtype == AMX_F32)
                      ? amx::fv_kernel_f32(cfg->dimensionality, rs, cfg->mhd != 0, scheme, &p->fv)
                      : amx::fv_kernel_f64(cfg->dimensionality, rs, cfg->mhd != 0, scheme, &p->fv);
  if (!ok) { amx_plan_destroy(p); return AMX_ERR_UNSUPPORTED; }
  if (cfg->limiter == AMX_VAN_ALBADA_PP && !cfg->split) p->fv.smem += p->fv.smem_pp;
  if (cudaFuncSetAttribute(p->fv.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->fv.smem) != cudaSuccess) {
    amx_plan_destroy(p);
    return AMX_ERR_CUDA;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, p->fv.fn, amx::kFVThreads, p->fv.smem) != cudaSuccess ||
      per_sm < 1) {
    amx_plan_destroy(p);
    return AMX_ERR_CUDA;
  }
  // AMX_FV_BLOCKS_PER_SM (optional) caps the resident blocks per SM of the
  // persistent kernel: fewer blocks make the grid barrier cheaper, more hide
  // latency better.
  if (const char* env = std::getenv("AMX_FV_BLOCKS_PER_SM")) {
    const int want = std::atoi(env);
    if (want >= 1 && want < per_sm) per_sm = want;
  }
  const long long cap = (long long)per_sm * p->num_sms;
  const long long need = std::max<long long>(1, (p->ncells + amx::kFVThreads - 1) / amx::kFVThreads);
  p->fv_grid = (int)std::min<long long>(cap, need);

  // ---- workspace: stage buffer, two magnetic iterate buffers, control, history
  const int nv_gas = cfg->dimensionality + 2;
  const size_t field = (size_t)p->ncells * p->elem;
  size_t off = 0;
  const size_t o_p1 = off; off = align256(off + nv_gas * field);
  const size_t o_m0 = off; off = align256(off + (cfg->mhd ? 6 : (cfg->split ? nv_gas : 0)) * field);
  const size_t o_m1 = off; off = align256(off + (cfg->mhd ? 6 : 0) * field);
  const size_t o_ctl = off; off = align256(off + sizeof(FVControl));
  const size_t o_dth = off; off = align256(off + sizeof(double) * (size_t)max_history);
  const size_t o_ith = off; off = align256(off + sizeof(int) * (size_t)max_history);
  p->ws_bytes = off;
  if (cudaMalloc(&p->ws, p->ws_bytes) != cudaSuccess) { amx_plan_destroy(p); return AMX_ERR_CUDA; }
  cudaMemset(p->ws, 0, p->ws_bytes);
  p->p1 = p->ws + o_p1;
  p->mag0 = p->ws + o_m0;
  p->mag1 = p->ws + o_m1;
  p->ctl = reinterpret_cast<FVControl*>(p->ws + o_ctl);
  p->max_hist = max_history;
  p->dt_hist = max_history ? reinterpret_cast<double*>(p->ws + o_dth) : nullptr;
  p->it_hist = max_history ? reinterpret_cast<int*>(p->ws + o_ith) : nullptr;
  if (cfg->self_gravity) {
    rc = amx::grav_plan_create(*cfg, &p->grav);
    if (rc) { amx_plan_destroy(p); return rc; }
  }
  if (cfg->turbulent_forcing) {
    rc = amx::forcing_plan_create(*cfg, &p->force);
    if (rc) { amx_plan_destroy(p); return rc; }
  }
  if (cudaDeviceSynchronize() != cudaSuccess) { amx_plan_destroy(p); return AMX_ERR_CUDA; }
  *out = p;
  return AMX_OK;
}

int amx_plan_destroy(amx_plan* p) {
  if (!p) return AMX_OK;
  if (p->diag) cudaFree(p->diag);
  if (p->fd) amx::fd_plan_destroy(p->fd);
  if (p->grav) amx::grav_plan_destroy(p->grav);
  if (p->force) amx::forcing_plan_destroy(p->force);
  if (p->ws) cudaFree(p->ws);
  delete p;
  return AMX_OK;
}

int amx_plan_set_limits(amx_plan* p, int32_t max_fixed_point_iterations, int64_t barrier_spin_limit) {
  if (!p || max_fixed_point_iterations < 0 || barrier_spin_limit < 0) return AMX_ERR_INVALID_ARG;
  if (p->fd) return AMX_ERR_UNSUPPORTED;  // the FD step has no fixed point and no grid barrier
  p->max_iters = max_fixed_point_iterations ? max_fixed_point_iterations : 1000;
  p->spin_limit = barrier_spin_limit ? (unsigned long long)barrier_spin_limit : AMX_BARRIER_SPIN_LIMIT;
  return AMX_OK;
}

int amx_plan_profile(amx_plan* p, int32_t enable) {
  if (!p) return AMX_ERR_INVALID_ARG;
  if (!p->fd) return AMX_ERR_UNSUPPORTED;
  return amx::fd_profile(p->fd, enable != 0);
}

int amx_plan_profile_read(amx_plan* p, double* ms, int64_t* launches, int32_t n, int32_t reset) {
  if (!p || n < 0) return AMX_ERR_INVALID_ARG;
  if (!p->fd) return AMX_ERR_UNSUPPORTED;
  return amx::fd_profile_read(p->fd, ms, launches, n, reset);
}

int amx_plan_workspace_bytes(const amx_plan* p, size_t* bytes) {
  if (!p || !bytes) return AMX_ERR_INVALID_ARG;
  *bytes = p->fd ? amx::fd_workspace_bytes(p->fd)
                 : p->ws_bytes + amx::grav_plan_bytes(p->grav) + amx::forcing_plan_bytes(p->force);
  return AMX_OK;
}

int amx_plan_reset(amx_plan* p, void* stream) {
  if (!p) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->fd) return amx::fd_reset(p->fd, s);
  return cuda_ok(cudaMemsetAsync(p->ctl, 0, sizeof(FVControl), s));
}

int amx_plan_set_time(amx_plan* p, double t, void* stream) {
  if (!p) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->fd) return amx::fd_set_time(p->fd, t, s);
  return cuda_ok(cudaMemcpyAsync(&p->ctl->t, &t, sizeof(double), cudaMemcpyHostToDevice, s)) |
         cuda_ok(cudaStreamSynchronize(s));
}

int amx_cfl_dt(amx_plan* p, const void* state, const amx_params* prm, double* dt_host, void* stream) {
  if (!p || !state || !prm || !dt_host) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->fd) return amx::fd_cfl_dt(p->fd, state, *prm, dt_host, s);
  int rc = fv_run_mode(p, const_cast<void*>(state), prm, amx::FV_MODE_CFL, 0.0, 1.0, 0, false, s);
  if (rc) return rc;
  rc = cuda_ok(cudaMemcpyAsync(dt_host, &p->ctl->dt, sizeof(double), cudaMemcpyDeviceToHost, s));
  rc |= cuda_ok(cudaStreamSynchronize(s));
  return rc;
}

int amx_fv_hydro_rk2(amx_plan* p, void* state, const amx_params* prm, double dt, void* stream) {
  if (!p || !state || !prm || p->fd) return AMX_ERR_INVALID_ARG;
  if (p->grav) {
    // the gas update followed by the gravitational source term (evolve_state.py:429-487)
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int one = 1;
    const size_t gas_bytes = (size_t)(p->cfg.dimensionality + 2) * (size_t)p->ncells * p->elem;
    void* old = amx::grav_old_state(p->grav);
    int rc = cuda_ok(cudaMemcpyAsync(&p->ctl->dt, &dt, sizeof(double), cudaMemcpyHostToDevice, s));
    rc |= cuda_ok(cudaMemcpyAsync(&p->ctl->active, &one, sizeof(int), cudaMemcpyHostToDevice, s));
    rc |= cuda_ok(cudaStreamSynchronize(s));
    rc |= cuda_ok(cudaMemcpyAsync(old, state, gas_bytes, cudaMemcpyDeviceToDevice, s));
    if (rc) return rc;
    rc = fv_seam(p, state, prm, amx::FV_MODE_HYDRO_RK2, 1.0, INFINITY, s);
    if (rc) return rc;
    return amx::grav_apply(p->grav, old, state, p->ctl, 1.0, *prm, s);
  }
  return fv_run_mode(p, state, prm, amx::FV_MODE_HYDRO_RK2, dt, 1.0, 0, false, static_cast<cudaStream_t>(stream));
}

int amx_fv_magnetic_update(amx_plan* p, void* state, const amx_params* prm, double dt, void* stream) {
  if (!p || !state || !prm || p->fd) return AMX_ERR_INVALID_ARG;
  if (!p->cfg.mhd) return AMX_ERR_INVALID_ARG;
  return fv_run_mode(p, state, prm, amx::FV_MODE_MAGNETIC, dt, 1.0, 0, false, static_cast<cudaStream_t>(stream));
}

int amx_evolve_state(amx_plan* p, void* state, const amx_params* prm, double dt, void* stream) {
  if (!p || !state || !prm) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->fd) return amx::fd_evolve(p->fd, state, *prm, dt, s);
  if (p->grav) {  // (forcing is not part of _evolve_state_fv)
    const int one = 1;
    int rc = cuda_ok(cudaMemcpyAsync(&p->ctl->dt, &dt, sizeof(double), cudaMemcpyHostToDevice, s));
    rc |= cuda_ok(cudaMemcpyAsync(&p->ctl->active, &one, sizeof(int), cudaMemcpyHostToDevice, s));
    rc |= cuda_ok(cudaStreamSynchronize(s));
    if (rc) return rc;
    return fv_device_step(p, state, prm, INFINITY, true, s);
  }
  return fv_run_mode(p, state, prm, amx::FV_MODE_EVOLVE, dt, 1.0, 0, false, s);
}

static int fv_run_steps(amx_plan* p, void* state, const amx_params* prm, int64_t max_steps, cudaStream_t s) {
  // one cooperative launch per chunk; the kernel stops by itself at t_end
  const int64_t chunk = 1 << 16;
  int64_t done = 0;
  while (done < max_steps) {
    const int64_t k = std::min<int64_t>(chunk, max_steps - done);
    int rc;
    if (p->cfg.dtype == AMX_F32) {
      auto a = make_fv_args<float>(p, state, prm, amx::FV_MODE_STEPS);
      a.max_steps = k;
      rc = fv_launch(p, a, s);
    } else {
      auto a = make_fv_args<double>(p, state, prm, amx::FV_MODE_STEPS);
      a.max_steps = k;
      rc = fv_launch(p, a, s);
    }
    if (rc) return rc;
    done += k;
  }
  return AMX_OK;
}

int amx_run_async(amx_plan* p, void* state, const amx_params* prm, int64_t max_steps, void* stream) {
  if (!p || !state || !prm || max_steps < 0) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->fd) return amx::fd_run(p->fd, state, *prm, max_steps, INFINITY, s);
  if (p->grav || p->force) {
    // a step is a sequence of launches: queue max_steps of them (bounded)
    if (max_steps > (1 << 20)) return AMX_ERR_TOO_LARGE;
    for (int64_t i = 0; i < max_steps; ++i) {
      const int rc = fv_device_step(p, state, prm, INFINITY, false, s);
      if (rc) return rc;
    }
    return AMX_OK;
  }
  return fv_run_steps(p, state, prm, max_steps, s);
}

static int read_info(amx_plan* p, amx_run_info* info, cudaStream_t s) {
  if (p->fd) return amx::fd_info(p->fd, info, s);
  FVControl h;
  int rc = cuda_ok(cudaMemcpyAsync(&h, p->ctl, sizeof(FVControl), cudaMemcpyDeviceToHost, s));
  rc |= cuda_ok(cudaStreamSynchronize(s));
  if (rc) return rc;
  info->t = h.t;
  info->last_dt = h.dt;
  info->steps = h.steps;
  info->magnetic_iterations = h.mag_iters_total;
  info->last_magnetic_iterations = h.mag_iters;
  info->status = h.status;
  return AMX_OK;
}

int amx_run(amx_plan* p, void* state, const amx_params* prm, int64_t max_steps, amx_run_info* info, void* stream) {
  return amx_run_until(p, state, prm, max_steps, INFINITY, info, stream);
}

int amx_run_until(amx_plan* p, void* state, const amx_params* prm, int64_t max_steps, double t_pause,
                  amx_run_info* info, void* stream) {
  if (!p || !state || !prm || max_steps < 0) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->fd) {
    int rc = amx::fd_run(p->fd, state, *prm, max_steps, t_pause, s);
    if (rc) return rc;
    amx_run_info tmp;
    return read_info(p, info ? info : &tmp, s);
  }
  if (p->grav || p->force) {
    // device-driven steps, the host checks t after 1, 2, 4, .. 32 steps
    int64_t done = 0, chunk = 1;
    amx_run_info g{};
    while (done < max_steps) {
      const int64_t k = std::min<int64_t>(chunk, max_steps - done);
      for (int64_t i = 0; i < k; ++i) {
        const int rc = fv_device_step(p, state, prm, t_pause, false, s);
        if (rc) return rc;
      }
      done += k;
      const int rc = read_info(p, &g, s);
      if (rc) return rc;
      if (!p->cfg.fixed_timestep && !(g.t < prm->t_end)) break;
      if (g.t >= t_pause) break;
      if (g.status & (AMX_ERR_TIMEOUT | AMX_ERR_NAN)) break;
      chunk = std::min<int64_t>(chunk * 2, 32);
    }
    if (max_steps == 0) {
      const int rc = read_info(p, &g, s);
      if (rc) return rc;
    }
    if (info) *info = g;
    return AMX_OK;
  }
  // FV: the history records are indexed from the first step of this call
  int rc = AMX_OK;
  const int64_t chunk = 1 << 16;
  int64_t done = 0;
  amx_run_info tmp{};
  while (done < max_steps) {
    const int64_t k = std::min<int64_t>(chunk, max_steps - done);
    if (p->cfg.dtype == AMX_F32) {
      auto a = make_fv_args<float>(p, state, prm, amx::FV_MODE_STEPS);
      a.max_steps = k;
      a.t_pause = t_pause;
      rc = fv_launch(p, a, s);
    } else {
      auto a = make_fv_args<double>(p, state, prm, amx::FV_MODE_STEPS);
      a.max_steps = k;
      a.t_pause = t_pause;
      rc = fv_launch(p, a, s);
    }
    if (rc) return rc;
    rc = read_info(p, &tmp, s);
    if (rc) return rc;
    done += k;
    if (!p->cfg.fixed_timestep && !(tmp.t < prm->t_end)) break;
    if (tmp.t >= t_pause) break;
    if (tmp.status & (AMX_ERR_TIMEOUT | AMX_ERR_NAN)) break;
  }
  if (max_steps == 0) {
    rc = read_info(p, &tmp, s);
    if (rc) return rc;
  }
  if (info) *info = tmp;
  return AMX_OK;
}

}  // extern "C"

namespace amx {

// Full FV steps in tape mode (fv_kernels.cuh): the start state is at
// tape + tape_off[steps so far]; every intermediate state of every step is
// appended to the tape and tape_off records where each step's end state
// starts.  Stops at t_end, after max_steps, or with AMX_ERR_TOO_LARGE in
// info->status when the tape is full.  Used by the adjoint's forward pass.
int fv_run_tape(amx_plan* p, const amx_params* prm, void* tape, long long tape_cap, long long* tape_off,
                int64_t max_steps, amx_run_info* info, cudaStream_t s) {
  if (!p || p->fd || !prm || !tape || !tape_off || !info) return AMX_ERR_INVALID_ARG;
  const int64_t chunk = 1 << 16;
  int64_t done = 0;
  amx_run_info tmp{};
  while (done < max_steps) {
    const int64_t k = std::min<int64_t>(chunk, max_steps - done);
    int rc;
    if (p->cfg.dtype == AMX_F32) {
      auto a = make_fv_args<float>(p, tape, prm, amx::FV_MODE_STEPS);
      a.max_steps = k;
      a.tape = static_cast<float*>(tape);
      a.tape_cap = tape_cap;
      a.tape_off = tape_off;
      rc = fv_launch(p, a, s);
    } else {
      auto a = make_fv_args<double>(p, tape, prm, amx::FV_MODE_STEPS);
      a.max_steps = k;
      a.tape = static_cast<double*>(tape);
      a.tape_cap = tape_cap;
      a.tape_off = tape_off;
      rc = fv_launch(p, a, s);
    }
    if (rc) return rc;
    rc = read_info(p, &tmp, s);
    if (rc) return rc;
    done += k;
    if (!(tmp.t < prm->t_end)) break;
    if (tmp.status & (AMX_ERR_TIMEOUT | AMX_ERR_NAN | AMX_ERR_TOO_LARGE)) break;
  }
  *info = tmp;
  return AMX_OK;
}

}  // namespace amx

extern "C" {

int amx_history(amx_plan* p, double* dt_host, int32_t* iters_host, int64_t n, void* stream) {
  if (!p || n < 0) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->fd) return amx::fd_history(p->fd, dt_host, n, s);
  if (n > p->max_hist) return AMX_ERR_INVALID_ARG;
  int rc = AMX_OK;
  if (dt_host && n) rc |= cuda_ok(cudaMemcpyAsync(dt_host, p->dt_hist, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  if (iters_host && n) rc |= cuda_ok(cudaMemcpyAsync(iters_host, p->it_hist, sizeof(int) * n, cudaMemcpyDeviceToHost, s));
  rc |= cuda_ok(cudaStreamSynchronize(s));
  return rc;
}

int amx_conservation_sums(amx_plan* p, const void* state, const amx_params* prm, double out_host[5],
                          void* stream) {
  if (!p || !state || !prm || !out_host) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  amx_config c = p->cfg;
  if (c.solver_mode == AMX_FINITE_DIFFERENCE) c.dimensionality = 3;
  int rc = amx_diag_sums_raw(&c, state, prm->gamma, p->diag, stream);
  if (rc) return rc;
  double h[5];
  rc = cuda_ok(cudaMemcpyAsync(h, p->diag, sizeof(h), cudaMemcpyDeviceToHost, s));
  rc |= cuda_ok(cudaStreamSynchronize(s));
  if (rc) return rc;
  const int d = c.dimensionality;
  const double dv = std::pow(c.grid_spacing, d);
  // total_quantities.py:155-176: 1D sums rho * cell volume (dx), 2D/3D sum(rho) * box^d
  out_host[0] = (d == 1) ? h[0] * c.grid_spacing : h[0] * std::pow(c.box_size, d);
  out_host[1] = h[1] * dv;
  out_host[2] = h[2] * dv;
  out_host[3] = h[3] * dv;
  out_host[4] = h[4];
  return AMX_OK;
}

int amx_status(amx_plan* p, int32_t* status_host, int32_t clear, void* stream) {
  if (!p || !status_host) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (p->fd) return amx::fd_status(p->fd, status_host, clear, s);
  int rc = cuda_ok(cudaMemcpyAsync(status_host, &p->ctl->status, sizeof(int), cudaMemcpyDeviceToHost, s));
  rc |= cuda_ok(cudaStreamSynchronize(s));
  if (clear) rc |= cuda_ok(cudaMemsetAsync(&p->ctl->status, 0, sizeof(int), s));
  rc |= cuda_ok(cudaStreamSynchronize(s));
  return rc;
}

}  // extern "C"
