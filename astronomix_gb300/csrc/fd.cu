// Finite-difference WENO-CT MHD step: host plan.  The kernels live in
// fd_impl.cuh and are instantiated per precision in fd_f32.cu / fd_f64.cu.
//
// A step is 1 CFL reduction + 5 SSPRK(5,4) stages x 7 sweeps + 1 finalize
// sweep, all stream-ordered; dt, t and the "step active" flag live in the
// device control block, so the host enqueues steps without a round trip and
// only checks the control block every few steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <new>

#include "fd_api.h"
#include "fd_kernels.cuh"
#include "forcing.h"

namespace amx {
namespace fd {

// seam mode: a caller-given dt activates one step
__global__ void k_set_dt(FDControl* ctl, double dt) {
  ctl->dt = dt;
  ctl->active = 1;
}

}  // namespace fd

struct FDPlan {
  amx_config cfg;
  size_t elem = 4;
  long long nc = 0;
  size_t ws_bytes = 0;
  unsigned char* ws = nullptr;
  fd::FDLaunch L{};
  double wind_V = 0.0;              // stellar wind: sum of the injection mask x dx^3
  int wind_lo = 0, wind_n = 0;      // the cube of cells that holds the taper
  void* wind_src = nullptr;         // [5][wind_n^3] stage source
  ForcingPlan* force = nullptr;     // turbulent forcing (null without)
  // per-kernel timing (amx_plan_profile): events after every launch of a step
  bool profile = false;
  cudaEvent_t ev_start = nullptr;
  cudaEvent_t marks[fd::kFDMaxMarks] = {};
  int marks_kind[fd::kFDMaxMarks] = {};
  int marks_used = 0;
  double prof_ms[fd::FD_PH_COUNT] = {};
  long long prof_launches[fd::FD_PH_COUNT] = {};
};

namespace {

inline int ok(cudaError_t e) { return e == cudaSuccess ? AMX_OK : AMX_ERR_CUDA; }
inline size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

// rows per buffer: Q0 Q QF QC ACC (y, z) B BF M OM OB
const int kRows[10] = {8, 8, 8, 8, 16, 3, 3, 6, 3, 3};

fd::FDArgs make_args(const FDPlan* p, const amx_params& prm, double t_pause) {
  fd::FDArgs a;
  a.n = p->cfg.num_cells;
  a.nc = p->nc;
  a.dx = p->cfg.grid_spacing;
  a.gamma = prm.gamma;
  a.rhomin = prm.minimum_density;
  a.pgmin = prm.minimum_pressure;
  a.C_cfl = prm.C_cfl;
  a.dt_max = prm.dt_max;
  a.t_end = prm.t_end;
  a.enforce_positivity = p->cfg.enforce_positivity;
  a.exact_end_time = p->cfg.exact_end_time;
  a.fixed_timestep = p->cfg.fixed_timestep;
  a.dt_fixed = p->cfg.num_timesteps > 0 ? prm.t_end / p->cfg.num_timesteps : 0.0;
  a.t_pause = t_pause;
  a.wind = p->cfg.stellar_wind;
  a.wind_mdot = prm.wind_mass_loss_rate;
  a.wind_vinf = prm.wind_final_velocity;
  a.wind_V = p->wind_V;
  a.wind_rinj = p->cfg.num_injection_cells * p->cfg.grid_spacing;
  a.wind_r1 = 1.3 * a.wind_rinj;
  a.box = p->cfg.box_size;
  a.wind_lo = p->wind_lo;
  a.wind_n = p->wind_n;
  return a;
}

// V = sum over cells of the wind's injection mask x dx^3 (stellar_wind.py:503-522),
// summed over the cube that holds the taper
double wind_volume(const amx_config& c) {
  const int n = c.num_cells;
  const double dx = c.grid_spacing, half = c.box_size / 2;
  const double rinj = c.num_injection_cells * dx, r1 = 1.3 * rinj;
  double sum = 0.0;
  for (int i = 0; i < n; ++i) {
    const double x = dx / 2 + i * dx - half;
    if (std::fabs(x) > r1) continue;
    for (int j = 0; j < n; ++j) {
      const double y = dx / 2 + j * dx - half;
      if (std::fabs(y) > r1) continue;
      for (int k = 0; k < n; ++k) {
        const double z = dx / 2 + k * dx - half;
        const double r = std::sqrt(x * x + y * y + z * z);
        if (r <= rinj) sum += 1.0;
        else if (r <= r1) sum += (r1 - r) / (r1 - rinj);
      }
    }
  }
  return sum * std::pow(dx, 3);
}

int stages(FDPlan* p, const fd::FDLaunch& L, void* state, const fd::FDArgs& a, cudaStream_t s) {
  return p->cfg.dtype == AMX_F32 ? fd::fd_launch_stages_f32(L, state, a, s)
                                 : fd::fd_launch_stages_f64(L, state, a, s);
}

int cfl(FDPlan* p, const fd::FDLaunch& L, const void* state, const fd::FDArgs& a, cudaStream_t s) {
  return p->cfg.dtype == AMX_F32 ? fd::fd_launch_cfl_f32(L, state, a, s)
                                 : fd::fd_launch_cfl_f64(L, state, a, s);
}

// the launch set of one step: with timing on, events after every launch
fd::FDLaunch step_launch(FDPlan* p, cudaStream_t s) {
  fd::FDLaunch L = p->L;
  if (p->profile) {
    p->marks_used = 0;
    cudaEventRecord(p->ev_start, s);
    L.marks = p->marks;
    L.marks_kind = p->marks_kind;
    L.marks_used = &p->marks_used;
  }
  return L;
}

// adds the kernel durations of the step just launched (waits for it)
int step_timing(FDPlan* p) {
  if (!p->profile || p->marks_used == 0) return AMX_OK;
  if (cudaEventSynchronize(p->marks[p->marks_used - 1]) != cudaSuccess) return AMX_ERR_CUDA;
  cudaEvent_t prev = p->ev_start;
  for (int i = 0; i < p->marks_used; ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, prev, p->marks[i]) != cudaSuccess) return AMX_ERR_CUDA;
    p->prof_ms[p->marks_kind[i]] += ms;
    p->prof_launches[p->marks_kind[i]] += 1;
    prev = p->marks[i];
  }
  p->marks_used = 0;
  return AMX_OK;
}

}  // namespace

int fd_plan_create(const amx_config& cfg, int64_t max_history, FDPlan** out) {
  (void)max_history;
  FDPlan* p = new (std::nothrow) FDPlan();
  if (!p) return AMX_ERR_INVALID_ARG;
  p->cfg = cfg;
  p->elem = cfg.dtype == AMX_F32 ? 4 : 8;
  p->nc = (long long)cfg.num_cells * cfg.num_cells * cfg.num_cells;
  size_t off = a256(sizeof(fd::FDControl));
  size_t offs[10];
  for (int i = 0; i < 10; ++i) {
    offs[i] = off;
    off = a256(off + (size_t)kRows[i] * p->nc * p->elem);
  }
  p->ws_bytes = off;
  if (cudaMalloc(&p->ws, p->ws_bytes) != cudaSuccess) { delete p; return AMX_ERR_CUDA; }
  if (cudaMemset(p->ws, 0, p->ws_bytes) != cudaSuccess) { cudaFree(p->ws); delete p; return AMX_ERR_CUDA; }
  p->L.ctl = reinterpret_cast<fd::FDControl*>(p->ws);
  for (int i = 0; i < 10; ++i) p->L.bufs[i] = p->ws + offs[i];
  p->L.n = cfg.num_cells;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (p->nc + 255) / 256;  // 256-thread blocks (fd_impl.cuh kThreads)
  p->L.grid = (int)(want < (long long)sms * 8 ? want : (long long)sms * 8);
  int rc = (cfg.dtype == AMX_F32) ? fd::fd_set_attrs_f32() : fd::fd_set_attrs_f64();
  if (rc || cudaDeviceSynchronize() != cudaSuccess) { cudaFree(p->ws); delete p; return AMX_ERR_CUDA; }
  if (cfg.stellar_wind) {
    p->wind_V = wind_volume(cfg);
    // cells whose centre lies within 1.3 r_inj (plus one cell) of the box centre along every axis
    const double lim = 1.3 * cfg.num_injection_cells + 1.0;
    const double mid = 0.5 * cfg.num_cells - 0.5;
    const int lo = std::max(0, (int)std::floor(mid - lim));
    const int hi = std::min(cfg.num_cells - 1, (int)std::ceil(mid + lim));
    p->wind_lo = lo;
    p->wind_n = hi - lo + 1;
    const size_t wbytes = (size_t)5 * p->wind_n * p->wind_n * p->wind_n * p->elem;
    if (cudaMalloc(&p->wind_src, wbytes) != cudaSuccess) { fd_plan_destroy(p); return AMX_ERR_CUDA; }
    p->L.wind_src = p->wind_src;
  }
  if (cfg.turbulent_forcing) {
    rc = forcing_plan_create(cfg, &p->force);
    if (rc) { fd_plan_destroy(p); return rc; }
  }
  *out = p;
  return AMX_OK;
}

void fd_plan_destroy(FDPlan* p) {
  if (!p) return;
  fd_profile(p, 0);
  if (p->force) forcing_plan_destroy(p->force);
  if (p->wind_src) cudaFree(p->wind_src);
  if (p->ws) cudaFree(p->ws);
  delete p;
}

size_t fd_workspace_bytes(const FDPlan* p) { return p->ws_bytes + forcing_plan_bytes(p->force); }

int fd_reset(FDPlan* p, cudaStream_t s) { return ok(cudaMemsetAsync(p->L.ctl, 0, sizeof(fd::FDControl), s)); }

int fd_set_time(FDPlan* p, double t, cudaStream_t s) {
  return ok(cudaMemcpyAsync(&p->L.ctl->t, &t, sizeof(double), cudaMemcpyHostToDevice, s)) |
         ok(cudaStreamSynchronize(s));
}

int fd_cfl_dt(FDPlan* p, const void* state, const amx_params& prm, double* dt_host, cudaStream_t s) {
  // the pure CFL estimate: no end-time clamp, no pause
  fd::FDArgs a = make_args(p, prm, INFINITY);
  a.exact_end_time = 0;
  a.fixed_timestep = 0;
  a.t_end = INFINITY;
  int rc = cfl(p, p->L, state, a, s);
  rc |= ok(cudaMemcpyAsync(dt_host, &p->L.ctl->dt, sizeof(double), cudaMemcpyDeviceToHost, s));
  rc |= ok(cudaStreamSynchronize(s));
  return rc;
}

int fd_evolve(FDPlan* p, void* state, const amx_params& prm, double dt, cudaStream_t s) {
  // finalize advances t; the seam does not, so t is restored afterwards
  double t_before = 0.0;
  int rc = ok(cudaMemcpyAsync(&t_before, &p->L.ctl->t, sizeof(double), cudaMemcpyDeviceToHost, s)) |
           ok(cudaStreamSynchronize(s));
  if (rc) return rc;
  fd::k_set_dt<<<1, 1, 0, s>>>(p->L.ctl, dt);
  rc = ok(cudaGetLastError());
  if (rc) return rc;
  rc = stages(p, p->L, state, make_args(p, prm, INFINITY), s);
  if (rc) return rc;
  return ok(cudaMemcpyAsync(&p->L.ctl->t, &t_before, sizeof(double), cudaMemcpyHostToDevice, s)) |
         ok(cudaStreamSynchronize(s));
}

int fd_run(FDPlan* p, void* state, const amx_params& prm, int64_t max_steps, double t_pause, cudaStream_t s) {
  const fd::FDArgs a = make_args(p, prm, t_pause);
  const int64_t check_every = 4;
  for (int64_t st = 0; st < max_steps; ++st) {
    const fd::FDLaunch L = step_launch(p, s);
    int rc = cfl(p, L, state, a, s);
    // turbulent forcing between the dt and the evolve (time_integration.py:700-711)
    if (p->force) {
      rc |= forcing_apply(p->force, state, &p->L.ctl->dt, &p->L.ctl->active, &p->L.ctl->steps, prm, s);
      fd::fd_mark(L, fd::FD_PH_FORCING, s);
    }
    rc |= stages(p, L, state, a, s);
    rc |= step_timing(p);
    if (rc) return rc;
    if ((st + 1) % check_every == 0 && st + 1 < max_steps) {
      fd::FDControl h;
      rc = ok(cudaMemcpyAsync(&h, p->L.ctl, sizeof(h), cudaMemcpyDeviceToHost, s)) | ok(cudaStreamSynchronize(s));
      if (rc) return rc;
      if (!h.active) break;
      if (h.status & (AMX_ERR_NAN | AMX_ERR_TIMEOUT)) break;
    }
  }
  return AMX_OK;
}

int fd_info(FDPlan* p, amx_run_info* info, cudaStream_t s) {
  fd::FDControl h;
  int rc = ok(cudaMemcpyAsync(&h, p->L.ctl, sizeof(h), cudaMemcpyDeviceToHost, s)) | ok(cudaStreamSynchronize(s));
  if (rc) return rc;
  info->t = h.t;
  info->last_dt = h.dt;
  info->steps = h.steps;
  info->magnetic_iterations = 0;
  info->last_magnetic_iterations = 0;
  info->status = h.status;
  return AMX_OK;
}

int fd_history(FDPlan*, double*, int64_t, cudaStream_t) { return AMX_ERR_UNSUPPORTED; }

int fd_profile(FDPlan* p, int enable) {
  if (enable && !p->profile) {
    if (cudaEventCreate(&p->ev_start) != cudaSuccess) return AMX_ERR_CUDA;
    for (int i = 0; i < fd::kFDMaxMarks; ++i)
      if (cudaEventCreate(&p->marks[i]) != cudaSuccess) return AMX_ERR_CUDA;
    p->profile = true;
  } else if (!enable && p->profile) {
    cudaEventDestroy(p->ev_start);
    for (int i = 0; i < fd::kFDMaxMarks; ++i) cudaEventDestroy(p->marks[i]);
    p->ev_start = nullptr;
    p->profile = false;
  }
  return AMX_OK;
}

int fd_profile_read(FDPlan* p, double* ms, int64_t* launches, int n, int reset) {
  for (int i = 0; i < n && i < fd::FD_PH_COUNT; ++i) {
    if (ms) ms[i] = p->prof_ms[i];
    if (launches) launches[i] = p->prof_launches[i];
  }
  if (reset) {
    for (int i = 0; i < fd::FD_PH_COUNT; ++i) {
      p->prof_ms[i] = 0.0;
      p->prof_launches[i] = 0;
    }
  }
  return AMX_OK;
}

int fd_status(FDPlan* p, int32_t* status_host, int32_t clear, cudaStream_t s) {
  int rc = ok(cudaMemcpyAsync(status_host, &p->L.ctl->status, sizeof(int), cudaMemcpyDeviceToHost, s)) |
           ok(cudaStreamSynchronize(s));
  if (clear) rc |= ok(cudaMemsetAsync(&p->L.ctl->status, 0, sizeof(int), s)) | ok(cudaStreamSynchronize(s));
  return rc;
}

}  // namespace amx
