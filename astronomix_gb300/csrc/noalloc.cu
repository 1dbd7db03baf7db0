// Allocation-free variant of the finite-volume time stepper.
//
// Some callers cannot call cudaMalloc: a host framework that owns all device
// memory and forbids allocations behind its back (XLA preallocates most of
// the GPU for itself, and a JAX custom call must not grab more), a process
// held to a fixed device-memory budget, and latency-critical loops where an
// allocation, which may synchronise the device, is not acceptable.
// amx_fv_run_noalloc serves them: it runs the same fv_run_kernel as amx_run,
// but its scratch memory (the RK stage buffer, the two magnetic iterate
// buffers and the control block) lives in one file-scope __device__ array of
// fixed size instead of a plan's cudaMalloc'd workspace.  The caller passes
// the state; nothing else is allocated, by this file or by any library
// routine it calls.
//
// Limits and sharing rules:
//  * the array holds kNoallocScratchBytes (8 MiB) on every GPU that loads
//    the library, for the life of the process;
//  * a configuration whose scratch does not fit is rejected with
//    AMX_ERR_TOO_LARGE before anything is launched;
//  * all calls on a device share the one array and it keeps the previous
//    call's contents: each call clears the control block it needs zeroed
//    (time, step counters, reduction slots, barrier, status), and calls that
//    overlap on the GPU (two streams, or two host threads) race on it;
//  * the first call on each device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture begins;
//  * with a non-null `info` the call reads the control block back and
//    synchronises the stream; a capturing stream may not be synchronised, so
//    such a call on one returns AMX_ERR_INVALID_ARG before launching anything.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/amx.h"
#include "fv_kernels.cuh"
#include "fv_registry.h"
#include "validate.h"

namespace {

constexpr size_t kNoallocScratchBytes = size_t(8) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {nullptr};

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Device address of g_noalloc_scratch on the current device (host code only
// holds a host-side stand-in under that name, never a device address).
int scratch_address(unsigned char** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return AMX_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return AMX_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return AMX_ERR_CUDA;
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return AMX_OK;
}

// The plan's validation plus what needs no allocation: FV only, and none of
// the cuFFT-based physics that run between the kernel's phases.
int check_config(const amx_config* c) {
  const int rc = amx::validate_config(c);
  if (rc) return rc;
  if (c->solver_mode != AMX_FINITE_VOLUME) return AMX_ERR_UNSUPPORTED;
  if (c->self_gravity || c->turbulent_forcing || c->stellar_wind) return AMX_ERR_UNSUPPORTED;
  return AMX_OK;
}

// Cells of the grid, or -1 when they exceed `limit` (checked after every
// factor, so that no product can overflow).
long long cells_within(const amx_config* c, long long limit) {
  long long nc = 1;
  for (int k = 0; k < c->dimensionality; ++k) {
    nc *= c->num_cells;
    if (nc > limit) return -1;
  }
  return nc;
}

template <typename T>
int launch(const amx_config* c, void* state, const amx_params* prm, int64_t max_steps, unsigned char* scratch,
           size_t o_p1, size_t o_m0, size_t o_m1, const amx::FVKernelInfo& kinfo, int grid, cudaStream_t s) {
  amx::FVArgs<T> a{};
  long long nc = 1;
  for (int k = 0; k < c->dimensionality; ++k) nc *= c->num_cells;
  a.state = static_cast<T*>(state);
  a.p1 = reinterpret_cast<T*>(scratch + o_p1);
  a.mag0 = reinterpret_cast<T*>(scratch + o_m0);
  a.mag1 = reinterpret_cast<T*>(scratch + o_m1);
  a.ctl = reinterpret_cast<amx::FVControl*>(scratch);
  a.dt_hist = nullptr;
  a.it_hist = nullptr;
  a.max_hist = 0;
  a.n = c->num_cells;
  a.ncells = nc;
  for (int k = 0; k < 3; ++k) a.bc[k] = amx::AxisBC{c->bc_lo[k], c->bc_hi[k]};
  a.periodic_roll = (c->boundary_handling == AMX_PERIODIC_ROLL);
  a.limiter = c->limiter;
  a.integrator = c->fv_magnetic_integrator;
  a.lm = (c->riemann_solver == AMX_HLLC_LM);
  a.am = (c->riemann_solver == AMX_AM_HLLC) ? 1 : (c->riemann_solver == AMX_HYBRID_HLLC ? 2 : 0);
  a.exact_end_time = c->exact_end_time;
  a.fixed_timestep = c->fixed_timestep;
  a.mode = amx::FV_MODE_STEPS;
  a.dx = c->grid_spacing;
  a.inv_dx = 1.0 / c->grid_spacing;
  a.gamma = prm->gamma;
  a.C_cfl = prm->C_cfl;
  a.t_end = prm->t_end;
  a.dt_fixed = c->num_timesteps > 0 ? prm->t_end / c->num_timesteps : 0.0;
  a.dt_in = 0.0;
  a.dt_scale = 1.0;
  a.tol = (c->numerical_precision == 1) ? 1e-10 : 1e-5;
  a.mhd = c->mhd;
  a.split = c->split;
  a.first_order = c->first_order_fallback;
  a.use_dt_max = c->use_max_adaptive_timestep;
  a.dt_max = prm->dt_max;
  a.p2 = a.mag0;
  a.max_iters = 1000;
  a.spin_limit = AMX_BARRIER_SPIN_LIMIT;
  a.t_pause = INFINITY;
  const int64_t chunk = int64_t(1) << 16;
  for (int64_t done = 0; done < max_steps; done += chunk) {
    a.max_steps = (max_steps - done < chunk) ? (max_steps - done) : chunk;
    // reduction slots and the barrier start at zero in every launch
    if (cudaMemsetAsync(a.ctl, 0, offsetof(amx::FVControl, dt), s) != cudaSuccess) return AMX_ERR_CUDA;
    void* args[] = {&a};
    if (cudaLaunchCooperativeKernel(kinfo.fn, dim3(grid), dim3(amx::kFVThreads), args, kinfo.smem, s) !=
        cudaSuccess)
      return AMX_ERR_CUDA;
  }
  return AMX_OK;
}

}  // namespace

extern "C" int amx_fv_run_noalloc(const amx_config* cfg, void* state, const amx_params* prm, int64_t max_steps,
                                  amx_run_info* info, void* stream) {
  int rc = check_config(cfg);
  if (rc) return rc;
  if (!state || !prm || max_steps < 0) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (info) {
    // reading the status back synchronises the stream, which a capture forbids
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) return AMX_ERR_CUDA;
    if (cs != cudaStreamCaptureStatusNone) return AMX_ERR_INVALID_ARG;
  }
  const size_t elem = cfg->dtype == AMX_F32 ? 4 : 8;
  // no grid with more values than the scratch holds can fit: refuse it before any product could overflow
  const long long nc = cells_within(cfg, (long long)(kNoallocScratchBytes / elem));
  if (nc < 0) return AMX_ERR_TOO_LARGE;
  const size_t field = (size_t)nc * elem;
  const size_t o_p1 = align256(sizeof(amx::FVControl));
  const size_t o_m0 = align256(o_p1 + (cfg->dimensionality + 2) * field);
  const size_t o_m1 = align256(o_m0 + (cfg->mhd ? 6 : (cfg->split ? cfg->dimensionality + 2 : 0)) * field);
  const size_t need = align256(o_m1 + (cfg->mhd ? 6 : 0) * field);
  if (need > kNoallocScratchBytes) return AMX_ERR_TOO_LARGE;

  unsigned char* scratch = nullptr;
  rc = scratch_address(&scratch);
  if (rc) return rc;

  amx::FVKernelInfo kinfo{};
  const int rs = amx::fv_riemann_family(cfg->riemann_solver);
  const int scheme = cfg->split ? amx::FV_SPLIT
                                 : (cfg->limiter == AMX_VAN_ALBADA_PP ? amx::FV_UNSPLIT_PP : amx::FV_UNSPLIT);
  const bool ok = (cfg->dtype == AMX_F32) ? amx::fv_kernel_f32(cfg->dimensionality, rs, cfg->mhd != 0, scheme, &kinfo)
                                          : amx::fv_kernel_f64(cfg->dimensionality, rs, cfg->mhd != 0, scheme, &kinfo);
  if (!ok) return AMX_ERR_UNSUPPORTED;
  if (scheme == amx::FV_UNSPLIT_PP) kinfo.smem += kinfo.smem_pp;  // as amx_plan_create
  if (cudaFuncSetAttribute(kinfo.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kinfo.smem) != cudaSuccess)
    return AMX_ERR_CUDA;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return AMX_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return AMX_ERR_CUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kinfo.fn, amx::kFVThreads, kinfo.smem) != cudaSuccess ||
      per_sm < 1)
    return AMX_ERR_CUDA;
  const long long cap = (long long)per_sm * sms;
  const long long want = (nc + amx::kFVThreads - 1) / amx::kFVThreads;
  const int grid = (int)(want < cap ? (want < 1 ? 1 : want) : cap);

  // a fresh run: time, counters and status start at zero
  if (cudaMemsetAsync(scratch, 0, sizeof(amx::FVControl), s) != cudaSuccess) return AMX_ERR_CUDA;
  rc = (cfg->dtype == AMX_F32) ? launch<float>(cfg, state, prm, max_steps, scratch, o_p1, o_m0, o_m1, kinfo, grid, s)
                               : launch<double>(cfg, state, prm, max_steps, scratch, o_p1, o_m0, o_m1, kinfo, grid, s);
  if (rc) return rc;
  if (info) {
    amx::FVControl h;
    if (cudaMemcpyAsync(&h, scratch, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess) return AMX_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return AMX_ERR_CUDA;
    info->t = h.t;
    info->last_dt = h.dt;
    info->steps = h.steps;
    info->magnetic_iterations = h.mag_iters_total;
    info->last_magnetic_iterations = h.mag_iters;
    info->status = h.status;
  }
  return AMX_OK;
}
