// Batched ensemble: host plan, work tables, CUDA-graph launch and the tile
// autotuner.  The kernel is fv_batch_kernel (fv_batch.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/amx.h"
#include "fv_batch.cuh"
#include "fv_batch_registry.h"

using amx::BatchControl;
using amx::BatchKernelInfo;
using amx::BatchRunCtl;
using amx::BatchRunDesc;

struct amx_batch {
  amx_config cfg;                 // template: everything but num_cells / grid spacing
  int num_runs = 0;
  int device = 0;
  int num_sms = 0;
  size_t elem = 4;
  int rs = 0;
  std::vector<int> n;
  std::vector<double> box;
  std::vector<BatchRunDesc> desc;  // host copy of the device table
  size_t ws_bytes = 0;
  unsigned char* ws = nullptr;
  BatchRunDesc* d_desc = nullptr;
  BatchRunCtl* d_rctl = nullptr;
  BatchControl* d_ctl = nullptr;
  // tiling: kernel variant and resident blocks per SM
  BatchKernelInfo kern{};
  int blocks_per_sm = 0;
  int max_blocks_per_sm = 0;
  // graph of (prepare, batch kernel), keyed on the launch arguments
  cudaStream_t capture_stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  std::vector<unsigned char> graph_key;
  int graph_launches = 0;
};

namespace {

inline int cuda_ok(cudaError_t e) { return e == cudaSuccess ? AMX_OK : AMX_ERR_CUDA; }
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// zeroes the reduction rings of every run and the grid barrier
__global__ void batch_prepare_kernel(BatchRunCtl* rc, int R, BatchControl* ctl) {
  for (int e = threadIdx.x; e < R * 15; e += blockDim.x) {
    const int r = e / 15, k = e % 15;
    if (k < 12) rc[r].red[k / 4][k % 4] = 0ull;
    else rc[r].mag[k - 12] = 0ull;
  }
  if (threadIdx.x == 0) {
    ctl->bar_count = 0ull;
    ctl->abort_flag = 0;
  }
}

bool lookup(const amx_batch* b, int variant, BatchKernelInfo* out) {
  const bool mhd = b->cfg.mhd != 0;
  return b->cfg.dtype == AMX_F32 ? amx::fv_batch_kernel_f32(2, b->rs, mhd, variant, out)
                                 : amx::fv_batch_kernel_f64(2, b->rs, mhd, variant, out);
}

int max_resident(const BatchKernelInfo& k, int* per_sm) {
  if (cudaFuncSetAttribute(k.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem) != cudaSuccess)
    return AMX_ERR_CUDA;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k.fn, amx::kFVThreads, k.smem) != cudaSuccess)
    return AMX_ERR_CUDA;
  return *per_sm >= 1 ? AMX_OK : AMX_ERR_CUDA;
}

int validate_template(const amx_config* c) {
  if (!c) return AMX_ERR_INVALID_ARG;
  if (c->solver_mode != AMX_FINITE_VOLUME) return AMX_ERR_UNSUPPORTED;
  // need cuFFT work between the phases of a step
  if (c->self_gravity || c->turbulent_forcing || c->stellar_wind) return AMX_ERR_UNSUPPORTED;
  if (c->dtype != AMX_F32 && c->dtype != AMX_F64) return AMX_ERR_INVALID_ARG;
  if (c->dimensionality != 2) return AMX_ERR_UNSUPPORTED;
  if (c->num_vars != 4 + (c->mhd ? 3 : 0)) return AMX_ERR_INVALID_ARG;
  if (c->riemann_solver != AMX_HLL && c->riemann_solver != AMX_HLLC && c->riemann_solver != AMX_HLLC_LM)
    return AMX_ERR_UNSUPPORTED;
  if (c->limiter < AMX_MINMOD || c->limiter > AMX_VAN_ALBADA) return AMX_ERR_UNSUPPORTED;
  if (c->fixed_timestep || c->split) return AMX_ERR_UNSUPPORTED;
  if (c->boundary_handling == AMX_GHOST_CELLS) {
    for (int k = 0; k < 2; ++k) {
      for (int side = 0; side < 2; ++side) {
        const int bc = side ? c->bc_hi[k] : c->bc_lo[k];
        if (bc != AMX_BC_OPEN && bc != AMX_BC_PERIODIC && bc != AMX_BC_REFLECTIVE) return AMX_ERR_UNSUPPORTED;
        if (c->mhd && bc == AMX_BC_REFLECTIVE) return AMX_ERR_UNSUPPORTED;
      }
      if ((c->bc_lo[k] == AMX_BC_PERIODIC) != (c->bc_hi[k] == AMX_BC_PERIODIC)) return AMX_ERR_UNSUPPORTED;
    }
  }
  return AMX_OK;
}

template <typename T>
amx::BatchArgs<T> make_args(const amx_batch* b, const amx_params* prm, long long max_steps) {
  amx::BatchArgs<T> a{};
  const amx_config& c = b->cfg;
  for (int k = 0; k < 3; ++k) a.base.bc[k] = amx::AxisBC{c.bc_lo[k], c.bc_hi[k]};
  a.base.periodic_roll = (c.boundary_handling == AMX_PERIODIC_ROLL);
  a.base.limiter = c.limiter;
  a.base.integrator = c.fv_magnetic_integrator;
  a.base.lm = (c.riemann_solver == AMX_HLLC_LM);
  a.base.exact_end_time = c.exact_end_time;
  a.base.mode = amx::FV_MODE_STEPS;
  a.base.gamma = prm->gamma;
  a.base.C_cfl = prm->C_cfl;
  a.base.tol = (c.numerical_precision == 1) ? 1e-10 : 1e-5;
  a.base.max_iters = 1000;
  a.base.spin_limit = AMX_BARRIER_SPIN_LIMIT;
  a.base.t_pause = INFINITY;
  a.runs = b->d_desc;
  a.rctl = b->d_rctl;
  a.ctl = b->d_ctl;
  a.num_runs = b->num_runs;
  a.max_steps = max_steps;
  return a;
}

int grid_of(const amx_batch* b) { return b->blocks_per_sm * b->num_sms; }

template <typename T>
int launch_direct(amx_batch* b, amx::BatchArgs<T>& a, cudaStream_t s) {
  batch_prepare_kernel<<<1, 256, 0, s>>>(b->d_rctl, b->num_runs, b->d_ctl);
  int rc = cuda_ok(cudaGetLastError());
  if (rc) return rc;
  void* args[] = {&a};
  return cuda_ok(cudaLaunchCooperativeKernel(b->kern.fn, dim3(grid_of(b)), dim3(amx::kFVThreads), args,
                                             b->kern.smem, s));
}

// The same two launches captured once into a graph (on the batch's own
// stream: the legacy default stream cannot be captured) and replayed on `s`
// while the arguments and the tiling stay the same.
template <typename T>
int launch_graph(amx_batch* b, amx::BatchArgs<T>& a, cudaStream_t s) {
  std::vector<unsigned char> key(sizeof(a) + 3 * sizeof(int));
  std::memcpy(key.data(), &a, sizeof(a));
  const int extra[3] = {b->kern.variant, b->blocks_per_sm, (int)b->cfg.dtype};
  std::memcpy(key.data() + sizeof(a), extra, sizeof(extra));
  if (!b->graph || key != b->graph_key) {
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    cudaStream_t cs = b->capture_stream;
    int rc = cuda_ok(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    if (rc) return rc;
    batch_prepare_kernel<<<1, 256, 0, cs>>>(b->d_rctl, b->num_runs, b->d_ctl);
    cudaLaunchConfig_t lc{};
    lc.gridDim = dim3(grid_of(b));
    lc.blockDim = dim3(amx::kFVThreads);
    lc.dynamicSmemBytes = b->kern.smem;
    lc.stream = cs;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    void* args[] = {&a};
    cudaError_t le = cudaLaunchKernelExC(&lc, b->kern.fn, args);
    cudaGraph_t g = nullptr;
    cudaError_t ee = cudaStreamEndCapture(cs, &g);
    if (le != cudaSuccess || ee != cudaSuccess || !g) {
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      return AMX_ERR_CUDA;
    }
    cudaError_t ie = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) {
      b->graph = nullptr;
      return AMX_ERR_CUDA;
    }
    b->graph_key = key;
  }
  ++b->graph_launches;
  return cuda_ok(cudaGraphLaunch(b->graph, s));
}

// Points the device table at `states` with end times `t_end`; uploads only
// when something changed, after the work queued on `s` (which may read the
// table) has finished (synchronous copy: the table is small and changes
// rarely).
int set_table(amx_batch* b, void* const* states, const double* t_end, cudaStream_t s) {
  bool changed = false;
  for (int r = 0; r < b->num_runs; ++r) {
    if (b->desc[r].state != states[r] || b->desc[r].t_end != t_end[r]) {
      b->desc[r].state = states[r];
      b->desc[r].t_end = t_end[r];
      changed = true;
    }
  }
  if (!changed) return AMX_OK;
  if (cudaStreamSynchronize(s) != cudaSuccess) return AMX_ERR_CUDA;
  return cuda_ok(cudaMemcpy(b->d_desc, b->desc.data(), sizeof(BatchRunDesc) * b->num_runs,
                            cudaMemcpyHostToDevice));
}

int run_once(amx_batch* b, const amx_params* prm, long long max_steps, bool use_graph, cudaStream_t s) {
  if (b->cfg.dtype == AMX_F32) {
    auto a = make_args<float>(b, prm, max_steps);
    return use_graph ? launch_graph(b, a, s) : launch_direct(b, a, s);
  }
  auto a = make_args<double>(b, prm, max_steps);
  return use_graph ? launch_graph(b, a, s) : launch_direct(b, a, s);
}

int select_tiling(amx_batch* b, int variant, int blocks_per_sm) {
  BatchKernelInfo k{};
  if (!lookup(b, variant, &k)) return AMX_ERR_UNSUPPORTED;
  int per_sm = 0;
  int rc = max_resident(k, &per_sm);
  if (rc) return rc;
  if (blocks_per_sm <= 0) blocks_per_sm = std::min(per_sm, 2);
  if (blocks_per_sm > per_sm) return AMX_ERR_INVALID_ARG;
  b->kern = k;
  b->blocks_per_sm = blocks_per_sm;
  b->max_blocks_per_sm = per_sm;
  return AMX_OK;
}

}  // namespace

extern "C" {

int amx_batch_create(const amx_config* tmpl, int32_t num_runs, const int32_t* num_cells, const double* box_size,
                     amx_batch** out) {
  if (!out) return AMX_ERR_INVALID_ARG;
  *out = nullptr;
  int rc = validate_template(tmpl);
  if (rc) return rc;
  if (num_runs < 1 || !num_cells || !box_size) return AMX_ERR_INVALID_ARG;
  if (num_runs > amx::kBatchMaxRuns) return AMX_ERR_TOO_LARGE;
  for (int r = 0; r < num_runs; ++r) {
    if (num_cells[r] < 4 || !(box_size[r] > 0.0)) return AMX_ERR_INVALID_ARG;
    // work items of a run are counted in int
    if ((long long)num_cells[r] * num_cells[r] > (1ll << 30)) return AMX_ERR_TOO_LARGE;
  }
  amx_batch* b = new (std::nothrow) amx_batch();
  if (!b) return AMX_ERR_INVALID_ARG;
  b->cfg = *tmpl;
  b->num_runs = num_runs;
  b->elem = tmpl->dtype == AMX_F32 ? 4 : 8;
  b->rs = (tmpl->riemann_solver == AMX_HLLC_LM) ? AMX_HLLC : tmpl->riemann_solver;
  b->n.assign(num_cells, num_cells + num_runs);
  b->box.assign(box_size, box_size + num_runs);
  if (cudaGetDevice(&b->device) != cudaSuccess) { delete b; return AMX_ERR_CUDA; }
  cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, b->device);
  rc = select_tiling(b, 0, 0);
  if (rc) { delete b; return rc; }

  // workspace: control, run table, run control, then per run p1 / mag0 / mag1
  const int nv_gas = 4;
  const int mag_rows = tmpl->mhd ? 6 : 0;
  size_t off = 0;
  const size_t o_ctl = off; off = align256(off + sizeof(BatchControl));
  const size_t o_desc = off; off = align256(off + sizeof(BatchRunDesc) * num_runs);
  const size_t o_rctl = off; off = align256(off + sizeof(BatchRunCtl) * num_runs);
  std::vector<size_t> o_run(num_runs);
  for (int r = 0; r < num_runs; ++r) {
    o_run[r] = off;
    const size_t field = (size_t)num_cells[r] * num_cells[r] * b->elem;
    off = align256(off + field * nv_gas);
    off = align256(off + field * mag_rows);
    off = align256(off + field * mag_rows);
  }
  b->ws_bytes = off;
  if (cudaMalloc(&b->ws, b->ws_bytes) != cudaSuccess) { delete b; return AMX_ERR_CUDA; }
  if (cudaMemset(b->ws, 0, b->ws_bytes) != cudaSuccess) { amx_batch_destroy(b); return AMX_ERR_CUDA; }
  b->d_ctl = reinterpret_cast<BatchControl*>(b->ws + o_ctl);
  b->d_desc = reinterpret_cast<BatchRunDesc*>(b->ws + o_desc);
  b->d_rctl = reinterpret_cast<BatchRunCtl*>(b->ws + o_rctl);
  b->desc.assign(num_runs, BatchRunDesc{});
  for (int r = 0; r < num_runs; ++r) {
    const long long nc = (long long)num_cells[r] * num_cells[r];
    const size_t field = (size_t)nc * b->elem;
    BatchRunDesc& d = b->desc[r];
    d.state = nullptr;
    d.p1 = b->ws + o_run[r];
    d.mag0 = tmpl->mhd ? b->ws + align256(o_run[r] + field * nv_gas) : nullptr;
    d.mag1 = tmpl->mhd ? b->ws + align256(align256(o_run[r] + field * nv_gas) + field * mag_rows) : nullptr;
    d.ncells = nc;
    d.n = num_cells[r];
    d.dx = box_size[r] / num_cells[r];
    d.inv_dx = 1.0 / d.dx;
    d.t_end = 0.0;
  }
  if (cudaMemcpy(b->d_desc, b->desc.data(), sizeof(BatchRunDesc) * num_runs, cudaMemcpyHostToDevice) !=
      cudaSuccess) {
    amx_batch_destroy(b);
    return AMX_ERR_CUDA;
  }
  if (cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking) != cudaSuccess) {
    amx_batch_destroy(b);
    return AMX_ERR_CUDA;
  }
  *out = b;
  return AMX_OK;
}

int amx_batch_destroy(amx_batch* b) {
  if (!b) return AMX_OK;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
  if (b->ws) cudaFree(b->ws);
  delete b;
  return AMX_OK;
}

int amx_batch_workspace_bytes(const amx_batch* b, size_t* bytes) {
  if (!b || !bytes) return AMX_ERR_INVALID_ARG;
  *bytes = b->ws_bytes;
  return AMX_OK;
}

int amx_batch_reset(amx_batch* b, void* stream) {
  if (!b) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = cuda_ok(cudaMemsetAsync(b->d_rctl, 0, sizeof(BatchRunCtl) * b->num_runs, s));
  rc |= cuda_ok(cudaMemsetAsync(b->d_ctl, 0, sizeof(BatchControl), s));
  return rc;
}

int amx_batch_run(amx_batch* b, void* const* states, const amx_params* prm, const double* t_end, int64_t max_steps,
                  int32_t use_graph, void* stream) {
  if (!b || !states || !prm || !t_end || max_steps < 0) return AMX_ERR_INVALID_ARG;
  for (int r = 0; r < b->num_runs; ++r)
    if (!states[r]) return AMX_ERR_INVALID_ARG;
  int rc = set_table(b, states, t_end, static_cast<cudaStream_t>(stream));
  if (rc) return rc;
  if (max_steps == 0) return AMX_OK;
  return run_once(b, prm, max_steps, use_graph != 0, static_cast<cudaStream_t>(stream));
}

int amx_batch_info(amx_batch* b, amx_run_info* infos, int64_t* lock_steps, void* stream) {
  if (!b || !infos) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::vector<BatchRunCtl> h(b->num_runs);
  BatchControl c{};
  int rc = cuda_ok(cudaMemcpyAsync(h.data(), b->d_rctl, sizeof(BatchRunCtl) * b->num_runs,
                                   cudaMemcpyDeviceToHost, s));
  rc |= cuda_ok(cudaMemcpyAsync(&c, b->d_ctl, sizeof(c), cudaMemcpyDeviceToHost, s));
  rc |= cuda_ok(cudaStreamSynchronize(s));
  if (rc) return rc;
  for (int r = 0; r < b->num_runs; ++r) {
    infos[r].t = h[r].t;
    infos[r].last_dt = h[r].dt;
    infos[r].steps = h[r].steps;
    infos[r].magnetic_iterations = h[r].mag_iters_total;
    infos[r].last_magnetic_iterations = h[r].mag_iters;
    infos[r].status = h[r].status | c.status;
  }
  if (lock_steps) *lock_steps = c.lock_steps;
  return AMX_OK;
}

int amx_batch_tiling(const amx_batch* b, int32_t* variant, int32_t* blocks_per_sm, int32_t* tile0,
                     int32_t* tile1) {
  if (!b) return AMX_ERR_INVALID_ARG;
  if (variant) *variant = b->kern.variant;
  if (blocks_per_sm) *blocks_per_sm = b->blocks_per_sm;
  if (tile0) *tile0 = b->kern.tile0;
  if (tile1) *tile1 = b->kern.tile1;
  return AMX_OK;
}

int amx_batch_set_tiling(amx_batch* b, int32_t variant, int32_t blocks_per_sm) {
  if (!b) return AMX_ERR_INVALID_ARG;
  return select_tiling(b, variant, blocks_per_sm);
}

int amx_batch_tune(amx_batch* b, void* const* states, const amx_params* prm, const double* t_end, int32_t steps,
                   double* best_ms, void* stream) {
  if (!b || !states || !prm || !t_end || steps < 1) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int R = b->num_runs;
  const int nvars = b->cfg.num_vars;
  // trial runs work on copies of the states and restore the run control
  std::vector<BatchRunCtl> saved(R);
  BatchControl saved_ctl{};
  int rc = cuda_ok(cudaMemcpyAsync(saved.data(), b->d_rctl, sizeof(BatchRunCtl) * R, cudaMemcpyDeviceToHost, s));
  rc |= cuda_ok(cudaMemcpyAsync(&saved_ctl, b->d_ctl, sizeof(saved_ctl), cudaMemcpyDeviceToHost, s));
  rc |= cuda_ok(cudaStreamSynchronize(s));
  if (rc) return rc;
  std::vector<size_t> bytes(R), offs(R);
  size_t total = 0;
  for (int r = 0; r < R; ++r) {
    bytes[r] = (size_t)b->n[r] * b->n[r] * nvars * b->elem;
    offs[r] = total;
    total = align256(total + bytes[r]);
  }
  unsigned char* scratch = nullptr;
  if (cudaMalloc(&scratch, total) != cudaSuccess) return AMX_ERR_CUDA;
  std::vector<void*> trial(R);
  for (int r = 0; r < R; ++r) trial[r] = scratch + offs[r];
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const BatchKernelInfo keep = b->kern;
  const int keep_bps = b->blocks_per_sm;
  double best = INFINITY;
  int best_v = keep.variant, best_bps = keep_bps;
  auto restore = [&]() -> int {
    int r2 = AMX_OK;
    for (int r = 0; r < R; ++r)
      r2 |= cuda_ok(cudaMemcpyAsync(trial[r], states[r], bytes[r], cudaMemcpyDeviceToDevice, s));
    r2 |= cuda_ok(cudaMemcpyAsync(b->d_rctl, saved.data(), sizeof(BatchRunCtl) * R, cudaMemcpyHostToDevice, s));
    r2 |= cuda_ok(cudaStreamSynchronize(s));
    return r2;
  };
  rc = set_table(b, trial.data(), t_end, s);
  for (int v = 0; v < amx::kBatchVariants && !rc; ++v) {
    BatchKernelInfo k{};
    if (!lookup(b, v, &k)) continue;
    int per_sm = 0;
    if (max_resident(k, &per_sm)) continue;
    for (int bps = 1; bps <= std::min(per_sm, 4) && !rc; ++bps) {
      b->kern = k;
      b->blocks_per_sm = bps;
      rc = restore();
      if (!rc) rc = run_once(b, prm, 1, false, s);  // warm-up
      if (!rc) rc = restore();
      if (rc) break;
      cudaEventRecord(e0, s);
      rc = run_once(b, prm, steps, false, s);
      cudaEventRecord(e1, s);
      rc |= cuda_ok(cudaEventSynchronize(e1));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      BatchControl c{};
      rc |= cuda_ok(cudaMemcpy(&c, b->d_ctl, sizeof(c), cudaMemcpyDeviceToHost));
      if (!rc && !(c.status & AMX_ERR_TIMEOUT) && ms < best) {
        best = ms;
        best_v = v;
        best_bps = bps;
      }
    }
  }
  // back to the caller's states and counters, with the fastest tiling
  int rc2 = cuda_ok(cudaMemcpyAsync(b->d_rctl, saved.data(), sizeof(BatchRunCtl) * R, cudaMemcpyHostToDevice, s));
  rc2 |= cuda_ok(cudaMemcpyAsync(b->d_ctl, &saved_ctl, sizeof(saved_ctl), cudaMemcpyHostToDevice, s));
  rc2 |= cuda_ok(cudaStreamSynchronize(s));
  rc2 |= set_table(b, states, t_end, s);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(scratch);
  b->kern = keep;
  b->blocks_per_sm = keep_bps;
  if (rc || rc2) return rc | rc2;
  if (best_ms) *best_ms = best;
  return select_tiling(b, best_v, best_bps);
}

}  // extern "C"
