// Discrete adjoint of the FV time integration: host driver.
//
// Two ways to get the tape (every intermediate state of every step) that the
// adjoint kernels (adjoint.cuh) walk in reverse:
//
// * Stored tape: when a tape budget is set and the run fits in it, the
//   persistent FV kernel itself writes the tape during the forward pass
//   (tape mode, fv_kernels.cuh); the backward needs no recompute.
// * Checkpoints: the ordinary persistent kernel advances the state
//   `checkpoint_every` steps at a time and the state at the start of every
//   segment is kept; the backward takes the segments last to first and
//   replays each from its checkpoint with the recorded dt and iteration
//   counts to rebuild that segment's tape.  One extra forward pass, and the
//   memory of the checkpoints plus one segment's tape.
//
// A stored-tape forward that runs out of room falls back to checkpoints.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "../../include/amx.h"
#include "adjoint_api.h"

namespace amx {
int fv_run_tape(amx_plan* p, const amx_params* prm, void* tape, long long tape_cap, long long* tape_off,
                int64_t max_steps, amx_run_info* info, cudaStream_t s);
}

using amx::adj::Ops;
using amx::adj::ScratchView;
using amx::adj::TapeView;

struct amx_adjoint {
  amx_config cfg;
  amx_params prm{};
  int every = 20;
  int64_t max_steps = 0;
  amx_plan* plan = nullptr;
  Ops ops{};
  size_t elem = 4;
  long long nc = 0;
  int nvt = 0, nvg = 0;
  std::vector<void*> ckpt;          // state at the start of segment s
  std::vector<double> dt;           // recorded schedule
  std::vector<int32_t> iters;
  int64_t steps = 0;
  bool have_forward = false;
  // stored tape (written by the forward)
  size_t budget = 0;
  unsigned char* ftape = nullptr;
  size_t ftape_bytes = 0;
  long long* d_tape_off = nullptr;
  std::vector<long long> tape_off;
  bool taped = false;
  // replay buffers
  unsigned char* tape = nullptr;
  size_t tape_bytes = 0;
  unsigned char* scratch = nullptr;
  size_t scratch_bytes = 0;
};

namespace {

inline int cuda_ok(cudaError_t e) { return e == cudaSuccess ? AMX_OK : AMX_ERR_CUDA; }

// rows are dense (the kernels index row v of a slot as v * ncells)
size_t row_bytes(const amx_adjoint* a) { return (size_t)a->nc * a->elem; }

// tape rows of one step with k iterations after the first evaluation
size_t step_rows(const amx_adjoint* a, int k) {
  if (!a->cfg.mhd) return (size_t)a->nvt + a->nvg;
  return (size_t)a->nvt * 3 + a->nvg * 2 + 6 * (size_t)(k + 1);
}

int grow(unsigned char** p, size_t* have, size_t want) {
  if (*have >= want) return AMX_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *have = 0;
  if (cudaMalloc(p, want) != cudaSuccess) return AMX_ERR_CUDA;
  *have = want;
  return AMX_OK;
}

// Lays out the tape of steps [s0, s1): S0 slots chain (S5 of a step is the
// next step's S0), the last S5 after them.
void layout(const amx_adjoint* a, int64_t s0, int64_t s1, std::vector<TapeView>* out) {
  const size_t R = row_bytes(a);
  unsigned char* p = a->tape;
  out->assign((size_t)(s1 - s0), TapeView{});
  void* prev_s5 = nullptr;
  for (int64_t s = s0; s < s1; ++s) {
    TapeView& t = (*out)[(size_t)(s - s0)];
    t.dt = a->dt[(size_t)s];
    t.iters = a->iters[(size_t)s];
    t.S0 = prev_s5 ? prev_s5 : p;
    if (!prev_s5) p += R * a->nvt;
    t.S1 = p; p += R * a->nvg;
    if (a->cfg.mhd) {
      t.S2 = p; p += R * a->nvt;
      t.Z = p; p += R * 6 * (size_t)(t.iters + 1);
      t.S3 = p; p += R * a->nvt;
      t.S4 = p; p += R * a->nvg;
    }
    t.S5 = p; p += R * a->nvt;
    prev_s5 = t.S5;
  }
}

// The stored tape's step views (layout of fv_kernels.cuh's tape mode).
void layout_stored(const amx_adjoint* a, std::vector<TapeView>* out) {
  const size_t E = a->elem;
  const long long nc = a->nc;
  out->assign((size_t)a->steps, TapeView{});
  for (int64_t s = 0; s < a->steps; ++s) {
    TapeView& t = (*out)[(size_t)s];
    t.dt = a->dt[(size_t)s];
    t.iters = a->iters[(size_t)s];
    unsigned char* p = a->ftape + (size_t)a->tape_off[(size_t)s] * E;
    t.S0 = p; p += E * nc * a->nvt;
    t.S1 = p; p += E * nc * a->nvg;
    if (a->cfg.mhd) {
      t.S2 = p; p += E * nc * a->nvt;
      t.Z = p; p += E * nc * 6 * (size_t)(t.iters + 1);
      t.S3 = p; p += E * nc * a->nvt;
      t.S4 = p;
    }
    t.S5 = a->ftape + (size_t)a->tape_off[(size_t)s + 1] * E;
  }
}

size_t tape_need(const amx_adjoint* a, int64_t s0, int64_t s1) {
  const size_t R = row_bytes(a);
  size_t rows = (size_t)a->nvt;  // first S0
  for (int64_t s = s0; s < s1; ++s) rows += step_rows(a, a->iters[(size_t)s]);
  return rows * R;
}

int scratch_view(amx_adjoint* a, ScratchView* w, void** lamA, void** lamB) {
  const size_t R = row_bytes(a);
  const size_t rows = (size_t)a->nvg * 3 + a->nvt * 2 + 6 * 2 + 3 * 4 + a->nvt * 2;
  int rc = grow(&a->scratch, &a->scratch_bytes, rows * R);
  if (rc) return rc;
  unsigned char* p = a->scratch;
  w->lS4 = p; p += R * a->nvg;
  w->lS3 = p; p += R * a->nvt;
  w->lS2 = p; p += R * a->nvt;
  w->lS1 = p; p += R * a->nvg;
  w->lU = p; p += R * a->nvg;
  w->lZ0 = p; p += R * 6;
  w->lZ1 = p; p += R * 6;
  w->lJ = p; p += R * 3;
  w->lBa = p; p += R * 3;
  w->lva = p; p += R * 3;
  w->lv0 = p; p += R * 3;
  *lamA = p; p += R * a->nvt;
  *lamB = p;
  return AMX_OK;
}

int copy_state(const amx_adjoint* a, void* dst, const void* src, cudaStream_t s) {
  return cuda_ok(cudaMemcpyAsync(dst, src, (size_t)a->nc * a->elem * a->nvt, cudaMemcpyDeviceToDevice, s));
}

}  // namespace

extern "C" {

int amx_adjoint_create(const amx_config* cfg, int32_t checkpoint_every, int64_t max_steps, amx_adjoint** out) {
  if (!out || !cfg || checkpoint_every < 1 || max_steps < 1) return AMX_ERR_INVALID_ARG;
  *out = nullptr;
  if (cfg->solver_mode != AMX_FINITE_VOLUME) return AMX_ERR_UNSUPPORTED;
  if (cfg->dimensionality != 2 && cfg->dimensionality != 3) return AMX_ERR_UNSUPPORTED;
  if (cfg->riemann_solver != AMX_HLL || cfg->limiter != AMX_MINMOD) return AMX_ERR_UNSUPPORTED;
  if (cfg->fixed_timestep || cfg->split || cfg->self_gravity || cfg->turbulent_forcing || cfg->stellar_wind)
    return AMX_ERR_UNSUPPORTED;
  const bool roll = cfg->boundary_handling == AMX_PERIODIC_ROLL;
  for (int k = 0; k < cfg->dimensionality && !roll; ++k)
    if (cfg->bc_lo[k] != AMX_BC_PERIODIC || cfg->bc_hi[k] != AMX_BC_PERIODIC) return AMX_ERR_UNSUPPORTED;
  amx_adjoint* a = new (std::nothrow) amx_adjoint();
  if (!a) return AMX_ERR_INVALID_ARG;
  a->cfg = *cfg;
  a->every = checkpoint_every;
  a->max_steps = max_steps;
  a->elem = cfg->dtype == AMX_F32 ? 4 : 8;
  a->nc = 1;
  for (int k = 0; k < cfg->dimensionality; ++k) a->nc *= cfg->num_cells;
  a->nvg = cfg->dimensionality + 2;
  a->nvt = a->nvg + (cfg->mhd ? 3 : 0);
  const bool ok = cfg->dtype == AMX_F32 ? amx::adj::ops_f32(cfg->dimensionality, &a->ops)
                                        : amx::adj::ops_f64(cfg->dimensionality, &a->ops);
  if (!ok) { delete a; return AMX_ERR_UNSUPPORTED; }
  int rc = a->ops.set_attrs();
  if (!rc) rc = amx_plan_create(cfg, max_steps, &a->plan);
  if (rc) { delete a; return rc; }
  *out = a;
  return AMX_OK;
}

int amx_adjoint_set_tape_budget(amx_adjoint* a, size_t bytes) {
  if (!a) return AMX_ERR_INVALID_ARG;
  a->budget = bytes;
  if (a->ftape && a->ftape_bytes != bytes) {
    cudaFree(a->ftape);
    a->ftape = nullptr;
    a->ftape_bytes = 0;
  }
  return AMX_OK;
}

int amx_adjoint_destroy(amx_adjoint* a) {
  if (!a) return AMX_OK;
  for (void* p : a->ckpt) cudaFree(p);
  if (a->ftape) cudaFree(a->ftape);
  if (a->d_tape_off) cudaFree(a->d_tape_off);
  if (a->tape) cudaFree(a->tape);
  if (a->scratch) cudaFree(a->scratch);
  if (a->plan) amx_plan_destroy(a->plan);
  delete a;
  return AMX_OK;
}

int amx_adjoint_forward(amx_adjoint* a, void* state, const amx_params* prm, amx_run_info* info, void* stream) {
  if (!a || !state || !prm) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  a->prm = *prm;
  a->have_forward = false;
  a->taped = false;
  int rc = amx_plan_reset(a->plan, stream);
  if (rc) return rc;
  const size_t bytes = (size_t)a->nc * a->elem * a->nvt;
  amx_run_info inf{};
  if (a->budget >= 3 * bytes) {
    if (!a->ftape) {
      if (cudaMalloc(&a->ftape, a->budget) != cudaSuccess) return AMX_ERR_CUDA;
      a->ftape_bytes = a->budget;
    }
    if (!a->d_tape_off && cudaMalloc(&a->d_tape_off, sizeof(long long) * (size_t)(a->max_steps + 1)) != cudaSuccess)
      return AMX_ERR_CUDA;
    rc = cuda_ok(cudaMemsetAsync(a->d_tape_off, 0, sizeof(long long), s));
    rc |= cuda_ok(cudaMemcpyAsync(a->ftape, state, bytes, cudaMemcpyDeviceToDevice, s));
    if (!rc) rc = amx::fv_run_tape(a->plan, prm, a->ftape, (long long)(a->ftape_bytes / a->elem), a->d_tape_off,
                                   a->max_steps, &inf, s);
    if (rc) return rc;
    if (!(inf.status & AMX_ERR_TOO_LARGE)) {
      a->steps = inf.steps;
      a->tape_off.assign((size_t)a->steps + 1, 0);
      rc = cuda_ok(cudaMemcpyAsync(a->tape_off.data(), a->d_tape_off, sizeof(long long) * (a->steps + 1),
                                   cudaMemcpyDeviceToHost, s));
      rc |= cuda_ok(cudaStreamSynchronize(s));
      if (rc) return rc;
      rc = cuda_ok(cudaMemcpyAsync(state, a->ftape + (size_t)a->tape_off[(size_t)a->steps] * a->elem, bytes,
                                   cudaMemcpyDeviceToDevice, s));
      a->dt.assign((size_t)a->steps, 0.0);
      a->iters.assign((size_t)a->steps, 0);
      if (!rc && a->steps) rc = amx_history(a->plan, a->dt.data(), a->iters.data(), a->steps, stream);
      if (rc) return rc;
      if (info) *info = inf;
      a->taped = (inf.status == 0);
      a->have_forward = (inf.status == 0);
      return inf.status ? inf.status : AMX_OK;
    }
    // out of room: run again with checkpoints (the caller's state is untouched)
    rc = amx_plan_reset(a->plan, stream);
    if (rc) return rc;
    inf = amx_run_info{};
  }
  int64_t done = 0;
  for (size_t seg = 0;; ++seg) {
    if (seg >= a->ckpt.size()) {
      void* p = nullptr;
      if (cudaMalloc(&p, bytes) != cudaSuccess) return AMX_ERR_CUDA;
      a->ckpt.push_back(p);
    }
    rc = cuda_ok(cudaMemcpyAsync(a->ckpt[seg], state, bytes, cudaMemcpyDeviceToDevice, s));
    if (rc) return rc;
    const int64_t k = std::min<int64_t>(a->every, a->max_steps - done);
    if (k <= 0) return AMX_ERR_TOO_LARGE;  // more steps than the schedule can record
    rc = amx_run(a->plan, state, prm, k, &inf, stream);
    if (rc) return rc;
    if (inf.status & (AMX_ERR_NAN | AMX_ERR_TIMEOUT | AMX_ERR_NOT_CONVERGED)) break;
    if (inf.steps - done < k || !(inf.t < prm->t_end)) break;
    done = inf.steps;
  }
  a->steps = inf.steps;
  a->dt.assign((size_t)a->steps, 0.0);
  a->iters.assign((size_t)a->steps, 0);
  if (a->steps) rc = amx_history(a->plan, a->dt.data(), a->iters.data(), a->steps, stream);
  if (rc) return rc;
  if (info) *info = inf;
  a->have_forward = (inf.status == 0);
  return inf.status ? inf.status : AMX_OK;
}

int amx_adjoint_uses_stored_tape(const amx_adjoint* a, int32_t* yes) {
  if (!a || !yes) return AMX_ERR_INVALID_ARG;
  *yes = a->taped ? 1 : 0;
  return AMX_OK;
}

int amx_adjoint_schedule(amx_adjoint* a, double* dt_host, int32_t* iters_host, int64_t n, int64_t* steps) {
  if (!a) return AMX_ERR_INVALID_ARG;
  if (steps) *steps = a->steps;
  if (n < 0 || n > a->steps) return AMX_ERR_INVALID_ARG;
  for (int64_t i = 0; i < n; ++i) {
    if (dt_host) dt_host[i] = a->dt[(size_t)i];
    if (iters_host) iters_host[i] = a->iters[(size_t)i];
  }
  return AMX_OK;
}

int amx_adjoint_backward(amx_adjoint* a, const void* grad_final, void* grad_initial, void* stream) {
  if (!a || !grad_final || !grad_initial) return AMX_ERR_INVALID_ARG;
  if (!a->have_forward) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  ScratchView w{};
  void *lamA = nullptr, *lamB = nullptr;
  int rc = scratch_view(a, &w, &lamA, &lamB);
  if (rc) return rc;
  if (a->taped) {
    std::vector<TapeView> tv;
    layout_stored(a, &tv);
    rc = copy_state(a, lamA, grad_final, s);
    for (int64_t i = (int64_t)tv.size() - 1; i >= 0 && !rc; --i) {
      rc = a->ops.adjoint(&a->cfg, &a->prm, tv[(size_t)i], lamA, lamB, w, s);
      std::swap(lamA, lamB);
    }
    if (rc) return rc;
    rc = copy_state(a, grad_initial, lamA, s);
    rc |= cuda_ok(cudaStreamSynchronize(s));
    return rc;
  }
  size_t need = 0;
  const int64_t nseg = (a->steps + a->every - 1) / a->every;
  for (int64_t g = 0; g < nseg; ++g)
    need = std::max(need, tape_need(a, g * a->every, std::min<int64_t>(a->steps, (g + 1) * a->every)));
  rc = grow(&a->tape, &a->tape_bytes, need);
  if (rc) return rc;
  rc = copy_state(a, lamA, grad_final, s);
  if (rc) return rc;
  std::vector<TapeView> tv;
  for (int64_t g = nseg - 1; g >= 0; --g) {
    const int64_t s0 = g * a->every, s1 = std::min<int64_t>(a->steps, (g + 1) * a->every);
    layout(a, s0, s1, &tv);
    rc = copy_state(a, tv[0].S0, a->ckpt[(size_t)g], s);
    for (size_t i = 0; i < tv.size() && !rc; ++i) rc = a->ops.tape(&a->cfg, &a->prm, tv[i], s);
    for (int64_t i = (int64_t)tv.size() - 1; i >= 0 && !rc; --i) {
      rc = a->ops.adjoint(&a->cfg, &a->prm, tv[(size_t)i], lamA, lamB, w, s);
      std::swap(lamA, lamB);
    }
    if (rc) return rc;
  }
  rc = copy_state(a, grad_initial, lamA, s);
  rc |= cuda_ok(cudaStreamSynchronize(s));
  return rc;
}

int amx_adjoint_replay(amx_adjoint* a, void* state, void* stream) {
  if (!a || !state) return AMX_ERR_INVALID_ARG;
  if (!a->have_forward) return AMX_ERR_INVALID_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t R = row_bytes(a);
  int kmax = 0;
  for (int32_t k : a->iters) kmax = std::max(kmax, (int)k);
  // one step's slots, reused; S5 ping-pongs with S0
  const size_t need = (step_rows(a, kmax) + a->nvt) * R;
  int rc = grow(&a->tape, &a->tape_bytes, need);
  if (rc) return rc;
  unsigned char* p = a->tape;
  TapeView t{};
  t.S0 = p; p += R * a->nvt;
  t.S1 = p; p += R * a->nvg;
  if (a->cfg.mhd) {
    t.S2 = p; p += R * a->nvt;
    t.Z = p; p += R * 6 * (size_t)(kmax + 1);
    t.S3 = p; p += R * a->nvt;
    t.S4 = p; p += R * a->nvg;
  }
  t.S5 = p;
  rc = copy_state(a, t.S0, state, s);
  for (int64_t i = 0; i < a->steps && !rc; ++i) {
    t.dt = a->dt[(size_t)i];
    t.iters = a->iters[(size_t)i];
    rc = a->ops.tape(&a->cfg, &a->prm, t, s);
    std::swap(t.S0, t.S5);
  }
  if (rc) return rc;
  rc = copy_state(a, state, t.S0, s);
  rc |= cuda_ok(cudaStreamSynchronize(s));
  return rc;
}

int amx_adjoint_memory(const amx_adjoint* a, size_t* checkpoint_bytes, size_t* tape_bytes) {
  if (!a) return AMX_ERR_INVALID_ARG;
  if (checkpoint_bytes) *checkpoint_bytes = a->ckpt.size() * (size_t)a->nc * a->elem * a->nvt;
  // the stored tape counts what the last forward used
  const size_t stored = a->taped ? (size_t)a->tape_off.back() * a->elem + (size_t)a->nc * a->elem * a->nvt : 0;
  if (tape_bytes) *tape_bytes = a->tape_bytes + a->scratch_bytes + stored;
  return AMX_OK;
}

}  // extern "C"
