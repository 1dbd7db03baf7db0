// Batched ensemble: many independent FV runs of uneven grid sizes advanced
// by one persistent cooperative kernel.
//
// Every run follows the single-run step of fv_kernels.cuh exactly (same
// per-tile and per-cell functions, so a run's result does not depend on the
// batch it is in), with its own dt, t, t_end, step count and fixed-point
// iteration count.  The runs advance in lock-step phases separated by the
// grid barrier: a phase works through one global list of work items (hydro
// tiles, or chunks of cells for the point-wise phases) of the runs it
// concerns, so a run that has reached its end time, or whose magnetic
// fixed point has converged, drops out of the list and costs nothing.
// Every block rebuilds the list (a prefix sum of items per run) from the
// same reduced values after each barrier, so all blocks agree on it.
//
// Reductions are per run: the maxima of |u_a| + c (CFL dt, Lax-Friedrichs
// alpha) and the fixed-point residual go to per-run slots, folded by a
// block whenever the run of its next item differs from the last one.
#pragma once

#include "fv_kernels.cuh"

namespace amx {

constexpr int kBatchMaxRuns = 256;
constexpr int kBatchChunk = 1024;  // cells per work item of the point-wise phases
constexpr int kBatchVariants = 3;  // tile shapes (TileV) the autotuner chooses from

// Per-run description (device table, written by the host).
struct BatchRunDesc {
  void* state;   // [nvars][n^DIM] the caller's buffer
  void* p1;      // [DIM + 2][n^DIM] workspace
  void* mag0;    // [6][n^DIM]
  void* mag1;
  long long ncells;
  int n;
  int pad;
  double dx;
  double inv_dx;
  double t_end;
};

// Per-run progress and reduction slots (device).
struct BatchRunCtl {
  unsigned long long red[3][4];  // ring of maxima of |u_a| + c
  unsigned long long mag[3];     // ring of fixed-point residuals
  unsigned long long pad0;
  double t;
  double dt;
  long long steps;
  long long mag_iters_total;
  int mag_iters;                 // iterations of the last magnetic update
  int status;                    // AMX_ERR_* of this run
  long long pad1;
};

struct BatchControl {
  unsigned long long bar_count;  // grid-barrier arrivals of the current launch
  int abort_flag;
  int status;        // launch-level status (barrier timeout)
  long long passes;  // grid-barrier phases run (all launches)
  long long lock_steps;
};

template <typename T>
struct BatchArgs {
  FVArgs<T> base;    // settings shared by all runs; per-run fields are filled per item
  const BatchRunDesc* runs;
  BatchRunCtl* rctl;
  BatchControl* ctl;
  int num_runs;
  long long max_steps;  // lock-step steps of this launch
};

template <typename T, int DIM>
__device__ __forceinline__ FVArgs<T> batch_run_args(const BatchArgs<T>& b, int r) {
  FVArgs<T> a = b.base;
  const BatchRunDesc& d = b.runs[r];
  a.state = static_cast<T*>(d.state);
  a.p1 = static_cast<T*>(d.p1);
  a.mag0 = static_cast<T*>(d.mag0);
  a.mag1 = static_cast<T*>(d.mag1);
  a.n = d.n;
  a.ncells = d.ncells;
  a.dx = d.dx;
  a.inv_dx = d.inv_dx;
  a.t_end = d.t_end;
  return a;
}

// Largest r in [0, R) with pref[r] <= g: the run owning global item g.
__device__ __forceinline__ int batch_find_run(const int* pref, int R, int g) {
  int lo = 0, hi = R - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (pref[mid] <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// pref[r] = sum of items of the selected runs before r; pref[R] = total.
// Warp 0 scans; every thread must call it (it ends with a block barrier).
template <typename F>
__device__ __forceinline__ void batch_prefix(int* pref, int R, F items_of) {
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const int per = (R + 31) / 32;
    const int lo = lane * per, hi = min(R, lo + per);
    int local = 0;
    for (int r = lo; r < hi; ++r) local += items_of(r);
    int incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    int run = incl - local;
    for (int r = lo; r < hi; ++r) {
      pref[r] = run;
      run += items_of(r);
    }
    if (lane == 31) pref[R] = incl;
  }
  __syncthreads();
}

template <int DIM, typename T>
__device__ __forceinline__ void batch_fold(const T* m, unsigned long long* slot, double* red) {
  fold_maxima<DIM>(m, slot, red);
}

// launch bounds as the single-run kernel's, so that the shared per-item
// functions are compiled under the same register budget (and give the same
// arithmetic)
template <typename T, int DIM, int RS, bool MHD, int V>
__global__ void __launch_bounds__(kFVThreads, (DIM == 3 && sizeof(T) == 4) ? 3 : 2)
fv_batch_kernel(BatchArgs<T> b) {
  using G = TileGeom<T, DIM, V>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  __shared__ double red[32];
  __shared__ double s_t[kBatchMaxRuns], s_dt[kBatchMaxRuns];
  __shared__ int s_pref[kBatchMaxRuns + 1];
  __shared__ int s_it[kBatchMaxRuns];
  // per-run flags: bit 0 active in this step, bit 1 still iterating,
  // bit 2 the current iterate is in mag1, bit 3 stopped (non-finite dt)
  __shared__ unsigned char s_flag[kBatchMaxRuns];
  BatchControl* ctl = b.ctl;
  BatchRunCtl* rc = b.rctl;
  int* status = &ctl->status;
  const GridBarrier bar{&ctl->bar_count, &ctl->abort_flag};
  const int R = b.num_runs;

  for (int r = threadIdx.x; r < R; r += blockDim.x) {
    s_t[r] = *(volatile double*)&rc[r].t;
    s_flag[r] = (*(volatile int*)&rc[r].status & AMX_ERR_NAN) ? 8 : 0;
    s_it[r] = 0;
  }
  __syncthreads();

  int rp = 0, mag_pass = 0;
  long long passes = 0;
  auto sync = [&]() -> bool {
    ++passes;
    return grid_sync(bar, status);
  };
  // block 0 clears the ring slot the next producer will write
  auto clear_next_red = [&]() {
    if (blockIdx.x == 0)
      for (int e = threadIdx.x; e < R * 4; e += blockDim.x) rc[e >> 2].red[(rp + 1) % 3][e & 3] = 0ull;
  };
  auto last_max = [&](int r, int k) -> double {
    return bits_to_double(*(volatile unsigned long long*)&rc[r].red[(rp + 2) % 3][k]);
  };
  auto hydro_items = [&](int r) -> int {
    if (!(s_flag[r] & 1)) return 0;
    const int n = b.runs[r].n;
    return (int)fv_num_tiles<DIM>(n, G::T0, G::T1, G::T2);
  };
  auto chunk_items = [&](int r, int need) -> int {
    if (!(s_flag[r] & need)) return 0;
    return (int)((b.runs[r].ncells + kBatchChunk - 1) / kBatchChunk);
  };

  // One hydro stage over the tiles of the active runs (evolve_state.py:339-414);
  // `p0_is_state`: the RK2 combination with the state as U0; `track`: fold the
  // maxima of the output into the producer slot.
  auto stage = [&](bool from_state, bool p0_is_state, T div, bool track) -> bool {
    clear_next_red();
    const int total = s_pref[R];
    int cur = -1;
    T m[3] = {T(0), T(0), T(0)};
    for (int g = blockIdx.x; g < total; g += gridDim.x) {
      const int r = batch_find_run(s_pref, R, g);
      if (r != cur) {
        if (track && cur >= 0) {
          batch_fold<DIM>(m, rc[cur].red[rp % 3], red);
          m[0] = m[1] = m[2] = T(0);
        }
        cur = r;
      }
      const FVArgs<T> a = batch_run_args<T, DIM>(b, r);
      T alpha[3] = {T(0), T(0), T(0)};
      if (RS == RS_LF) {
#pragma unroll
        for (int k = 0; k < DIM; ++k) alpha[k] = T(last_max(r, k));
      }
      int o[3];
      tile_origin<DIM>(g - s_pref[r], a.n, G::T0, G::T1, G::T2, o);
      const T h = T(s_dt[r]) / div;  // the single-run kernel's dtT / 2 (MHD) or dtT
      const T* in = from_state ? a.state : a.p1;
      T* out = from_state ? a.p1 : a.state;
      FVItems<T, DIM, RS, V>::hydro(a, o, in, out, p0_is_state ? a.state : nullptr, h,
                                    RS == RS_LF ? alpha : nullptr, smem, m, track);
    }
    if (track && cur >= 0) batch_fold<DIM>(m, rc[cur].red[rp % 3], red);
    ++rp;
    return sync();
  };
  // RK2 update of the gas rows of every active run with stage dt dt_r / div
  auto rk2 = [&](T div, bool last) -> bool {
    batch_prefix(s_pref, R, hydro_items);
    if (!stage(true, false, div, RS == RS_LF)) return false;
    return stage(false, true, div, last || RS == RS_LF);
  };

  // per-cell phases over chunks of the runs with flag bit `need`
  auto mag_iterate = [&](bool first) -> bool {
    batch_prefix(s_pref, R, [&](int r) { return chunk_items(r, first ? 1 : 2); });
    const int total = s_pref[R];
    int cur = -1;
    T change = T(0);
    for (int g = blockIdx.x; g < total; g += gridDim.x) {
      const int r = batch_find_run(s_pref, R, g);
      if (r != cur) {
        if (cur >= 0) {
          const double v = block_max<double>((double)change, red);
          if (threadIdx.x == 0) atomic_max_nonneg(&rc[cur].mag[mag_pass % 3], v);
          change = T(0);
        }
        cur = r;
      }
      const FVArgs<T> a = batch_run_args<T, DIM>(b, r);
      const long long nc = a.ncells;
      const bool in1 = (s_flag[r] & 4) != 0;
      T* src = in1 ? a.mag1 : a.mag0;
      T* dst = in1 ? a.mag0 : a.mag1;
      MagSrc<T, DIM> ms;
      if (first) {
        ms = MagSrc<T, DIM>{a.state + (DIM + 2) * nc, a.state + nc, true};
        dst = a.mag0;
      } else {
        ms = MagSrc<T, DIM>{src, src + 3 * nc, false};
      }
      const long long c0 = (long long)(g - s_pref[r]) * kBatchChunk;
      const long long c1 = min(nc, c0 + kBatchChunk);
      const T h = T(s_dt[r]);
      MagItems<T, DIM>::direct(a, a.state, ms, dst, h, c0 + threadIdx.x, c1, blockDim.x, &change);
    }
    if (cur >= 0) {
      const double v = block_max<double>((double)change, red);
      if (threadIdx.x == 0) atomic_max_nonneg(&rc[cur].mag[mag_pass % 3], v);
    }
    return sync();
  };
  // after a fixed-point pass: read residuals, update flags, clear the ring
  auto mag_advance = [&](bool first) {
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
      unsigned char f = s_flag[r];
      const bool ran = first ? (f & 1) : (f & 2);
      if (!ran) continue;
      const double change = bits_to_double(*(volatile unsigned long long*)&rc[r].mag[mag_pass % 3]);
      if (first) {
        s_it[r] = 0;
        f &= ~4;  // the iterate is in mag0
      } else {
        s_it[r] += 1;
        f ^= 4;
      }
      const bool more = change > b.base.tol && s_it[r] < b.base.max_iters;
      f = more ? (f | 2) : (f & ~2);
      if (!more && blockIdx.x == 0) {
        if (change > b.base.tol) raise_status(&rc[r].status, AMX_ERR_NOT_CONVERGED);
        if (change != change) raise_status(&rc[r].status, AMX_ERR_NAN);
      }
      s_flag[r] = f;
    }
    if (blockIdx.x == 0)
      for (int r = threadIdx.x; r < R; r += blockDim.x) rc[r].mag[(mag_pass + 2) % 3] = 0ull;
    ++mag_pass;
    __syncthreads();
  };
  auto magnetic = [&]() -> bool {
    if (!mag_iterate(true)) return false;
    mag_advance(true);
    while (true) {
      int any = 0;
      for (int r = threadIdx.x; r < R; r += blockDim.x) any |= (s_flag[r] & 2);
      if (!__syncthreads_or(any)) break;
      if (!mag_iterate(false)) return false;
      mag_advance(false);
    }
    // write-back with the gamma = 5/3 pressure refresh
    clear_next_red();
    batch_prefix(s_pref, R, [&](int r) { return chunk_items(r, 1); });
    const int total = s_pref[R];
    int cur = -1;
    T m[3] = {T(0), T(0), T(0)};
    const bool track = RS == RS_LF;
    for (int g = blockIdx.x; g < total; g += gridDim.x) {
      const int r = batch_find_run(s_pref, R, g);
      if (r != cur) {
        if (track && cur >= 0) {
          batch_fold<DIM>(m, rc[cur].red[rp % 3], red);
          m[0] = m[1] = m[2] = T(0);
        }
        cur = r;
      }
      const FVArgs<T> a = batch_run_args<T, DIM>(b, r);
      const T* Bv = (s_flag[r] & 4) ? a.mag1 : a.mag0;
      const long long c0 = (long long)(g - s_pref[r]) * kBatchChunk;
      const long long c1 = min(a.ncells, c0 + kBatchChunk);
      MagItems<T, DIM>::finalize(a, a.state, Bv, a.state, c0 + threadIdx.x, c1, blockDim.x, track, m);
    }
    if (track && cur >= 0) batch_fold<DIM>(m, rc[cur].red[rp % 3], red);
    ++rp;
    return sync();
  };

  // ---- initial CFL maxima of the runs that will step
  for (int r = threadIdx.x; r < R; r += blockDim.x) {
    const bool go = !(s_flag[r] & 8) && s_t[r] < b.runs[r].t_end;
    s_flag[r] = (s_flag[r] & 8) | (go ? 1 : 0);
  }
  {
    clear_next_red();
    batch_prefix(s_pref, R, [&](int r) { return chunk_items(r, 1); });
    const int total = s_pref[R];
    int cur = -1;
    T m[3] = {T(0), T(0), T(0)};
    for (int g = blockIdx.x; g < total; g += gridDim.x) {
      const int r = batch_find_run(s_pref, R, g);
      if (r != cur) {
        if (cur >= 0) {
          batch_fold<DIM>(m, rc[cur].red[rp % 3], red);
          m[0] = m[1] = m[2] = T(0);
        }
        cur = r;
      }
      const FVArgs<T> a = batch_run_args<T, DIM>(b, r);
      const long long c0 = (long long)(g - s_pref[r]) * kBatchChunk;
      const long long c1 = min(a.ncells, c0 + kBatchChunk);
      const T gamma = T(a.gamma);
      for (long long c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        T q[DIM + 2];
#pragma unroll
        for (int v = 0; v < DIM + 2; ++v) q[v] = a.state[v * a.ncells + c];
        track_maxima<T, DIM>(q, gamma, m);
      }
    }
    if (cur >= 0) batch_fold<DIM>(m, rc[cur].red[rp % 3], red);
    ++rp;
    if (!sync()) return;
  }

  // ---- lock-step time steps (time_integration.py:386-762 per run)
  long long s = 0;
  for (; s < b.max_steps; ++s) {
    int any = 0;
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
      unsigned char f = s_flag[r] & 8;
      const double t = s_t[r];
      const double t_end = b.runs[r].t_end;
      if (!f && t < t_end) {
        // _timestep_estimator.py:118-128 with this run's maxima
        double sum = 0.0;
        const double dx = b.runs[r].dx;
#pragma unroll
        for (int k = 0; k < DIM; ++k) sum = (k == 0) ? last_max(r, k) / dx : sum + last_max(r, k) / dx;
        double dt = b.base.C_cfl * 1.0 / sum;
        if (b.base.exact_end_time) dt = nanmin(dt, t_end - t);
        if (dt > 0.0 && dt == dt) {
          s_dt[r] = dt;
          f |= 1;
          any = 1;
        } else {
          f |= 8;
          if (blockIdx.x == 0) raise_status(&rc[r].status, AMX_ERR_NAN);
        }
      }
      s_flag[r] = f;
    }
    if (!__syncthreads_or(any)) break;
    if (MHD) {
      if (!rk2(T(2), false)) return;
      if (!magnetic()) return;
      if (!rk2(T(2), true)) return;
    } else {
      if (!rk2(T(1), true)) return;
    }
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
      if (!(s_flag[r] & 1)) continue;
      s_t[r] = s_t[r] + s_dt[r];
      if (blockIdx.x == 0) {
        BatchRunCtl& q = rc[r];
        q.t = s_t[r];
        q.dt = s_dt[r];
        q.steps += 1;
        q.mag_iters = MHD ? s_it[r] : 0;
        q.mag_iters_total += MHD ? s_it[r] : 0;
      }
    }
    __syncthreads();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    ctl->passes += passes;
    ctl->lock_steps += s;
  }
}

}  // namespace amx
