// Common device-side machinery of the amx MHD kernels (sm_103a).
//
// * status bits reported to the host (never a trap or a device assert),
// * a bounded grid barrier for the persistent cooperative kernels,
// * bitwise max reductions of non-negative reals,
// * boundary-condition index mapping that replaces the reference's ghost-cell
//   fills (astronomix/_geometry/boundaries.py:74-385): the state lives in HBM
//   without ghost cells and every stencil load maps its index instead.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/amx.h"

namespace amx {

// ------------------------------------------------------------ status

__device__ __forceinline__ void raise_status(int* status, int bit) {
  if (status) atomicOr(status, bit);
}

// ------------------------------------------------------------ reductions

// Max of non-negative doubles through their bit patterns: for x >= 0 the
// IEEE order equals the unsigned-integer order, and a NaN (0x7ff8...) wins
// over +inf, so a NaN anywhere propagates like jnp.max does.
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* slot, double v) {
  atomicMax(slot, (unsigned long long)__double_as_longlong(v));
}

__device__ __forceinline__ double bits_to_double(unsigned long long b) {
  return __longlong_as_double((long long)b);
}

template <typename T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T w = __shfl_xor_sync(0xffffffffu, v, o);
    // NaN-propagating max (a NaN in either operand wins)
    v = (v != v) ? v : ((w != w) ? w : (w > v ? w : v));
  }
  return v;
}

// Block-wide NaN-propagating max; every thread gets the result.
template <typename T>
__device__ T block_max(T v, T* scratch /* >= 32 entries */) {
  v = warp_max(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  T r = (lane < nw) ? scratch[lane] : T(0);
  if (wid == 0) r = warp_max(r);
  if (threadIdx.x == 0) scratch[0] = r;
  __syncthreads();
  r = scratch[0];
  __syncthreads();
  return r;
}

template <typename T>
__device__ __forceinline__ T nanmax(T a, T b) {
  return (a != a) ? a : ((b != b) ? b : (b > a ? b : a));
}

// jnp.minimum: a NaN in either operand wins (fmin would drop it, and a NaN
// dt would then turn into a finite one)
template <typename T>
__device__ __forceinline__ T nanmin(T a, T b) {
  return (a != a) ? a : ((b != b) ? b : (b < a ? b : a));
}

// ------------------------------------------------------------ grid barrier

// Grid barrier for cooperative launches.  Every spin is bounded: after
// `spin_limit` polls (AMX_BARRIER_SPIN_LIMIT unless the plan sets another)
// the block gives up, records AMX_ERR_TIMEOUT and the barrier returns false
// so the caller can unwind.  A block that has seen `abort` set also returns
// false immediately.
#ifndef AMX_BARRIER_SPIN_LIMIT
#define AMX_BARRIER_SPIN_LIMIT (1ull << 24)
#endif

struct GridBarrier {
  unsigned long long* count;  // arrivals since the launch began (zeroed before it)
  int* abort_flag;            // set once any block timed out
  unsigned long long spin_limit = AMX_BARRIER_SPIN_LIMIT;
};

// Barrier number b of a launch is passed when the arrival counter reaches
// b * gridDim.x: every block adds one and waits for the multiple of the grid
// size above the value it drew, so no block resets anything and the last
// arrival needs no extra round trips.  (No block can arrive at barrier b + 1
// before all have arrived at b, so the values drawn at b lie in
// [(b - 1) N, b N).)  64-bit, so the counter cannot wrap within a launch.
__device__ __forceinline__ bool grid_sync(const GridBarrier& b, int* status) {
  __syncthreads();
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile int* ab = b.abort_flag;
    if (*ab) {
      ok = 0;
    } else {
      __threadfence();
      const unsigned long long n = gridDim.x;
      const unsigned long long arrived = atomicAdd(b.count, 1ull);
      const unsigned long long target = (arrived / n + 1ull) * n;
      volatile unsigned long long* cnt = b.count;
      unsigned long long spins = 0;
      while (*cnt < target) {
        if (*ab) { ok = 0; break; }
        if (++spins > b.spin_limit) {
          ok = 0;
          atomicExch(b.abort_flag, 1);
          raise_status(status, AMX_ERR_TIMEOUT);
          break;
        }
        __nanosleep(32);
      }
      __threadfence();
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ------------------------------------------------------------ boundaries

// Per-axis boundary codes (the reference's OPEN / REFLECTIVE / PERIODIC).
// `mode1d` selects the 1D reflective variant of boundaries.py:360-385,
// which copies the edge cell (with flipped velocity) into both ghost layers,
// instead of the mirror of boundaries.py:324-355 used in 2D/3D.
struct AxisBC {
  int lo, hi;  // AMX_BC_*
};

// Maps a logical index g in [-2, n+1] onto the stored cells [0, n).  Sets
// *flip when the value must be loaded with its axis-normal velocity negated.
__device__ __forceinline__ int map_index(int g, int n, AxisBC bc, bool mode1d, bool* flip) {
  if (g >= 0 && g < n) return g;
  if (g < 0) {
    switch (bc.lo) {
      case AMX_BC_PERIODIC: return g + n;
      case AMX_BC_OPEN: return 0;
      default:  // reflective
        *flip = !*flip;
        return mode1d ? 0 : (-g - 1);
    }
  }
  switch (bc.hi) {
    case AMX_BC_PERIODIC: return g - n;
    case AMX_BC_OPEN: return n - 1;
    default:
      *flip = !*flip;
      return mode1d ? (n - 1) : (2 * n - 1 - g);
  }
}

// Always-periodic wrap for offsets of at most one period.
__device__ __forceinline__ int wrap(int g, int n) {
  return g < 0 ? g + n : (g >= n ? g - n : g);
}

// Asynchronous global -> shared copy of one 4- or 8-byte element
// (cp.async): a thread issues every copy of a tile before it waits for any.
template <typename T>
__device__ __forceinline__ void cp_async_elem(T* smem, const T* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
// Asynchronous global -> shared copy of 16 bytes (cp.async.cg, around L1):
// both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async_16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

}  // namespace amx
