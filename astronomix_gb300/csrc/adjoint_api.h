// Host-side interface of the adjoint kernels (one implementation per precision).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/amx.h"

namespace amx {
namespace adj {

// Device pointers of one step's tape slots (see StepTape in adjoint.cuh).
struct TapeView {
  void* S0;
  void* S1;
  void* S2;
  void* Z;
  void* S3;
  void* S4;
  void* S5;
  int iters;
  double dt;
};

// Cotangent scratch of one reverse step (see AdjScratch).
struct ScratchView {
  void* lS4;
  void* lS3;
  void* lS2;
  void* lS1;
  void* lU;
  void* lZ0;
  void* lZ1;
  void* lJ;
  void* lBa;
  void* lva;
  void* lv0;
};

struct Ops {
  int (*set_attrs)();
  int (*tape)(const amx_config* cfg, const amx_params* prm, const TapeView& t, cudaStream_t s);
  int (*adjoint)(const amx_config* cfg, const amx_params* prm, const TapeView& t, const void* lam, void* lS0,
                 const ScratchView& w, cudaStream_t s);
};

bool ops_f32(int dim, Ops* out);
bool ops_f64(int dim, Ops* out);

}  // namespace adj
}  // namespace amx
