// Per-precision glue of the adjoint: FVArgs from the C configuration, and
// the type-erased entry points of adjoint_api.h.
#pragma once

#include "adjoint.cuh"
#include "adjoint_api.h"

namespace amx {
namespace adj {

template <typename T>
FVArgs<T> fv_args(const amx_config* c, const amx_params* p) {
  FVArgs<T> a{};
  a.n = c->num_cells;
  long long nc = 1;
  for (int k = 0; k < c->dimensionality; ++k) nc *= c->num_cells;
  a.ncells = nc;
  for (int k = 0; k < 3; ++k) a.bc[k] = AxisBC{AMX_BC_PERIODIC, AMX_BC_PERIODIC};
  a.periodic_roll = 1;
  a.limiter = c->limiter;
  a.integrator = c->fv_magnetic_integrator;
  a.lm = 0;
  a.dx = c->grid_spacing;
  a.inv_dx = 1.0 / c->grid_spacing;
  a.gamma = p->gamma;
  a.C_cfl = p->C_cfl;
  return a;
}

template <typename T>
AdjGrid<T> grid(const amx_config* c, const amx_params* p) {
  AdjGrid<T> g;
  g.n = c->num_cells;
  g.nc = 1;
  for (int k = 0; k < c->dimensionality; ++k) g.nc *= c->num_cells;
  g.dx = c->grid_spacing;
  g.inv_dx = 1.0 / c->grid_spacing;
  g.gamma = p->gamma;
  return g;
}

template <typename T>
StepTape<T> typed(const TapeView& v) {
  return StepTape<T>{static_cast<T*>(v.S0), static_cast<T*>(v.S1), static_cast<T*>(v.S2), static_cast<T*>(v.Z),
                     static_cast<T*>(v.S3), static_cast<T*>(v.S4), static_cast<T*>(v.S5), v.iters, v.dt};
}

template <typename T>
AdjScratch<T> typed(const ScratchView& v) {
  return AdjScratch<T>{static_cast<T*>(v.lS4), static_cast<T*>(v.lS3), static_cast<T*>(v.lS2),
                       static_cast<T*>(v.lS1), static_cast<T*>(v.lU),  static_cast<T*>(v.lZ0),
                       static_cast<T*>(v.lZ1), static_cast<T*>(v.lJ),  static_cast<T*>(v.lBa),
                       static_cast<T*>(v.lva), static_cast<T*>(v.lv0)};
}

template <typename T, int DIM>
int tape_entry(const amx_config* c, const amx_params* p, const TapeView& t, cudaStream_t s) {
  return tape_step<T, DIM>(fv_args<T>(c, p), typed<T>(t), c->mhd != 0, s);
}

template <typename T, int DIM>
int adjoint_entry(const amx_config* c, const amx_params* p, const TapeView& t, const void* lam, void* lS0,
                  const ScratchView& w, cudaStream_t s) {
  return adjoint_step<T, DIM>(grid<T>(c, p), typed<T>(t), c->mhd != 0, c->fv_magnetic_integrator == 0,
                              static_cast<const T*>(lam), static_cast<T*>(lS0), typed<T>(w), s);
}

template <typename T>
bool ops(int dim, Ops* out) {
  if (dim == 2) {
    *out = Ops{&set_attrs<T, 2>, &tape_entry<T, 2>, &adjoint_entry<T, 2>};
    return true;
  }
  if (dim == 3) {
    *out = Ops{&set_attrs<T, 3>, &tape_entry<T, 3>, &adjoint_entry<T, 3>};
    return true;
  }
  return false;
}

}  // namespace adj
}  // namespace amx
