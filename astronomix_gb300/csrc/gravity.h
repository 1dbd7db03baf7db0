// Self-gravity of the finite-volume scheme: the library-internal interface
// between the step driver (amx_api.cu) and the Poisson solve and source-term
// kernels (gravity.cu).
#pragma once

#include <cuda_runtime.h>

#include "../../include/amx.h"

namespace amx {

struct FVControl;
struct GravPlan;

// The gravity workspace of a run: the FFT plans and buffers of the Poisson
// solve on the grid the reference solves on (the padded grid with ghost-cell
// handling, the stored grid with periodic roll), and a copy of the gas rows
// of the state before each gas update.
int grav_plan_create(const amx_config& cfg, GravPlan** out);
void grav_plan_destroy(GravPlan* g);
size_t grav_plan_bytes(const GravPlan* g);
void* grav_old_state(GravPlan* g);

// _apply_self_gravity (_self_gravity.py:341-390) after a gas update of
// ctl->dt * dt_scale: the potential of the density of `old_state`, the
// source term of the configured version, and the explicit update of the gas
// rows of `state` in conserved variables.  Nothing is changed unless
// ctl->active.
int grav_apply(GravPlan* g, const void* old_state, void* state, const FVControl* ctl, double dt_scale,
               const amx_params& prm, cudaStream_t s);

}  // namespace amx
