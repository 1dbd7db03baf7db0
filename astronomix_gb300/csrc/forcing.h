// Turbulent forcing: the library-internal interface between the step drivers
// (fd.cu, amx_api.cu) and the forcing kernels (forcing.cu).
#pragma once

#include <cuda_runtime.h>

#include "../../include/amx.h"

namespace amx {

struct ForcingPlan;

// The forcing workspace of an n^3 run: three complex fields and the cuFFT
// plan of their inverse transform, reduction scratch.
int forcing_plan_create(const amx_config& cfg, ForcingPlan** out);
void forcing_plan_destroy(ForcingPlan* f);
size_t forcing_plan_bytes(const ForcingPlan* f);

// _apply_forcing (_turbulent_forcing.py:72-128) on the primitive state (rows
// rho, v_x, v_y, v_z first) before the evolve of a step: a new solenoidal
// field for step *steps, the amplitude that injects energy_injection_rate *
// (*dt) of kinetic energy, velocities += amp * w.  Nothing happens unless
// *active.  dt, active and steps are device pointers into a control block.
int forcing_apply(ForcingPlan* f, void* state, const double* dt, const int* active, const long long* steps,
                  const amx_params& prm, cudaStream_t s);

}  // namespace amx
