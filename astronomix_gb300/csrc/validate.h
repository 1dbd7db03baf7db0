// Validation of an amx_config against what the kernels implement: the
// checks of finalize_config (astronomix/option_classes/simulation_config.py:
// 345-470) that concern the kernels, and the options outside them.  Shared by
// the plan (amx_api.cu) and the allocation-free entry point (noalloc.cu).
#pragma once

#include "../../include/amx.h"

namespace amx {

// The FV kernel family of a Riemann solver: HLLC-LM is a runtime mode of the
// HLLC kernel; AM_HLLC and HYBRID_HLLC share a kernel (4) whose compression
// switch is a runtime mode (FVArgs::am).
inline int fv_riemann_family(int riemann_solver) {
  if (riemann_solver == AMX_HLLC_LM) return AMX_HLLC;
  if (riemann_solver == AMX_HYBRID_HLLC || riemann_solver == AMX_AM_HLLC) return 4;
  return riemann_solver;
}

inline int validate_config(const amx_config* c) {
  if (!c) return AMX_ERR_INVALID_ARG;
  if (c->dtype != AMX_F32 && c->dtype != AMX_F64) return AMX_ERR_INVALID_ARG;
  if (c->dimensionality < 1 || c->dimensionality > 3) return AMX_ERR_INVALID_ARG;
  if (c->num_cells < 4) return AMX_ERR_INVALID_ARG;
  if (!(c->grid_spacing > 0.0)) return AMX_ERR_INVALID_ARG;
  if (c->solver_mode == AMX_FINITE_VOLUME) {
    const int nv = c->dimensionality + 2 + (c->mhd ? 3 : 0);
    if (c->num_vars != nv) return AMX_ERR_INVALID_ARG;
    if (c->mhd && c->dimensionality < 2) return AMX_ERR_UNSUPPORTED;
    if (c->split != 0 && c->split != 1) return AMX_ERR_INVALID_ARG;
    if (c->riemann_solver < AMX_HLL || c->riemann_solver > AMX_AM_HLLC) return AMX_ERR_UNSUPPORTED;
    if (c->limiter < AMX_MINMOD || c->limiter > AMX_VAN_ALBADA_PP) return AMX_ERR_UNSUPPORTED;
    // the reference's 1D VAN_ALBADA_PP sums its velocity terms over the whole grid
    if (c->limiter == AMX_VAN_ALBADA_PP && !c->split && c->dimensionality < 2) return AMX_ERR_UNSUPPORTED;
    // FV wind injection (the physics-module path) is not part of this library
    if (c->stellar_wind) return AMX_ERR_UNSUPPORTED;
    // the forcing field has the unpadded grid's shape (_turbulent_forcing.py:30-40):
    // 3D with periodic roll, as in the reference
    if (c->turbulent_forcing && (c->dimensionality != 3 || c->boundary_handling != AMX_PERIODIC_ROLL))
      return AMX_ERR_UNSUPPORTED;
    if (c->self_gravity) {
      if (c->self_gravity_version < AMX_SIMPLE_SOURCE_TERM || c->self_gravity_version > AMX_HALF_SPLIT)
        return AMX_ERR_INVALID_ARG;
      // the reference sets MINMOD for self-gravity (simulation_config.py:384-389);
      // the source term reconstructs with any limited-linear limiter, not VAN_ALBADA_PP
      if (c->limiter == AMX_VAN_ALBADA_PP) return AMX_ERR_UNSUPPORTED;
      // _self_gravity.py:163-167: the Riemann-split versions are HLLC-only
      if ((c->self_gravity_version == AMX_RIEMANN_SPLIT || c->self_gravity_version == AMX_RIEMANN_SPLIT_UNSTABLE) &&
          c->riemann_solver != AMX_HLLC && c->riemann_solver != AMX_HLLC_LM)
        return AMX_ERR_UNSUPPORTED;
    }
    if (c->boundary_handling == AMX_GHOST_CELLS) {
      for (int k = 0; k < c->dimensionality; ++k) {
        for (int side = 0; side < 2; ++side) {
          const int b = side ? c->bc_hi[k] : c->bc_lo[k];
          if (b != AMX_BC_OPEN && b != AMX_BC_PERIODIC && b != AMX_BC_REFLECTIVE) return AMX_ERR_UNSUPPORTED;
        }
        // periodic must be set on both sides (boundaries.py:105-111)
        if ((c->bc_lo[k] == AMX_BC_PERIODIC) != (c->bc_hi[k] == AMX_BC_PERIODIC)) return AMX_ERR_UNSUPPORTED;
      }
    }
    return AMX_OK;
  }
  if (c->solver_mode == AMX_FINITE_DIFFERENCE) {
    if (c->dimensionality != 3 || !c->mhd) return AMX_ERR_UNSUPPORTED;
    if (c->self_gravity) return AMX_ERR_UNSUPPORTED;
    if (c->num_vars != 11) return AMX_ERR_INVALID_ARG;
    if (c->num_cells < 8) return AMX_ERR_INVALID_ARG;
    return AMX_OK;
  }
  return AMX_ERR_INVALID_ARG;
}

}  // namespace amx
