// Finite-difference WENO-CT path (placeholder until the kernels land).
#include "fd_api.h"

namespace amx {

struct FDPlan {};

int fd_plan_create(const amx_config&, int64_t, FDPlan**) { return AMX_ERR_UNSUPPORTED; }
void fd_plan_destroy(FDPlan* p) { delete p; }
size_t fd_workspace_bytes(const FDPlan*) { return 0; }
int fd_reset(FDPlan*, cudaStream_t) { return AMX_ERR_UNSUPPORTED; }
int fd_set_time(FDPlan*, double, cudaStream_t) { return AMX_ERR_UNSUPPORTED; }
int fd_cfl_dt(FDPlan*, const void*, const amx_params&, double*, cudaStream_t) { return AMX_ERR_UNSUPPORTED; }
int fd_evolve(FDPlan*, void*, const amx_params&, double, cudaStream_t) { return AMX_ERR_UNSUPPORTED; }
int fd_run(FDPlan*, void*, const amx_params&, int64_t, double, cudaStream_t) { return AMX_ERR_UNSUPPORTED; }
int fd_info(FDPlan*, amx_run_info*, cudaStream_t) { return AMX_ERR_UNSUPPORTED; }
int fd_history(FDPlan*, double*, int64_t, cudaStream_t) { return AMX_ERR_UNSUPPORTED; }
int fd_status(FDPlan*, int32_t*, int32_t, cudaStream_t) { return AMX_ERR_UNSUPPORTED; }

}  // namespace amx
