// Host interface of the finite-difference WENO-CT path (fd.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/amx.h"

namespace amx {

struct FDPlan;

int fd_plan_create(const amx_config& cfg, int64_t max_history, FDPlan** out);
void fd_plan_destroy(FDPlan* p);
size_t fd_workspace_bytes(const FDPlan* p);
int fd_reset(FDPlan* p, cudaStream_t s);
int fd_set_time(FDPlan* p, double t, cudaStream_t s);
int fd_cfl_dt(FDPlan* p, const void* state, const amx_params& prm, double* dt_host, cudaStream_t s);
int fd_evolve(FDPlan* p, void* state, const amx_params& prm, double dt, cudaStream_t s);
int fd_run(FDPlan* p, void* state, const amx_params& prm, int64_t max_steps, double t_pause, cudaStream_t s);
int fd_info(FDPlan* p, amx_run_info* info, cudaStream_t s);
int fd_history(FDPlan* p, double* dt_host, int64_t n, cudaStream_t s);
int fd_status(FDPlan* p, int32_t* status_host, int32_t clear, cudaStream_t s);
int fd_profile(FDPlan* p, int enable);
int fd_profile_read(FDPlan* p, double* ms, int64_t* launches, int n, int reset);

}  // namespace amx
