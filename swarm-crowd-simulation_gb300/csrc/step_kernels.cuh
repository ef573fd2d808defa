// Host launchers of the step's kernels (step_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "step_args.cuh"

namespace swarm_gpu {

// hash, scan, scatter, rank + gather: 4 launches
void launch_sort(const StepArgs& A, cudaStream_t st, int64_t* launches);
// predict, K - 1 sweeps, final; ev (optional): events recorded after predict and after the sweeps
void launch_physics(const StepArgs& A, cudaStream_t st, int64_t* launches, cudaEvent_t* ev);

}  // namespace swarm_gpu
