// Host launchers of the step's kernels (step_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "step_args.cuh"

namespace swarm_gpu {

// hash, scan, scatter, rank + gather: 4 launches
void launch_sort(const StepArgs& A, cudaStream_t st, int64_t* launches);
// stage 0: the sort (hash, scan, scatter, rank + gather); 1: predict; 2: the K - 1 sweeps; 3: the final pass
void launch_stage(const StepArgs& A, int stage, cudaStream_t st, int64_t* launches);
// the adjoint's taped forward step (grid venue, one instance): q[0 .. K - 1] the sweeps' inputs, corr[1 .. K] their
// corrections, qK the last sweep's result, pred predict's separation / headway record
void launch_step_taped(const StepArgs& A, float4* const* q, float4* const* corr, float4* qK, float4* pred, cudaStream_t st,
                       int64_t* launches);
// the same as one fused launch (grid venue, one instance): proj[0] = q[0] with the sweeps' inputs n apart, tapeCorr =
// corr[1] with the sweeps' corrections n apart, tapeQK, tapePred
cudaError_t launch_step_fused_taped(const StepArgs& A, cudaStream_t st);
// the whole step as one cooperative persistent kernel (grid barriers between the phases)
cudaError_t launch_step_fused(const StepArgs& A, cudaStream_t st);
// the fused step's scan tile (cells) for A's agent count, cell count and tuning: a fused step that counts the next
// step's keys leaves their per-tile sums in tileSums for a next step with the same tile (else clear both first)
int fusedScanTile(const StepArgs& A);

}  // namespace swarm_gpu
