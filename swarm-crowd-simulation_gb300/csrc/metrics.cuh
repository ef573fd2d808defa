// Arguments of the safety-metric kernels (metrics.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/swarm_cuda.h"

namespace swarm_gpu {

struct MetricArgs {
    const float4* prev;        // the step's input state (GpuBoid: position, velocity interleaved)
    const float4* cur;         // the step's output state
    int32_t n;
    int32_t res;               // metric cells per axis
    float cellsPerUnit, offset, centerX, centerY, speedScale;
    int32_t stadium;           // exit slots by the terrace's avenue gaps (1) or by the venue's exit boxes (0)
    float avenueHalf;
    int32_t nExits;
    const float4* exitBoxes;   // (lo_x, lo_y, hi_x, hi_y) per exit
    SwarmMetricCounters* counters;
    uint32_t* evacStep;
    uint2* mass;               // per cell: mass, speed mass of the step in flight
    const uint4* thresholds;   // per cell: threshold masses
    SwarmMetricCell* cells;
    uint32_t stepIndex;
};

void launch_metrics(const MetricArgs& M, cudaStream_t st);
// The active agents of a state (position.w != 0) into *out (an integer sum: exact, order-independent); *out must be 0
void launch_count_active(const float4* state, int n, uint32_t* out, cudaStream_t st);

}  // namespace swarm_gpu
