// Safety metrics after a step (DedovSergei/swarm-crowd-simulation shaders/metrics_deposit.comp :43-126 and
// shaders/metrics_finalize.comp :37-58; CPU mirror MetricsReference::record, src/metrics.cpp:429-476).
//
// k_metrics_deposit   per agent: the evacuation event (exit slot of its last active position, step index) and the
//                     cloud-in-cell deposit of one person (fixed point: weights on a 1/256-cell lattice that sum to
//                     65536) and of its horizontal speed; integer atomics, so the sums do not depend on order. The
//                     active count is summed per block first (one atomic per block).
// k_metrics_finalize  per floor cell: last / peak mass, occupied steps, steps at or above each threshold mass, 64-bit
//                     sums; clears the step's mass. Cell 0 publishes the step's active count and index.
#include "metrics.cuh"

#include "device_math.cuh"

namespace swarm_gpu {

__device__ __forceinline__ int exitSlot(const MetricArgs& M, float4 p) {
    if (M.stadium) {   // src/metrics.cpp:40-51 (the terrace's avenue gaps)
        const float ax = fabsf(p.x), ay = fabsf(p.y);
        const bool alongY = ay >= ax;
        const float lat = alongY ? ax : ay;
        if (lat >= M.avenueHalf) return 4;
        return alongY ? (p.y > 0.0f ? 2 : 3) : (p.x > 0.0f ? 0 : 1);
    }
    for (int e = 0; e < M.nExits; ++e) {
        const float4 b = M.exitBoxes[e];
        if (p.x >= b.x && p.x <= b.z && p.y >= b.y && p.y <= b.w) return 5 + e;
    }
    return 4;
}

__global__ void k_metrics_deposit(MetricArgs M) {
    __shared__ uint32_t groupActive;
    if (threadIdx.x == 0) groupActive = 0;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < M.n) {
        const float4 p0 = M.prev[2 * size_t(i)], p1 = M.cur[2 * size_t(i)];
        if (p0.w != 0.0f && p1.w == 0.0f) {
            atomicAdd(&M.counters->exits[exitSlot(M, p0)], 1u);
            atomicAdd(&M.counters->evacuated, 1u);
            M.evacStep[i] = M.stepIndex;
        }
        if (p1.w != 0.0f) {
            atomicAdd(&groupActive, 1u);
            const float4 v = M.cur[2 * size_t(i) + 1];
            const float speed = sqrtf(v.x * v.x + v.y * v.y) * M.speedScale;
            // position in cells relative to the centre of cell 0, multiply then add (no fused multiply-add)
            const float gx = (p1.x - M.centerX) * M.cellsPerUnit + M.offset, gy = (p1.y - M.centerY) * M.cellsPerUnit + M.offset;
            const float fx = floorf(gx), fy = floorf(gy);
            const float tx = gx - fx, ty = gy - fy;
            const uint32_t qx = uint32_t(floorf(tx * 256.0f + 0.5f)), qy = uint32_t(floorf(ty * 256.0f + 0.5f));
            const uint32_t rx = 256u - qx, ry = 256u - qy;
            const int ix = int(fx), iy = int(fy), r = M.res;
            const int cs[4] = {sclamp(ix, 0, r - 1) + sclamp(iy, 0, r - 1) * r, sclamp(ix + 1, 0, r - 1) + sclamp(iy, 0, r - 1) * r,
                               sclamp(ix, 0, r - 1) + sclamp(iy + 1, 0, r - 1) * r, sclamp(ix + 1, 0, r - 1) + sclamp(iy + 1, 0, r - 1) * r};
            const uint32_t ws[4] = {rx * ry, qx * ry, rx * qy, qx * qy};
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (ws[k] == 0u) continue;
                atomicAdd(&M.mass[cs[k]].x, ws[k]);
                atomicAdd(&M.mass[cs[k]].y, uint32_t(floorf(float(ws[k]) * speed + 0.5f)));
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && groupActive) atomicAdd(&M.counters->active_accum, groupActive);
}

__device__ __forceinline__ void add64(uint32_t* a, uint32_t b) {
    const uint32_t lo = a[0] + b;
    a[1] += lo < b ? 1u : 0u;
    a[0] = lo;
}

__global__ void k_metrics_finalize(MetricArgs M) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c == 0) {
        M.counters->active = M.counters->active_accum;
        M.counters->active_accum = 0u;
        M.counters->step = M.stepIndex;
    }
    if (c >= M.res * M.res) return;
    const uint2 m = M.mass[c];
    M.mass[c] = make_uint2(0u, 0u);
    const uint4 thr = M.thresholds[c];
    SwarmMetricCell s = M.cells[c];
    s.last_mass = m.x;
    s.last_speed_mass = m.y;
    s.peak_mass = max(s.peak_mass, m.x);
    s.occupied_steps += m.x != 0u ? 1u : 0u;
    s.steps_above[0] += m.x >= thr.x ? 1u : 0u;
    s.steps_above[1] += m.x >= thr.y ? 1u : 0u;
    s.steps_above[2] += m.x >= thr.z ? 1u : 0u;
    s.steps_above[3] += m.x >= thr.w ? 1u : 0u;
    add64(s.mass_steps, m.x);
    add64(s.speed_mass_steps, m.y);
    if (m.x >= thr.z) add64(s.exposure_mass_steps, m.x);
    M.cells[c] = s;
}

__global__ void k_count_active(const float4* __restrict__ state, int n, uint32_t* out) {
    __shared__ uint32_t blockCount;
    if (threadIdx.x == 0) blockCount = 0;
    __syncthreads();
    uint32_t c = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        c += state[2 * size_t(i)].w != 0.0f ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31u) == 0 && c) atomicAdd(&blockCount, c);
    __syncthreads();
    if (threadIdx.x == 0 && blockCount) atomicAdd(out, blockCount);
}

void launch_count_active(const float4* state, int n, uint32_t* out, cudaStream_t st) {
    const int blocks = (n + 255) / 256 < 256 ? (n + 255) / 256 : 256;
    k_count_active<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(state, n, out);
}

void launch_metrics(const MetricArgs& M, cudaStream_t st) {
    k_metrics_deposit<<<(M.n + 255) / 256, 256, 0, st>>>(M);
    const int cells = M.res * M.res;
    k_metrics_finalize<<<(cells + 255) / 256, 256, 0, st>>>(M);
}

}  // namespace swarm_gpu
