// The navigation field on the GPU: the first-order Godunov upwind eikonal solution (the fixed point of the update
// the host's fast marching applies, Sethian 1996) by tiled relaxation (a block-iterative form of Jeong & Whitaker's
// fast iterative method, 2008). Values only decrease from +inf and the update is monotone in its neighbours, so every
// order of updates converges to the same fixed point: the result does not depend on the schedule, and it is the
// fast marching result node for node (FP64 arithmetic, the same operations in the same order).
//
// Layout: the nav grid row-major (x fastest), D in FP64 on the device; tiles of 32 x 32 nodes, one block each. A pass
// runs every active tile: it loads the tile and its one-node ring into shared memory, relaxes it to convergence (at
// most EIK_LOCAL_ITERS sweeps of in-place updates), writes it back and activates the neighbours across each edge it
// changed (itself too if it did not converge). Passes repeat until one activates nothing.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <vector>

#include "../../include/swarm_cuda.h"

namespace swarm_gpu {
namespace {

constexpr int EIK_TILE = 32;
constexpr int EIK_THREADS = 256;          // 32 x 8: each thread owns 4 nodes of a column
constexpr int EIK_LOCAL_ITERS = 64;
constexpr int EIK_PASSES_PER_CHECK = 8;   // passes launched between host reads of the activity counters
constexpr int EIK_MAX_PASSES = 1 << 20;

struct EikArgs {
    int nx, ny, tilesX, tilesY;
    double h;
    const uint8_t* kind;     // 0 free, 1 source, 3 wall
    const float* speed;      // per node (null: 1)
    double* D;
    uint8_t* activeIn;       // tiles to run in this pass (each run clears its own flag)
    uint8_t* activeOut;      // tiles to run in the next pass
    unsigned* activated;     // this pass's count of activations (any nonzero: not converged)
    unsigned long long* runs;
};

__global__ void k_eik_init(const uint8_t* kind, double* D, size_t m) {
    const size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < m) D[k] = kind[k] == 1 ? 0.0 : __longlong_as_double(0x7FF0000000000000ll);
}

// The local update of one free node (the host fast marching's formula, operation for operation)
__device__ __forceinline__ double eikUpdate(double a, double b, double hs) {
    const bool infA = isinf(a), infB = isinf(b);
    if (infA || infB || fabs(a - b) >= hs) return fmin(a, b) + hs;
    return 0.5 * (a + b + sqrt(2.0 * hs * hs - (a - b) * (a - b)));
}

__global__ void __launch_bounds__(EIK_THREADS) k_eik_pass(EikArgs A) {
    const int tile = blockIdx.x;
    __shared__ int run;
    if (threadIdx.x == 0) {   // one thread reads and clears the flag: the block's decision is uniform
        run = A.activeIn[tile];
        if (run) {
            A.activeIn[tile] = 0;
            atomicAdd(A.runs, 1ull);
        }
    }
    __syncthreads();
    if (!run) return;
    const double INF = __longlong_as_double(0x7FF0000000000000ll);
    __shared__ double sD[EIK_TILE + 2][EIK_TILE + 2];
    __shared__ double sH[EIK_TILE][EIK_TILE];   // h / speed of a free node, -1 for a fixed one
    const int x0 = (tile % A.tilesX) * EIK_TILE, y0 = (tile / A.tilesX) * EIK_TILE;
    for (int i = threadIdx.x; i < (EIK_TILE + 2) * (EIK_TILE + 2); i += EIK_THREADS) {
        const int lx = i % (EIK_TILE + 2), ly = i / (EIK_TILE + 2);
        const int gx = x0 - 1 + lx, gy = y0 - 1 + ly;
        const bool in = gx >= 0 && gy >= 0 && gx < A.nx && gy < A.ny;
        sD[ly][lx] = in ? A.D[size_t(gy) * size_t(A.nx) + size_t(gx)] : INF;
    }
    const int lx = threadIdx.x % EIK_TILE, ly0 = threadIdx.x / EIK_TILE;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int ly = ly0 + 8 * r, gx = x0 + lx, gy = y0 + ly;
        double hs = -1.0;
        if (gx < A.nx && gy < A.ny) {
            const size_t g = size_t(gy) * size_t(A.nx) + size_t(gx);
            if (A.kind[g] == 0) hs = A.speed ? A.h / double(A.speed[g]) : A.h;
        }
        sH[ly][lx] = hs;
    }
    // which nodes changed in the last sweep, one bit per node per parity (the ring never changes within a run): a
    // node is updated again only when a neighbour changed, since its update reads nothing else
    __shared__ uint32_t sChg[2][EIK_TILE];   // [parity][row], bit x
    if (threadIdx.x < 2 * EIK_TILE) (&sChg[0][0])[threadIdx.x] = 0u;
    __syncthreads();
    bool eL = false, eR = false, eB = false, eT = false, changed = false;
    int it = 0;
    for (; it < EIK_LOCAL_ITERS; ++it) {
        const uint32_t* prev = sChg[(it + 1) & 1];
        uint32_t* cur = sChg[it & 1];
        bool ch = false;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int ly = ly0 + 8 * r;
            const double hs = sH[ly][lx];
            if (hs < 0.0) continue;
            if (it > 0) {
                const uint32_t row = prev[ly], below = ly > 0 ? prev[ly - 1] : 0u, above = ly + 1 < EIK_TILE ? prev[ly + 1] : 0u;
                const uint32_t side = (lx > 0 ? row >> (lx - 1) : 0u) | (lx + 1 < EIK_TILE ? row >> (lx + 1) : 0u);
                if (!(((side | (below >> lx) | (above >> lx)) & 1u))) continue;
            }
            const double a = fmin(sD[ly + 1][lx], sD[ly + 1][lx + 2]);
            const double b = fmin(sD[ly][lx + 1], sD[ly + 2][lx + 1]);
            const double T = eikUpdate(a, b, hs);
            if (T < sD[ly + 1][lx + 1]) {
                sD[ly + 1][lx + 1] = T;
                ch = true;
                atomicOr(&cur[ly], 1u << lx);
                eL |= lx == 0;
                eR |= lx == EIK_TILE - 1;
                eB |= ly == 0;
                eT |= ly == EIK_TILE - 1;
            }
        }
        changed |= ch;
        if (!__syncthreads_or(ch)) break;
        if (threadIdx.x < EIK_TILE) sChg[(it + 1) & 1][threadIdx.x] = 0u;   // the next sweep's bits (prev is done)
        __syncthreads();
    }
    const bool again = it == EIK_LOCAL_ITERS;   // (the same in every thread: the loop ends on a block-wide vote)
    if (__syncthreads_or(changed)) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int ly = ly0 + 8 * r;
            if (sH[ly][lx] >= 0.0) A.D[size_t(y0 + ly) * size_t(A.nx) + size_t(x0 + lx)] = sD[ly + 1][lx + 1];
        }
    }
    const bool left = __syncthreads_or(eL), right = __syncthreads_or(eR), bottom = __syncthreads_or(eB),
               top = __syncthreads_or(eT);
    if (threadIdx.x == 0) {
        const int tx = tile % A.tilesX, ty = tile / A.tilesX;
        unsigned n = 0;
        auto activate = [&](int t) { A.activeOut[t] = 1; ++n; };
        if (left && tx > 0) activate(tile - 1);
        if (right && tx + 1 < A.tilesX) activate(tile + 1);
        if (bottom && ty > 0) activate(tile - A.tilesX);
        if (top && ty + 1 < A.tilesY) activate(tile + A.tilesX);
        if (again) activate(tile);
        if (n) atomicAdd(A.activated, n);
    }
}

// The largest reached value (non-negative doubles order as their bit patterns)
__global__ void k_eik_max(const double* D, size_t m, unsigned long long* out) {
    unsigned long long best = 0;
    for (size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x; k < m; k += size_t(gridDim.x) * blockDim.x) {
        const double d = D[k];
        if (!isinf(d)) best = max(best, static_cast<unsigned long long>(__double_as_longlong(d)));
    }
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xFFFFFFFFu, best, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, best);
}

// Reached nodes: their distance; walls and unreached nodes: the largest reached distance + 10 m
__global__ void k_eik_out(const double* D, size_t m, const unsigned long long* maxBits, float* out) {
    const size_t k = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= m) return;
    const double d = D[k];
    out[k] = float(isinf(d) ? __longlong_as_double(static_cast<long long>(*maxBits)) + 10.0 : d);
}

}  // namespace
}  // namespace swarm_gpu

using namespace swarm_gpu;

extern "C" int swarm_nav_field_gpu(int nx, int ny, double h, const uint8_t* kind, const float* speed, float* out,
                                   SwarmNavFieldStats* stats) {
    if (nx < 2 || ny < 2 || !(h > 0.0) || !kind || !out) return SWARM_E_INVALID;
    const size_t m = size_t(nx) * size_t(ny);
    if (speed)
        for (size_t k = 0; k < m; ++k)
            if (kind[k] == 0 && !(speed[k] > 0.0f)) return SWARM_E_INVALID;   // a free node must be passable
    const auto t0 = std::chrono::steady_clock::now();
    const int tilesX = (nx + EIK_TILE - 1) / EIK_TILE, tilesY = (ny + EIK_TILE - 1) / EIK_TILE, tiles = tilesX * tilesY;
    uint8_t *dKind = nullptr, *dAct = nullptr;
    float *dSpeed = nullptr, *dOut = nullptr;
    double* dD = nullptr;
    unsigned* dActivated = nullptr;
    unsigned long long *dRuns = nullptr, *dMax = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int rc = SWARM_OK;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == SWARM_OK) rc = e == cudaErrorMemoryAllocation ? SWARM_E_OOM : SWARM_E_CUDA;
        return rc == SWARM_OK;
    };
    int passes = 0;
    unsigned long long runs = 0;
    if (ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) && ok(cudaMalloc(&dKind, m)) &&
        ok(cudaMalloc(&dD, m * sizeof(double))) && ok(cudaMalloc(&dOut, m * sizeof(float))) &&
        ok(cudaMalloc(&dAct, size_t(2) * size_t(tiles))) &&
        ok(cudaMalloc(&dActivated, EIK_PASSES_PER_CHECK * sizeof(unsigned))) &&
        ok(cudaMalloc(&dRuns, 2 * sizeof(unsigned long long))) && (!speed || ok(cudaMalloc(&dSpeed, m * sizeof(float)))) &&
        ok(cudaMemcpyAsync(dKind, kind, m, cudaMemcpyHostToDevice, st)) &&
        (!speed || ok(cudaMemcpyAsync(dSpeed, speed, m * sizeof(float), cudaMemcpyHostToDevice, st))) &&
        ok(cudaMemsetAsync(dAct, 1, size_t(tiles), st)) && ok(cudaMemsetAsync(dAct + tiles, 0, size_t(tiles), st)) &&
        ok(cudaMemsetAsync(dRuns, 0, 2 * sizeof(unsigned long long), st))) {
        dMax = dRuns + 1;
        k_eik_init<<<unsigned((m + 255) / 256), 256, 0, st>>>(dKind, dD, m);
        ok(cudaGetLastError());
        EikArgs A{nx, ny, tilesX, tilesY, h, dKind, dSpeed, dD, dAct, dAct + tiles, nullptr, dRuns};
        cudaEventCreate(&ev[0]);
        cudaEventCreate(&ev[1]);
        cudaEventRecord(ev[0], st);
        unsigned last = 1;
        while (rc == SWARM_OK && last != 0) {
            if (passes >= EIK_MAX_PASSES) { rc = SWARM_E_TIMEOUT; break; }
            if (!ok(cudaMemsetAsync(dActivated, 0, EIK_PASSES_PER_CHECK * sizeof(unsigned), st))) break;
            for (int p = 0; p < EIK_PASSES_PER_CHECK; ++p) {
                A.activated = dActivated + p;
                k_eik_pass<<<unsigned(tiles), EIK_THREADS, 0, st>>>(A);
                std::swap(A.activeIn, A.activeOut);
            }
            passes += EIK_PASSES_PER_CHECK;
            if (!ok(cudaGetLastError()) ||
                !ok(cudaMemcpyAsync(&last, dActivated + EIK_PASSES_PER_CHECK - 1, sizeof(unsigned), cudaMemcpyDeviceToHost, st)) ||
                !ok(cudaStreamSynchronize(st)))
                break;
        }
        cudaEventRecord(ev[1], st);
        if (rc == SWARM_OK) {
            k_eik_max<<<1024, 256, 0, st>>>(dD, m, dMax);
            k_eik_out<<<unsigned((m + 255) / 256), 256, 0, st>>>(dD, m, dMax, dOut);
            ok(cudaGetLastError());
            ok(cudaMemcpyAsync(out, dOut, m * sizeof(float), cudaMemcpyDeviceToHost, st));
            ok(cudaMemcpyAsync(&runs, dRuns, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
            ok(cudaStreamSynchronize(st));
        }
    }
    if (st) cudaStreamSynchronize(st);
    cudaFree(dKind);
    cudaFree(dSpeed);
    cudaFree(dOut);
    cudaFree(dD);
    cudaFree(dAct);
    cudaFree(dActivated);
    cudaFree(dRuns);
    float solveMs = 0.0f;
    if (ev[0] && ev[1] && rc == SWARM_OK) cudaEventElapsedTime(&solveMs, ev[0], ev[1]);
    for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
    if (st) cudaStreamDestroy(st);
    if (stats) {
        stats->ms_solve = solveMs;
        stats->passes = passes;
        stats->tiles = tiles;
        stats->tile_runs = int64_t(runs);
        stats->ms = float(std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
    }
    return rc;
}
