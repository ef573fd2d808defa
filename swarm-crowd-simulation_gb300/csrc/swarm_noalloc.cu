// swarm_sort_grid_noalloc: the key sort of one state without any device allocation.
//
// Some callers cannot allocate device memory while they run. A plug-in step inside a host application's frame loop
// may not call cudaMalloc or cudaFree: both can synchronise the whole device, and the host owns the device's memory
// budget. A deployment that reserves its whole footprint at start-up (a fixed pool, or a process sharing the GPU
// under a hard memory limit) must not grow it later. This entry point sorts a state that already lives in device
// memory (the caller passes the state and the three output arrays) and keeps its working memory in a file-scope
// __device__ array of fixed size instead of allocating it.
//
// Limits: at most NOALLOC_MAX_AGENTS agents and NOALLOC_MAX_CELLS cells. The scratch array (about 1.8 MB) is part of
// this library's device image: every GPU that loads the library holds it until the process exits. Every call uses
// the same array and leaves its contents behind; each call clears what it needs at zero first. Two calls whose
// work overlaps on the GPU (from different host threads) race on the array: order them. The first call on a device
// looks up the array's device address (cudaGetSymbolAddress) with that device current and keeps it for the process;
// a cudaDeviceReset discards the module the address belongs to, so the library must not be called on that device
// after a reset (load it again in a new process).
//
// The call returns once its work on `stream` has finished: it reads back the kernels' bounds-check word, so an
// out-of-range slot (only possible when calls race on the array) returns SWARM_E_CUDA instead of a silent drop.
//
// Output, as the step's own sort: grid_id[slot] = the cell key (0xFFFFFFFF for evacuated agents, which sort last),
// boid_id[slot] = the agent (ascending within each cell and within the evacuated tail), cells[2c], cells[2c + 1] =
// (first slot, agent count) of cell c ((0, 0) when empty). A NaN position is hashed as (0, 0, 0, 1), as the step's
// hash does, but the input state is not written.

#include "../../include/swarm_cuda.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <tuple>

namespace {

constexpr int NOALLOC_MAX_AGENTS = 65536;
constexpr int NOALLOC_MAX_CELLS = 131072;
constexpr int NA_THREADS = 256, NA_ITEMS = 8, NA_TILE = NA_THREADS * NA_ITEMS;
constexpr int NA_MAX_TILES = (NOALLOC_MAX_CELLS + 1 + NA_TILE - 1) / NA_TILE + 1;
constexpr int NA_MAX_AGENT_TILES = (NOALLOC_MAX_AGENTS + NA_TILE - 1) / NA_TILE + 1;

// the scratch layout, in 32-bit words
constexpr size_t OFF_KEY = 0;                                          // cell key per agent
constexpr size_t OFF_RANK = OFF_KEY + NOALLOC_MAX_AGENTS;               // arrival rank in its cell's counter
constexpr size_t OFF_TMP = OFF_RANK + NOALLOC_MAX_AGENTS;               // ids in arrival order per cell
constexpr size_t OFF_COUNT = OFF_TMP + NOALLOC_MAX_AGENTS;              // per-cell counts (+ the evacuated bucket)
constexpr size_t OFF_START = OFF_COUNT + NOALLOC_MAX_CELLS + 1;         // their exclusive scan
constexpr size_t OFF_TILES = OFF_START + NOALLOC_MAX_CELLS + 1;         // the cell scan's tile totals
constexpr size_t OFF_ATILES = OFF_TILES + NA_MAX_TILES;                 // the evacuated tail's tile totals
constexpr size_t OFF_ERR = OFF_ATILES + NA_MAX_AGENT_TILES;             // bounds-check word (0: every index in range)
constexpr size_t SCRATCH_WORDS = OFF_ERR + 1;

static __device__ __align__(256) uint32_t g_noallocScratch[SCRATCH_WORDS];

struct Grid { int resX, resY, ncells; float minX, minY, spanX, spanY; };

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (hi < v ? hi : v); }

__device__ __forceinline__ uint32_t keyOf(const float4* boids, int i, const Grid& g) {
    float4 p = boids[2 * size_t(i)];
    if (isnan(p.x)) p = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    if (p.w == 0.0f) return 0xFFFFFFFFu;
    const int x = clampi(int((p.x - g.minX) / g.spanX * float(g.resX)), 0, g.resX - 1);
    const int y = clampi(int((p.y - g.minY) / g.spanY * float(g.resY)), 0, g.resY - 1);
    return uint32_t(x + y * g.resX);
}

__global__ void na_clear(uint32_t* scratch, int ncells) {
    if (blockIdx.x == 0 && threadIdx.x == 0) scratch[OFF_ERR] = 0u;
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b <= ncells; b += gridDim.x * blockDim.x) scratch[OFF_COUNT + b] = 0u;
}

__device__ __forceinline__ void naOutOfRange(uint32_t* scratch) { atomicOr(scratch + OFF_ERR, 1u); }

__global__ void na_hash(const float4* boids, int n, Grid g, uint32_t* scratch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t key = keyOf(boids, i, g);
    const uint32_t bucket = key == 0xFFFFFFFFu ? uint32_t(g.ncells) : key;
    scratch[OFF_KEY + i] = key;
    scratch[OFF_RANK + i] = atomicAdd(scratch + OFF_COUNT + bucket, 1u);
}

__device__ __forceinline__ uint32_t blockScan(uint32_t v, uint32_t* warpSums, uint32_t& total) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (int(lane) >= o) inc += u;
    }
    if (lane == 31) warpSums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < NA_THREADS / 32 ? warpSums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, w, o);
            if (int(lane) >= o) w += u;
        }
        if (lane < NA_THREADS / 32) warpSums[lane] = w;
    }
    __syncthreads();
    total = warpSums[NA_THREADS / 32 - 1];
    return inc - v + (warp > 0 ? warpSums[warp - 1] : 0u);
}

// Tiled exclusive scan of `len` words at `src` (value(i) = src[i], or for the tail: agent i is evacuated)
template <bool kTail>
__device__ __forceinline__ uint32_t naValue(const uint32_t* scratch, int i) {
    return kTail ? (scratch[OFF_KEY + i] == 0xFFFFFFFFu ? 1u : 0u) : scratch[OFF_COUNT + i];
}

template <bool kTail>
__global__ void na_scan_reduce(uint32_t* scratch, int len) {
    __shared__ uint32_t warpSums[32];
    const int base = blockIdx.x * NA_TILE + threadIdx.x * NA_ITEMS;
    uint32_t sum = 0;
    for (int j = 0; j < NA_ITEMS; ++j) sum += base + j < len ? naValue<kTail>(scratch, base + j) : 0u;
    uint32_t total;
    blockScan(sum, warpSums, total);
    if (threadIdx.x == 0) scratch[(kTail ? OFF_ATILES : OFF_TILES) + blockIdx.x] = total;
}

// The cell scan: run starts and the cell table
__global__ void na_scan_cells(uint32_t* scratch, int ncells, uint32_t* cellsOut) {
    __shared__ uint32_t warpSums[32];
    __shared__ uint32_t prefix;
    const int len = ncells + 1;
    uint32_t p = 0;
    for (int t = threadIdx.x; t < int(blockIdx.x); t += NA_THREADS) p += scratch[OFF_TILES + t];
    for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
    if (threadIdx.x == 0) prefix = 0;
    __syncthreads();
    if ((threadIdx.x & 31u) == 0 && p) atomicAdd(&prefix, p);
    const int base = blockIdx.x * NA_TILE + threadIdx.x * NA_ITEMS;
    uint32_t c[NA_ITEMS], sum = 0;
    for (int j = 0; j < NA_ITEMS; ++j) { c[j] = base + j < len ? scratch[OFF_COUNT + base + j] : 0u; sum += c[j]; }
    uint32_t total;
    uint32_t run = blockScan(sum, warpSums, total) + prefix;
    for (int j = 0; j < NA_ITEMS; ++j) {
        const int b = base + j;
        if (b >= len) break;
        scratch[OFF_START + b] = run;
        if (b < ncells) { cellsOut[2 * b] = c[j] ? run : 0u; cellsOut[2 * b + 1] = c[j]; }
        run += c[j];
    }
}

// Active agents: scatter in arrival order (their final place follows in na_rank)
__global__ void na_scatter(int n, int ncells, uint32_t* scratch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t key = scratch[OFF_KEY + i];
    if (key == 0xFFFFFFFFu) return;
    const uint32_t slot = scratch[OFF_START + key] + scratch[OFF_RANK + i];
    if (slot < uint32_t(n)) scratch[OFF_TMP + slot] = uint32_t(i);
    else naOutOfRange(scratch);
}

// Active slots: each agent's place is its rank by id among its cell's agents
__global__ void na_rank(int n, int ncells, uint32_t* scratch, uint32_t* gridOut, uint32_t* idOut) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int nActive = int(scratch[OFF_START + ncells]);
    if (s >= n || s >= nActive) return;
    const uint32_t me = scratch[OFF_TMP + s];
    if (me >= uint32_t(n)) { naOutOfRange(scratch); return; }
    const uint32_t c = scratch[OFF_KEY + me];
    if (c >= uint32_t(ncells)) { naOutOfRange(scratch); return; }
    const uint32_t st = scratch[OFF_START + c], cnt = scratch[OFF_START + c + 1] - st;
    if (st + cnt > uint32_t(n)) { naOutOfRange(scratch); return; }
    uint32_t r = 0;
    for (uint32_t j = st; j < st + cnt; ++j) r += scratch[OFF_TMP + j] < me ? 1u : 0u;
    gridOut[st + r] = c;
    idOut[st + r] = me;
}

// The evacuated tail in id order: place = nActive + (evacuated agents with a smaller id)
__global__ void na_tail(int n, int ncells, uint32_t* scratch, uint32_t* gridOut, uint32_t* idOut) {
    __shared__ uint32_t warpSums[32];
    __shared__ uint32_t prefix;
    uint32_t p = 0;
    for (int t = threadIdx.x; t < int(blockIdx.x); t += NA_THREADS) p += scratch[OFF_ATILES + t];
    for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
    if (threadIdx.x == 0) prefix = 0;
    __syncthreads();
    if ((threadIdx.x & 31u) == 0 && p) atomicAdd(&prefix, p);
    const int base = blockIdx.x * NA_TILE + threadIdx.x * NA_ITEMS;
    uint32_t f[NA_ITEMS], sum = 0;
    for (int j = 0; j < NA_ITEMS; ++j) { f[j] = base + j < n ? naValue<true>(scratch, base + j) : 0u; sum += f[j]; }
    uint32_t total;
    uint32_t run = blockScan(sum, warpSums, total) + prefix + scratch[OFF_START + ncells];
    for (int j = 0; j < NA_ITEMS; ++j) {
        if (!f[j]) continue;
        if (run >= uint32_t(n)) { naOutOfRange(scratch); break; }
        gridOut[run] = 0xFFFFFFFFu;
        idOut[run] = uint32_t(base + j);
        run += 1;
    }
}

std::mutex g_setupMutex;
uint32_t* g_scratchPtr[64] = {};   // per device ordinal

}  // namespace

// One launch; its own error, without reading or clearing an error that an earlier, unrelated call left behind
template <class... Params, class... Args>
cudaError_t naLaunch(void (*kernel)(Params...), int grid, int block, cudaStream_t st, Args... args) {
    static_assert(sizeof...(Params) == sizeof...(Args), "argument count");
    std::tuple<Params...> typed(args...);   // each argument converted to the kernel's own parameter type
    return std::apply([&](auto&... a) {
        void* argv[] = {static_cast<void*>(&a)...};
        return cudaLaunchKernel(reinterpret_cast<const void*>(kernel), dim3(unsigned(grid)), dim3(unsigned(block)), argv, 0, st);
    }, typed);
}

extern "C" int swarm_sort_grid_noalloc(const float* d_boids, int n, int grid_res_x, int grid_res_y, float domain_min_x,
                                       float domain_min_y, float domain_span_x, float domain_span_y, uint32_t* d_grid_id,
                                       uint32_t* d_boid_id, uint32_t* d_cells, void* stream) {
    if (!d_boids || !d_grid_id || !d_boid_id || !d_cells) return SWARM_E_INVALID;
    if (n <= 0 || n > NOALLOC_MAX_AGENTS) return SWARM_E_INVALID;
    if (grid_res_x <= 0 || grid_res_y <= 0 || double(grid_res_x) * double(grid_res_y) > double(NOALLOC_MAX_CELLS)) return SWARM_E_INVALID;
    if (!(domain_span_x > 0.0f) || !(domain_span_y > 0.0f)) return SWARM_E_INVALID;
    // the state is read as float4, the outputs as 32-bit words
    if (reinterpret_cast<uintptr_t>(d_boids) & 15u) return SWARM_E_INVALID;
    if ((reinterpret_cast<uintptr_t>(d_grid_id) | reinterpret_cast<uintptr_t>(d_boid_id) | reinterpret_cast<uintptr_t>(d_cells)) & 3u)
        return SWARM_E_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return SWARM_E_CUDA;
    uint32_t* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setupMutex);
        if (!g_scratchPtr[dev]) {   // once per device, with that device current
            void* ptr = nullptr;
            if (cudaGetSymbolAddress(&ptr, g_noallocScratch) != cudaSuccess || !ptr) return SWARM_E_CUDA;
            g_scratchPtr[dev] = static_cast<uint32_t*>(ptr);
        }
        scratch = g_scratchPtr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const Grid g{grid_res_x, grid_res_y, grid_res_x * grid_res_y, domain_min_x, domain_min_y, domain_span_x, domain_span_y};
    const float4* boids = reinterpret_cast<const float4*>(d_boids);
    const int blocksN = (n + 255) / 256;
    const int cellTiles = (g.ncells + 1 + NA_TILE - 1) / NA_TILE;
    const int agentTiles = (n + NA_TILE - 1) / NA_TILE;
    const int nc = g.ncells;
    cudaError_t e = naLaunch(na_clear, (nc + 1 + 255) / 256, 256, st, scratch, nc);
    if (e == cudaSuccess) e = naLaunch(na_hash, blocksN, 256, st, boids, n, g, scratch);
    if (e == cudaSuccess) e = naLaunch(na_scan_reduce<false>, cellTiles, NA_THREADS, st, scratch, nc + 1);
    if (e == cudaSuccess) e = naLaunch(na_scan_cells, cellTiles, NA_THREADS, st, scratch, nc, d_cells);
    if (e == cudaSuccess) e = naLaunch(na_scatter, blocksN, 256, st, n, nc, scratch);
    if (e == cudaSuccess) e = naLaunch(na_rank, blocksN, 256, st, n, nc, scratch, d_grid_id, d_boid_id);
    if (e == cudaSuccess) e = naLaunch(na_scan_reduce<true>, agentTiles, NA_THREADS, st, scratch, n);
    if (e == cudaSuccess) e = naLaunch(na_tail, agentTiles, NA_THREADS, st, n, nc, scratch, d_grid_id, d_boid_id);
    if (e != cudaSuccess) return SWARM_E_CUDA;
    // the bounds-check word, read back in stream order into host stack memory (no allocation)
    uint32_t outOfRange = 0;
    if (cudaMemcpyAsync(&outOfRange, scratch + OFF_ERR, sizeof outOfRange, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return SWARM_E_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return SWARM_E_CUDA;
    return outOfRange ? SWARM_E_CUDA : SWARM_OK;
}
