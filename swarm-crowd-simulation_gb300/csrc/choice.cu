// Queue-aware exit choice on grid venues: the reference's ExitChoice::QueueAware (physics.comp PHYSICS_PASS 0;
// nav::choiceStep and its stages evaluate / switchThreshold / apply, DedovSergei/swarm-crowd-simulation
// src/exit_choice.cpp:580-790; constants include/swarm/sim_params.hpp:395-427, include/swarm/exit_choice.hpp:121-137),
// restated for venues whose exits have their own distance fields on the nav grid.
//
// Each step, before the step's kernels, on the step's input state (agent order), four launches:
//   k_choice_prefix  per exit: the previous step's queue-ahead histogram (read parity) to exclusive prefix sums; the
//                    write parity's histogram and exit counts cleared
//   k_choice_eval    evaluation steps: per agent, its cell's candidates' estimated times E = d / V_FREE + A x 60 /
//                    (w J); an agent that gains more than both margins by switching is eligible: its gain bin goes
//                    into its exit's histogram
//   k_choice_thr     evaluation steps: per exit, the lowest gain bin whose eligible agents (with those above) fit the
//                    switch cap max(1, 10 % of the exit's agents); the histogram cleared
//   k_choice_apply   per agent: a forced choice (its exit is no candidate of its cell: the best candidate), else an
//                    eligible switch whose bin reaches its exit's threshold; then its count in its exit's queue and in
//                    the queue-ahead histogram at its cell's distance bin
// Every count is an integer atomic, so the result does not depend on the order the agents run in: the oracle's
// sequential pass gives the same assignments. The step's e_goal then follows the assigned exit's field.
//
// The candidate table lives on the hash cells: the reachable nav node nearest a cell's centre stands for the cell (the
// reference's FIT cell / nearest FIT neighbour rule, over nodes instead of navigation cells), and its candidates are
// the type rule's exits (the 2 nearest avenues, the nearest door) and the nearest others, ascending.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "device_math.cuh"
#include "sim_handle.cuh"
#include "step_kernels.cuh"

namespace swarm_gpu {

constexpr float CHOICE_T_S = 3.0f;            // re-evaluation interval (T_CHOICE_S)
constexpr float CHOICE_REL_MARGIN = 0.10f;    // hysteresis: share of E_current ...
constexpr float CHOICE_ABS_MARGIN_S = 5.0f;   // ... and seconds
constexpr float CHOICE_SWITCH_SHARE = 0.10f;  // per evaluation at most this share of an exit's agents switch away
constexpr uint32_t CHOICE_MIN_SWITCHES = 1;
constexpr int CHOICE_GAIN_BINS = 256;         // 1 s gain bins; gains >= 255 s in the last
constexpr int CHOICE_AHEAD_BINS = 1024;       // queue-ahead distance bins per exit (0.5 m; the last: 511.5 m on)
constexpr int CHOICE_STRIDE = 64;             // counts per parity (exit ids 0 .. 62)
constexpr float CHOICE_V_FREE = 1.34f;        // V_FREE_M_S, the estimate's walking speed
constexpr double CHOICE_J = 83.6;             // EXIT_FLOW_P_M_MIN, persons per metre of clear width per minute
constexpr int CHOICE_TYPE_MIN[2] = {2, 1};    // the type rule: nearest avenues, nearest doors

// seconds per metre of the estimate's walk, folded once in double
constexpr float CHOICE_S_PER_M = float(1.0 / double(CHOICE_V_FREE));

inline int choiceSteps(float dt) { return std::max(1, int(double(CHOICE_T_S) / double(dt) + 0.5)); }

struct ChoiceArgs {
    VenueArgs V;
    int n, nExits, K;
    uint32_t step;
    int evalStep;
    const float4* state;          // the step's input state (agent order)
    const uint8_t* cExit;         // ncells x K candidate exits
    const float* cDist;           // ncells x K candidate distances
    const float* invCap;          // per exit: seconds per queued agent, 60 / (w J)
    uint32_t* assign;             // per agent (SWARM_CHOICE_NONE: none)
    uint2* pending;               // per agent: (eligible switch's exit or NONE, gain bin)
    uint32_t* hist;               // nExits x CHOICE_GAIN_BINS
    uint32_t* threshold;          // per exit
    uint32_t* queue;              // 2 x CHOICE_STRIDE (parities)
    uint32_t* ahead;              // 2 x CHOICE_STRIDE x CHOICE_AHEAD_BINS
    uint32_t* counters;           // evaluations, eligible, switches, forced
};

__device__ __forceinline__ uint32_t aheadBin(float d) {
    return min(uint32_t(d * 2.0f), uint32_t(CHOICE_AHEAD_BINS - 1));
}

__device__ __forceinline__ float estimate(const ChoiceArgs& C, float d, uint32_t e, uint32_t queued) {
    const float walk = d * CHOICE_S_PER_M;
    const float wait = float(queued) * C.invCap[e];
    return walk + wait;
}

__device__ __forceinline__ int slotOf(const ChoiceArgs& C, size_t row, uint32_t e) {
    int k = -1;
    for (int i = 0; i < C.K; ++i)
        if (uint32_t(C.cExit[row + size_t(i)]) == e) k = i;
    return k;
}

__device__ __forceinline__ int bestCandidate(const ChoiceArgs& C, size_t row, const uint32_t* aRead, float& eBest) {
    int best = -1;
    eBest = 0.0f;
    for (int k = 0; k < C.K; ++k) {
        const uint32_t ex = C.cExit[row + size_t(k)];
        if (ex == SWARM_CHOICE_EMPTY) break;
        const float d = C.cDist[row + size_t(k)];
        const float e = estimate(C, d, ex, aRead[size_t(ex) * CHOICE_AHEAD_BINS + aheadBin(d)]);
        if (best < 0 || e < eBest) { best = k; eBest = e; }
    }
    return best;
}

// The agent's cell (the step's hash of its start-of-step position, NaN sanitised as the hash does), or -1 when it
// is evacuated
__device__ __forceinline__ long long choiceRow(const ChoiceArgs& C, int i) {
    float4 p = C.state[2 * size_t(i)];
    if (isnan(p.x)) p = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    if (p.w == 0.0f) return -1;
    const int x = sclamp(int((p.x - C.V.dminX) / C.V.dspanX * float(C.V.resX)), 0, C.V.resX - 1);
    const int y = sclamp(int((p.y - C.V.dminY) / C.V.dspanY * float(C.V.resY)), 0, C.V.resY - 1);
    return (long long)(x + y * C.V.resX) * C.K;
}

// Stage 3 of the reference (first of a step): per exit (one block each) the read parity's queue-ahead histogram to
// exclusive prefix sums in place, the write parity's cleared; block 0 also clears the write parity's exit counts
__global__ void __launch_bounds__(256) k_choice_prefix(ChoiceArgs C) {
    __shared__ uint32_t warpTot[8];
    const int e = blockIdx.x;
    const uint32_t par = C.step & 1u;
    uint32_t* aRead = C.ahead + (size_t(par) * CHOICE_STRIDE + size_t(e)) * CHOICE_AHEAD_BINS;
    uint32_t* aWrite = C.ahead + (size_t(1u - par) * CHOICE_STRIDE + size_t(e)) * CHOICE_AHEAD_BINS;
    constexpr int PER = CHOICE_AHEAD_BINS / 256;   // 4 bins a thread, in order
    uint32_t v[PER], sum = 0;
#pragma unroll
    for (int j = 0; j < PER; ++j) { v[j] = aRead[threadIdx.x * PER + j]; sum += v[j]; }
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t inc = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (int(lane) >= o) inc += u;
    }
    if (lane == 31) warpTot[warp] = inc;
    __syncthreads();
    uint32_t before = 0;
    for (unsigned w = 0; w < warp; ++w) before += warpTot[w];
    uint32_t run = before + inc - sum;
#pragma unroll
    for (int j = 0; j < PER; ++j) { aRead[threadIdx.x * PER + j] = run; run += v[j]; aWrite[threadIdx.x * PER + j] = 0u; }
    if (e == 0 && threadIdx.x < CHOICE_STRIDE) C.queue[(1u - par) * CHOICE_STRIDE + threadIdx.x] = 0u;
}

// Stage 1: nav::evaluate (src/exit_choice.cpp:605-623) for every agent
__global__ void __launch_bounds__(256) k_choice_eval(ChoiceArgs C) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C.n) return;
    C.pending[i] = make_uint2(SWARM_CHOICE_NONE, 0u);
    const long long r = choiceRow(C, i);
    if (r < 0) return;
    const size_t row = size_t(r);
    if (C.cExit[row] == SWARM_CHOICE_EMPTY) return;
    const uint32_t cur = C.assign[i];
    const int curK = slotOf(C, row, cur);
    if (curK < 0) return;
    atomicAdd(C.counters + 0, 1u);
    const uint32_t* aRead = C.ahead + size_t(C.step & 1u) * CHOICE_STRIDE * CHOICE_AHEAD_BINS;
    float eBest;
    const int best = bestCandidate(C, row, aRead, eBest);
    const float dCur = C.cDist[row + size_t(curK)];
    const float eCur = estimate(C, dCur, cur, aRead[size_t(cur) * CHOICE_AHEAD_BINS + aheadBin(dCur)]);
    const float gain = eCur - eBest;
    if (best != curK && gain > fmaxf(CHOICE_REL_MARGIN * eCur, CHOICE_ABS_MARGIN_S)) {
        const uint32_t bin = min(uint32_t(gain), uint32_t(CHOICE_GAIN_BINS - 1));
        C.pending[i] = make_uint2(uint32_t(C.cExit[row + size_t(best)]), bin);
        atomicAdd(C.hist + size_t(cur) * CHOICE_GAIN_BINS + bin, 1u);
        atomicAdd(C.counters + 1, 1u);
    }
}

// Stage 2: nav::switchThreshold (src/exit_choice.cpp:625-640) per exit, then the exit's histogram cleared
__global__ void k_choice_thr(ChoiceArgs C) {
    const int e = threadIdx.x;
    if (e >= C.nExits) return;
    uint32_t* h = C.hist + size_t(e) * CHOICE_GAIN_BINS;
    const uint32_t queued = C.queue[(C.step & 1u) * CHOICE_STRIDE + uint32_t(e)];
    const uint32_t cap = max(CHOICE_MIN_SWITCHES, uint32_t(float(queued) * CHOICE_SWITCH_SHARE));
    uint32_t cum = 0, thr = uint32_t(CHOICE_GAIN_BINS);
    for (int b = CHOICE_GAIN_BINS - 1; b >= 0; --b) {
        const uint32_t c = h[b];
        if (c == 0) continue;
        if (cum + c > cap) {
            if (cum == 0) thr = uint32_t(b);   // the highest bin alone exceeds the cap: it switches anyway
            break;
        }
        cum += c;
        thr = uint32_t(b);
    }
    C.threshold[e] = thr;
    for (int b = 0; b < CHOICE_GAIN_BINS; ++b) h[b] = 0u;
}

// Stage 0: nav::apply (src/exit_choice.cpp:642-658) and the agent's counts for the next step. The counts are sums of
// ones, aggregated before they reach global memory (the exit counts per block in shared memory, the queue-ahead bins
// per warp): the same integers, a few atomics per block instead of one per agent on ~40 addresses.
__global__ void __launch_bounds__(256) k_choice_apply(ChoiceArgs C) {
    __shared__ uint32_t sQueue[CHOICE_STRIDE];
    if (threadIdx.x < CHOICE_STRIDE) sQueue[threadIdx.x] = 0u;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t par = C.step & 1u;
    uint32_t aheadKey = 0xFFFFFFFFu;   // exit x CHOICE_AHEAD_BINS + bin of this agent's count (none: all ones)
    const long long r = i < C.n ? choiceRow(C, i) : -1;
    if (r >= 0) {
        const size_t row = size_t(r);
        const uint32_t* aRead = C.ahead + size_t(par) * CHOICE_STRIDE * CHOICE_AHEAD_BINS;
        const uint32_t cur = C.assign[i];
        uint32_t ex = cur;
        const bool hasPath = C.cExit[row] != SWARM_CHOICE_EMPTY;
        const int curK = hasPath ? slotOf(C, row, cur) : -1;
        if (hasPath && curK < 0) {   // forced (or the first choice)
            float eBest;
            ex = C.cExit[row + size_t(bestCandidate(C, row, aRead, eBest))];
            if (cur != SWARM_CHOICE_NONE) atomicAdd(C.counters + 3, 1u);
        } else if (C.evalStep && curK >= 0) {
            const uint2 pd = C.pending[i];
            if (pd.x != SWARM_CHOICE_NONE && pd.y >= C.threshold[cur]) {
                ex = pd.x;
                atomicAdd(C.counters + 2, 1u);
            }
        }
        C.assign[i] = ex;
        if (ex != SWARM_CHOICE_NONE) {
            atomicAdd(sQueue + ex, 1u);
            const int k = slotOf(C, row, ex);
            if (k >= 0) aheadKey = ex * uint32_t(CHOICE_AHEAD_BINS) + aheadBin(C.cDist[row + size_t(k)]);
        }
    }
    // the queue-ahead count: one atomic per distinct (exit, bin) in the warp
    const unsigned lane = threadIdx.x & 31u;
    const unsigned valid = __ballot_sync(0xffffffffu, aheadKey != 0xFFFFFFFFu);
    if (aheadKey != 0xFFFFFFFFu) {
        const unsigned peers = __match_any_sync(valid, aheadKey);
        if (int(lane) == __ffs(peers) - 1)
            atomicAdd(C.ahead + size_t(1u - par) * CHOICE_STRIDE * CHOICE_AHEAD_BINS + aheadKey, uint32_t(__popc(peers)));
    }
    __syncthreads();
    if (threadIdx.x < CHOICE_STRIDE && sQueue[threadIdx.x])
        atomicAdd(C.queue + (1u - par) * CHOICE_STRIDE + threadIdx.x, sQueue[threadIdx.x]);
}

}  // namespace swarm_gpu

// ---- host: the candidate table ----
namespace {

bool validChoice(const SwarmVenue* v, const SwarmExitChoiceSpec* c) {
    return v && c && v->kind == SWARM_VENUE_GRID && v->nav_nx > 0 && v->nav_ny > 0 && v->grid_res_x > 0 && v->grid_res_y > 0 &&
           c->n_exits >= 1 && c->n_exits <= SWARM_CHOICE_MAX_EXITS && c->candidates >= 1 &&
           c->candidates <= SWARM_CHOICE_MAX_CANDIDATES && c->fields && c->type;
}

}  // namespace

extern "C" int swarm_exit_choice_table(const SwarmVenue* v, const SwarmExitChoiceSpec* c, uint8_t* exits, float* dists) {
    if (!validChoice(v, c) || !exits || !dists) return SWARM_E_INVALID;
    const int nx = v->nav_nx, ny = v->nav_ny, E = c->n_exits, K = c->candidates;
    const size_t m = size_t(nx) * size_t(ny), cells = size_t(v->grid_res_x) * size_t(v->grid_res_y);
    // walls and unreached nodes hold each field's largest value: a node is reachable for e below it
    std::vector<float> top(size_t(E), 0.0f);
    for (int e = 0; e < E; ++e) {
        const float* f = c->fields + size_t(e) * m;
        float t = f[0];
        for (size_t k = 1; k < m; ++k) t = std::max(t, f[k]);
        top[size_t(e)] = t;
    }
    // each cell's node: the node reachable for some exit nearest the cell's centre (ties: the lower node index)
    std::vector<long long> node(cells, -1);
    std::vector<double> best(cells, 0.0);
    const double csx = double(v->domain_span_x) / v->grid_res_x, csy = double(v->domain_span_y) / v->grid_res_y;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const double x = double(v->nav_origin_x) + i * double(v->nav_h), y = double(v->nav_origin_y) + j * double(v->nav_h);
            const double fx = (x - v->domain_min_x) / csx, fy = (y - v->domain_min_y) / csy;
            if (fx < 0.0 || fy < 0.0 || fx >= v->grid_res_x || fy >= v->grid_res_y) continue;
            const size_t k = size_t(j) * size_t(nx) + size_t(i);
            bool reach = false;
            for (int e = 0; e < E && !reach; ++e) reach = c->fields[size_t(e) * m + k] < top[size_t(e)];
            if (!reach) continue;
            const int cx = int(fx), cy = int(fy);
            const size_t cell = size_t(cy) * size_t(v->grid_res_x) + size_t(cx);
            const double dx = x - (v->domain_min_x + (cx + 0.5) * csx), dy = y - (v->domain_min_y + (cy + 0.5) * csy);
            const double d2 = dx * dx + dy * dy;
            if (node[cell] < 0 || d2 < best[cell]) { node[cell] = (long long)k; best[cell] = d2; }
        }
    std::vector<std::pair<float, int>> cand;
    std::vector<char> taken(static_cast<size_t>(E), 0);
    for (size_t cell = 0; cell < cells; ++cell) {
        uint8_t* ex = exits + cell * size_t(K);
        float* di = dists + cell * size_t(K);
        std::fill(ex, ex + K, uint8_t(SWARM_CHOICE_EMPTY));
        std::fill(di, di + K, 0.0f);
        if (node[cell] < 0) continue;
        const size_t k = size_t(node[cell]);
        cand.clear();
        for (int e = 0; e < E; ++e) {
            const float d = c->fields[size_t(e) * m + k];
            if (d < top[size_t(e)]) cand.push_back({d, e});
        }
        std::sort(cand.begin(), cand.end());   // ascending distance, ties the lower exit id
        std::fill(taken.begin(), taken.end(), 0);
        std::vector<std::pair<float, int>> pick;
        for (int t = 0; t < 2; ++t) {   // the type rule first
            int got = 0;
            for (const auto& q : cand)
                if (got < swarm_gpu::CHOICE_TYPE_MIN[t] && int(pick.size()) < K && c->type[q.second] == t && !taken[size_t(q.second)]) {
                    pick.push_back(q);
                    taken[size_t(q.second)] = 1;
                    ++got;
                }
        }
        for (const auto& q : cand)   // then the nearest others
            if (int(pick.size()) < K && !taken[size_t(q.second)]) { pick.push_back(q); taken[size_t(q.second)] = 1; }
        std::sort(pick.begin(), pick.end());
        for (size_t q = 0; q < pick.size(); ++q) { ex[q] = uint8_t(pick[q].second); di[q] = pick[q].first; }
    }
    return SWARM_OK;
}

// ---- the handle ----
using swarm_gpu::ChoiceArgs;

bool SwarmSim::resetChoice() {
    choiceStep = 0;
    if (!choiceExits) return true;
    const size_t N = size_t(capacity);
    return cudaMemsetAsync(dAssign, 0xFF, N * 4, stream) == cudaSuccess &&
           cudaMemsetAsync(dPending, 0xFF, N * 8, stream) == cudaSuccess &&
           cudaMemsetAsync(dChoiceHist, 0, size_t(choiceExits) * swarm_gpu::CHOICE_GAIN_BINS * 4, stream) == cudaSuccess &&
           cudaMemsetAsync(dChoiceThr, 0, size_t(swarm_gpu::CHOICE_STRIDE) * 4, stream) == cudaSuccess &&
           cudaMemsetAsync(dChoiceQueue, 0, size_t(2) * swarm_gpu::CHOICE_STRIDE * 4, stream) == cudaSuccess &&
           cudaMemsetAsync(dChoiceAhead, 0, size_t(2) * swarm_gpu::CHOICE_STRIDE * swarm_gpu::CHOICE_AHEAD_BINS * 4, stream) == cudaSuccess &&
           cudaMemsetAsync(dChoiceCounters, 0, 16, stream) == cudaSuccess;
}

void SwarmSim::freeChoice() {
    cudaStreamSynchronize(stream);
    for (void* p : choiceAllocs) cudaFree(p);
    choiceAllocs.clear();
    choiceExits = 0;
    choiceK = 0;
    dExitFields = nullptr; dChoiceExit = nullptr; dChoiceDist = nullptr; dChoiceInvCap = nullptr; dAssign = nullptr;
    dPending = nullptr; dChoiceHist = nullptr; dChoiceThr = nullptr; dChoiceQueue = nullptr; dChoiceAhead = nullptr;
    dChoiceCounters = nullptr;
}

std::vector<std::pair<void*, size_t>> SwarmSim::choiceLive() const {
    if (!choiceExits) return {};
    return {{dAssign, size_t(capacity) * 4}, {dPending, size_t(capacity) * 8},
            {dChoiceHist, size_t(choiceExits) * swarm_gpu::CHOICE_GAIN_BINS * 4}, {dChoiceThr, size_t(swarm_gpu::CHOICE_STRIDE) * 4},
            {dChoiceQueue, size_t(2) * swarm_gpu::CHOICE_STRIDE * 4},
            {dChoiceAhead, size_t(2) * swarm_gpu::CHOICE_STRIDE * swarm_gpu::CHOICE_AHEAD_BINS * 4}, {dChoiceCounters, 16}};
}

int SwarmSim::enqueueChoice(int in) {
    ChoiceArgs C{};
    C.V = args(in).V;
    C.n = n;
    C.nExits = choiceExits;
    C.K = choiceK;
    C.step = choiceStep;
    C.evalStep = choiceStep > 0u && choiceStep % uint32_t(swarm_gpu::choiceSteps(P.dt)) == 0u;
    C.state = state[in];
    C.cExit = dChoiceExit; C.cDist = dChoiceDist; C.invCap = dChoiceInvCap;
    C.assign = dAssign; C.pending = dPending; C.hist = dChoiceHist; C.threshold = dChoiceThr; C.queue = dChoiceQueue;
    C.ahead = dChoiceAhead; C.counters = dChoiceCounters;
    const int blocks = (n + 255) / 256;
    swarm_gpu::k_choice_prefix<<<choiceExits, 256, 0, stream>>>(C);
    if (C.evalStep) {
        swarm_gpu::k_choice_eval<<<blocks, 256, 0, stream>>>(C);
        swarm_gpu::k_choice_thr<<<1, swarm_gpu::CHOICE_STRIDE, 0, stream>>>(C);
    }
    swarm_gpu::k_choice_apply<<<blocks, 256, 0, stream>>>(C);
    ++choiceStep;
    launches += C.evalStep ? 4 : 2;
    return cudaGetLastError() == cudaSuccess ? SWARM_OK : fail(SWARM_E_CUDA, "exit choice launch");
}

extern "C" int swarm_set_exit_choice(SwarmHandle h, const SwarmExitChoiceSpec* c) {
    if (!h) return SWARM_E_INVALID;
    h->dropGraphs();
    h->freeChoice();
    if (!c) return SWARM_OK;
    if (h->instances) return h->fail(SWARM_E_INVALID, "the exit choice runs on one venue (not a batch)");
    if (!validChoice(&h->V, c)) return h->fail(SWARM_E_INVALID, "exit choice: a grid venue, 1..63 exits, 1..24 candidates, fields and types");
    if (!c->width_m) return h->fail(SWARM_E_INVALID, "exit choice: clear widths");
    for (int e = 0; e < c->n_exits; ++e)
        if (!(c->width_m[e] > 0.0f) || c->type[e] > 1) return h->fail(SWARM_E_INVALID, "exit choice: widths > 0, types 0 or 1");
    const int E = c->n_exits, K = c->candidates;
    const size_t m = size_t(h->V.nav_nx) * size_t(h->V.nav_ny), cells = size_t(h->ncells), N = size_t(h->capacity);
    std::vector<uint8_t> ex(cells * size_t(K));
    std::vector<float> di(cells * size_t(K)), invCap(static_cast<size_t>(E));
    if (const int rc = swarm_exit_choice_table(&h->V, c, ex.data(), di.data()); rc != SWARM_OK) return h->fail(rc, "exit choice table");
    for (int e = 0; e < E; ++e) invCap[size_t(e)] = float(60.0 / (double(c->width_m[e]) * swarm_gpu::CHOICE_J));
    auto alloc = [&](auto** p, size_t bytes) {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(bytes, 16)) != cudaSuccess) return false;
        h->choiceAllocs.push_back(q);
        *p = static_cast<std::remove_pointer_t<decltype(p)>>(q);
        return true;
    };
    const bool ok = alloc(&h->dExitFields, size_t(E) * m * 4) && alloc(&h->dChoiceExit, ex.size()) &&
                    alloc(&h->dChoiceDist, di.size() * 4) && alloc(&h->dChoiceInvCap, size_t(E) * 4) && alloc(&h->dAssign, N * 4) &&
                    alloc(&h->dPending, N * 8) && alloc(&h->dChoiceHist, size_t(E) * swarm_gpu::CHOICE_GAIN_BINS * 4) &&
                    alloc(&h->dChoiceThr, size_t(swarm_gpu::CHOICE_STRIDE) * 4) &&
                    alloc(&h->dChoiceQueue, size_t(2) * swarm_gpu::CHOICE_STRIDE * 4) &&
                    alloc(&h->dChoiceAhead, size_t(2) * swarm_gpu::CHOICE_STRIDE * swarm_gpu::CHOICE_AHEAD_BINS * 4) &&
                    alloc(&h->dChoiceCounters, 16);
    if (!ok) { h->freeChoice(); return h->fail(SWARM_E_OOM, "exit choice buffers"); }
    const bool up = cudaMemcpy(h->dExitFields, c->fields, size_t(E) * m * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
                    cudaMemcpy(h->dChoiceExit, ex.data(), ex.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
                    cudaMemcpy(h->dChoiceDist, di.data(), di.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
                    cudaMemcpy(h->dChoiceInvCap, invCap.data(), size_t(E) * 4, cudaMemcpyHostToDevice) == cudaSuccess;
    if (!up) { h->freeChoice(); return h->fail(SWARM_E_CUDA, "exit choice upload"); }
    h->choiceExits = E;
    h->choiceK = K;
    if (!h->resetChoice()) { h->freeChoice(); return h->fail(SWARM_E_CUDA, "exit choice reset"); }
    return SWARM_OK;
}

extern "C" int swarm_get_exit_choice(SwarmHandle h, uint32_t* assigned, int n, uint32_t* counters) {
    if (!h) return SWARM_E_INVALID;
    if (!h->choiceExits) return h->fail(SWARM_E_STATE, "the exit choice is off");
    if (assigned && n != h->n) return h->fail(SWARM_E_INVALID, "assignment size mismatch");
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return h->fail(SWARM_E_CUDA, "sync");
    if (assigned && cudaMemcpy(assigned, h->dAssign, size_t(n) * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return h->fail(SWARM_E_CUDA, "download");
    if (counters && cudaMemcpy(counters, h->dChoiceCounters, 16, cudaMemcpyDeviceToHost) != cudaSuccess) return h->fail(SWARM_E_CUDA, "download");
    return SWARM_OK;
}
