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

#include "choice.cuh"
#include "sim_handle.cuh"
#include "step_kernels.cuh"
#include "venue_seated.cuh"

namespace swarm_gpu {

// ---- the seated venues: the reference's own table (nav::evaluate :605-623 and nav::apply :641-656 on its
// GpuNavChoiceCell; navEstimate :580-584 with the table's quantised distances) ----

// An agent's candidates: its choice cell's 36 words (null: a cell without candidates, every slot empty)
struct SeatedCands {
    const uint32_t* w;
    __device__ __forceinline__ uint32_t exit(int k) const { return w ? (__ldg(w + k) >> 25) & 63u : CHOICE_SLOT_EMPTY; }
    __device__ __forceinline__ uint32_t q(int k) const {   // distance quanta (nav::slotDistQ)
        return w ? (__ldg(w + 24 + (k >> 1)) >> ((k & 1) * 16)) & 0xFFFFu : 0xFFFFu;
    }
    __device__ __forceinline__ int slotOf(uint32_t e) const {   // the last slot holding e (:586-591)
        int k = -1;
        for (int i = 0; i < 24; ++i)
            if (exit(i) == e) k = i;
        return k;
    }
};

__device__ __forceinline__ SeatedChoice seatedChoice(const VenueArgs& V, const ChoiceArgs& C) {
    return SeatedChoice{SeatedNav{SeatedGeom{V.seatDev}, StepUpConst{C.suSample, C.suTol, C.suMax}, 0.0f, 0.0f, 0.0f,
                                  nullptr, V.navRes, V.navOrigin, V.navCell, V.navInv},
                        C.chIndex, C.chEntries};
}

// The agent's start position as the step's hash leaves it (a NaN position: (0, 0, 0, 1)): the reference's choice pass
// runs after the hash
__device__ __forceinline__ float4 choicePos(const ChoiceArgs& C, int i) {
    const float4 p = C.state[2 * size_t(i)];
    return isnan(p.x) ? make_float4(0.0f, 0.0f, 0.0f, 1.0f) : p;
}

// Each agent's choice cell (choiceCell, src/exit_choice.cpp:512-548) into chCell, by 8 lanes an agent (the surface
// rule's step-up scans shared out): the stages and the step's e_goal read it instead of each finding it again
constexpr int CHOICE_CELL_LANES = 8;
__global__ void __launch_bounds__(256) k_choice_cell(ChoiceArgs C, VenueArgs V) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / CHOICE_CELL_LANES, sub = t % CHOICE_CELL_LANES;
    const float4 p = i < C.n ? choicePos(C, i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const bool act = i < C.n && p.w != 0.0f;
    const int cell = choiceCellLanes(seatedChoice(V, C), f2{p.x, p.y}, act, CHOICE_CELL_LANES, sub);
    if (i < C.n && sub == 0) C.chCell[i] = act ? cell : -1;
}

__device__ __forceinline__ SeatedCands seatedCands(const VenueArgs& V, const ChoiceArgs& C, int i) {
    return SeatedCands{seatedChoice(V, C).entry(C.chCell[i])};
}

// slotDist (exit_choice.hpp:172-175): q x quantum, exact in float (an empty slot: +infinity, never read here)
__device__ __forceinline__ float seatedDist(const ChoiceArgs& C, uint32_t q) {
    return q == 0xFFFFu ? __int_as_float(0x7f800000) : float(q) * C.quantum;
}
__device__ __forceinline__ uint32_t seatedBin(uint32_t q) { return min(q >> 6, uint32_t(CHOICE_AHEAD_BINS - 1)); }
__device__ __forceinline__ float seatedEstimate(const ChoiceArgs& C, uint32_t q, uint32_t e, uint32_t queued) {
    const float walk = seatedDist(C, q) * C.sPerUnit;
    const float wait = float(queued) * C.invCap[e];
    return walk + wait;
}

// navBest (:593-603): the first candidate of least E on the queues ahead
__device__ __forceinline__ int seatedBest(const ChoiceArgs& C, const SeatedCands& c, const uint32_t* aRead, float& eBest) {
    int best = -1;
    eBest = 0.0f;
    for (int k = 0; k < 24; ++k) {
        const uint32_t ex = c.exit(k);
        if (ex == CHOICE_SLOT_EMPTY) break;
        const uint32_t q = c.q(k);
        const float e = seatedEstimate(C, q, ex, aRead[size_t(ex) * CHOICE_AHEAD_BINS + seatedBin(q)]);
        if (best < 0 || e < eBest) { best = k; eBest = e; }
    }
    return best;
}

// nav::evaluate for agent i (from its start-of-step position; an evacuated agent: none)
__device__ __forceinline__ void seatedEvalAgent(const VenueArgs& V, const ChoiceArgs& C, int i) {
    C.pending[i] = make_uint2(SWARM_CHOICE_NONE, 0u);
    if (choicePos(C, i).w == 0.0f) return;
    const SeatedCands c = seatedCands(V, C, i);
    if (c.exit(0) == CHOICE_SLOT_EMPTY) return;
    const uint32_t cur = C.assign[i];
    const int curK = c.slotOf(cur);
    if (curK < 0) return;
    atomicAdd(C.counters + 0, 1u);
    const uint32_t* aRead = C.ahead + size_t(C.step & 1u) * CHOICE_STRIDE * CHOICE_AHEAD_BINS;
    float eBest;
    const int best = seatedBest(C, c, aRead, eBest);
    const uint32_t qc = c.q(curK);
    const float eCur = seatedEstimate(C, qc, cur, aRead[size_t(cur) * CHOICE_AHEAD_BINS + seatedBin(qc)]);
    const float gain = eCur - eBest;
    if (best != curK && gain > fmaxf(CHOICE_REL_MARGIN * eCur, CHOICE_ABS_MARGIN_S)) {
        const uint32_t bin = min(uint32_t(gain), uint32_t(CHOICE_GAIN_BINS - 1));
        C.pending[i] = make_uint2(c.exit(best), bin);
        atomicAdd(C.hist + size_t(cur) * CHOICE_GAIN_BINS + bin, 1u);
        atomicAdd(C.counters + 1, 1u);
    }
}

// nav::apply for agent i, then its counts (choiceStep :743-760): its exit's queue (the block's shared counts), and the
// key of its queue-ahead count at its own distance to that exit (all ones: none)
__device__ __forceinline__ uint32_t seatedApplyAgent(const VenueArgs& V, const ChoiceArgs& C, int i, uint32_t* sQueue) {
    if (choicePos(C, i).w == 0.0f) return 0xFFFFFFFFu;
    const SeatedCands c = seatedCands(V, C, i);
    const uint32_t* aRead = C.ahead + size_t(C.step & 1u) * CHOICE_STRIDE * CHOICE_AHEAD_BINS;
    const uint32_t cur = C.assign[i];
    uint32_t ex = cur;
    const bool hasPath = c.exit(0) != CHOICE_SLOT_EMPTY;
    const int curK = hasPath ? c.slotOf(cur) : -1;
    if (hasPath && curK < 0) {   // forced (or the first choice)
        float eBest;
        ex = c.exit(seatedBest(C, c, aRead, eBest));
        if (cur != SWARM_CHOICE_NONE) atomicAdd(C.counters + 3, 1u);
    } else if (C.evalStep && curK >= 0) {
        const uint2 pd = C.pending[i];
        if (pd.x != SWARM_CHOICE_NONE && pd.y >= C.threshold[cur]) {
            ex = pd.x;
            atomicAdd(C.counters + 2, 1u);
        }
    }
    C.assign[i] = ex;
    if (ex == SWARM_CHOICE_NONE) return 0xFFFFFFFFu;
    atomicAdd(sQueue + ex, 1u);
    const int k = c.slotOf(ex);
    return k >= 0 ? ex * uint32_t(CHOICE_AHEAD_BINS) + seatedBin(c.q(k)) : 0xFFFFFFFFu;
}

// One block per exit; block 0 also clears the write parity's exit counts
__global__ void __launch_bounds__(CHOICE_PREFIX_THREADS) k_choice_prefix(ChoiceArgs C, VenueArgs) {
    choicePrefixBlock(C, blockIdx.x);
    if (blockIdx.x == 0 && threadIdx.x < CHOICE_STRIDE) C.queue[(1u - (C.step & 1u)) * CHOICE_STRIDE + threadIdx.x] = 0u;
}

__global__ void __launch_bounds__(256) k_choice_eval(ChoiceArgs C, VenueArgs V) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C.n) return;
    if (C.chIndex) seatedEvalAgent(V, C, i);
    else choiceEvalAgent(V, C, i);
}

// One warp per exit (grid: nExits x 32)
__global__ void __launch_bounds__(32) k_choice_thr(ChoiceArgs C, VenueArgs) { choiceThrWarp(C, blockIdx.x); }

// The exit counts aggregated per block in shared memory, the queue-ahead bins per warp: the same integers, a few
// atomics per block instead of one per agent on ~40 addresses
__global__ void __launch_bounds__(256) k_choice_apply(ChoiceArgs C, VenueArgs V) {
    __shared__ uint32_t sQueue[CHOICE_STRIDE];
    if (threadIdx.x < CHOICE_STRIDE) sQueue[threadIdx.x] = 0u;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t key = i >= C.n ? 0xFFFFFFFFu : C.chIndex ? seatedApplyAgent(V, C, i, sQueue) : choiceApplyAgent(V, C, i, sQueue);
    choiceAheadFlush(C, key);
    __syncthreads();
    choiceQueueFlush(C, sQueue);
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
    dChIndex = nullptr; dChEntries = nullptr; dChCell = nullptr; chSPerUnit = 0.0f; chQuantum = 0.0f; choiceEvery = 0;
}

std::vector<std::pair<void*, size_t>> SwarmSim::choiceLive() const {
    if (!choiceExits) return {};
    return {{dAssign, size_t(capacity) * 4}, {dPending, size_t(capacity) * 8},
            {dChoiceHist, size_t(choiceExits) * swarm_gpu::CHOICE_GAIN_BINS * 4}, {dChoiceThr, size_t(swarm_gpu::CHOICE_STRIDE) * 4},
            {dChoiceQueue, size_t(2) * swarm_gpu::CHOICE_STRIDE * 4},
            {dChoiceAhead, size_t(2) * swarm_gpu::CHOICE_STRIDE * swarm_gpu::CHOICE_AHEAD_BINS * 4}, {dChoiceCounters, 16}};
}

namespace {

ChoiceArgs choiceArgsOf(const SwarmSim& s, int in) {
    ChoiceArgs C{};
    C.n = s.n;
    C.nExits = s.choiceExits;
    C.K = s.choiceK;
    C.step = s.choiceStep;
    const int every = s.choiceEvery > 0 ? s.choiceEvery : swarm_gpu::choiceSteps(s.P.dt);
    C.evalStep = s.choiceStep > 0u && s.choiceStep % uint32_t(every) == 0u;   // nav::evaluationStep
    C.state = s.state[in];
    C.cExit = s.dChoiceExit; C.cDist = s.dChoiceDist; C.invCap = s.dChoiceInvCap;
    C.assign = s.dAssign; C.pending = s.dPending; C.hist = s.dChoiceHist; C.threshold = s.dChoiceThr;
    C.queue = s.dChoiceQueue; C.ahead = s.dChoiceAhead; C.counters = s.dChoiceCounters;
    C.chIndex = s.dChIndex; C.chEntries = s.dChEntries; C.chCell = s.dChCell; C.sPerUnit = s.chSPerUnit; C.quantum = s.chQuantum;
    C.suSample = s.P.step_up_sample; C.suTol = s.P.step_up_tol; C.suMax = s.P.step_up_max_samples;
    return C;
}

}  // namespace

int SwarmSim::enqueueChoice(int in) {
    const ChoiceArgs C = choiceArgsOf(*this, in);
    const swarm_gpu::VenueArgs V = args(in).V;
    const int blocks = (n + 255) / 256;
    swarm_gpu::k_choice_prefix<<<choiceExits, swarm_gpu::CHOICE_PREFIX_THREADS, 0, stream>>>(C, V);
    if (C.chIndex) {
        const long long lanes = static_cast<long long>(n) * swarm_gpu::CHOICE_CELL_LANES;
        swarm_gpu::k_choice_cell<<<unsigned((lanes + 255) / 256), 256, 0, stream>>>(C, V);
        ++launches;
    }
    if (C.evalStep) {
        swarm_gpu::k_choice_eval<<<blocks, 256, 0, stream>>>(C, V);
        swarm_gpu::k_choice_thr<<<choiceExits, 32, 0, stream>>>(C, V);
    }
    swarm_gpu::k_choice_apply<<<blocks, 256, 0, stream>>>(C, V);
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

extern "C" int swarm_set_seated_choice(SwarmHandle h, const SwarmSeatedChoiceSpec* c) {
    if (!h) return SWARM_E_INVALID;
    h->dropGraphs();
    h->freeChoice();
    if (!c) return SWARM_OK;
    if (h->instances) return h->fail(SWARM_E_INVALID, "the exit choice runs on one venue (not a batch)");
    if (h->V.kind != SWARM_VENUE_SEATED || !h->dNavCells || h->V.nav_res <= 0)
        return h->fail(SWARM_E_INVALID, "seated exit choice: a seated venue with its navigation field");
    if (c->grid_res != h->V.nav_res) return h->fail(SWARM_E_INVALID, "seated exit choice: the table's grid is the navigation grid");
    const int E = c->n_exits;
    if (E < 1 || E > SWARM_CHOICE_MAX_EXITS || c->n_entries < 0 || !c->index || (c->n_entries > 0 && !c->entries) || !c->inv_cap_s ||
        !(c->seconds_per_unit > 0.0f) || !(c->dist_quantum > 0.0f) || c->choice_steps < 1)
        return h->fail(SWARM_E_INVALID, "seated exit choice: 1..63 exits, index, entries, capacities, quantum and steps");
    const size_t cells = size_t(c->grid_res) * size_t(c->grid_res), ne = size_t(c->n_entries);
    for (size_t i = 0; i < cells; ++i)
        if ((c->index[i] & SWARM_CHOICE_INDEX_MASK) > ne) return h->fail(SWARM_E_INVALID, "seated exit choice: an index word beyond the entries");
    for (size_t e = 0; e < ne; ++e)
        for (int k = 0; k < 24; ++k) {
            const uint32_t w = c->entries[e].slot[k], ex = (w >> 25) & 63u;
            if (ex == swarm_gpu::CHOICE_SLOT_EMPTY) continue;
            if (ex >= uint32_t(E) || size_t(w & ((1u << 25) - 1u)) >= cells)
                return h->fail(SWARM_E_INVALID, "seated exit choice: a slot's exit or anchor outside the table");
        }
    const size_t N = size_t(h->capacity);
    auto alloc = [&](auto** p, size_t bytes) {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(bytes, 16)) != cudaSuccess) return false;
        h->choiceAllocs.push_back(q);
        *p = static_cast<std::remove_pointer_t<decltype(p)>>(q);
        return true;
    };
    const bool ok = alloc(&h->dChIndex, cells * 4) && alloc(&h->dChEntries, ne * sizeof(SwarmNavChoiceCell)) &&
                    alloc(&h->dChCell, N * 4) &&
                    alloc(&h->dChoiceInvCap, size_t(E) * 4) && alloc(&h->dAssign, N * 4) && alloc(&h->dPending, N * 8) &&
                    alloc(&h->dChoiceHist, size_t(E) * swarm_gpu::CHOICE_GAIN_BINS * 4) &&
                    alloc(&h->dChoiceThr, size_t(swarm_gpu::CHOICE_STRIDE) * 4) &&
                    alloc(&h->dChoiceQueue, size_t(2) * swarm_gpu::CHOICE_STRIDE * 4) &&
                    alloc(&h->dChoiceAhead, size_t(2) * swarm_gpu::CHOICE_STRIDE * swarm_gpu::CHOICE_AHEAD_BINS * 4) &&
                    alloc(&h->dChoiceCounters, 16);
    if (!ok) { h->freeChoice(); return h->fail(SWARM_E_OOM, "seated exit choice buffers"); }
    const bool up = cudaMemcpy(h->dChIndex, c->index, cells * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
                    (ne == 0 || cudaMemcpy(h->dChEntries, c->entries, ne * sizeof(SwarmNavChoiceCell), cudaMemcpyHostToDevice) == cudaSuccess) &&
                    cudaMemcpy(h->dChoiceInvCap, c->inv_cap_s, size_t(E) * 4, cudaMemcpyHostToDevice) == cudaSuccess;
    if (!up) { h->freeChoice(); return h->fail(SWARM_E_CUDA, "seated exit choice upload"); }
    h->choiceExits = E;
    h->choiceK = 24;
    h->chSPerUnit = c->seconds_per_unit;
    h->chQuantum = c->dist_quantum;
    h->choiceEvery = c->choice_steps;
    if (!h->resetChoice()) { h->freeChoice(); return h->fail(SWARM_E_CUDA, "exit choice reset"); }
    return SWARM_OK;
}
