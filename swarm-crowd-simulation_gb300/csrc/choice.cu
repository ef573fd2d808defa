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

namespace swarm_gpu {

// One block per exit; block 0 also clears the write parity's exit counts
__global__ void __launch_bounds__(CHOICE_PREFIX_THREADS) k_choice_prefix(ChoiceArgs C, VenueArgs) {
    choicePrefixBlock(C, blockIdx.x);
    if (blockIdx.x == 0 && threadIdx.x < CHOICE_STRIDE) C.queue[(1u - (C.step & 1u)) * CHOICE_STRIDE + threadIdx.x] = 0u;
}

__global__ void __launch_bounds__(256) k_choice_eval(ChoiceArgs C, VenueArgs V) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < C.n) choiceEvalAgent(V, C, i);
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
    choiceAheadFlush(C, i < C.n ? choiceApplyAgent(V, C, i, sQueue) : 0xFFFFFFFFu);
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
    C.evalStep = s.choiceStep > 0u && s.choiceStep % uint32_t(swarm_gpu::choiceSteps(s.P.dt)) == 0u;
    C.state = s.state[in];
    C.cExit = s.dChoiceExit; C.cDist = s.dChoiceDist; C.invCap = s.dChoiceInvCap;
    C.assign = s.dAssign; C.pending = s.dPending; C.hist = s.dChoiceHist; C.threshold = s.dChoiceThr;
    C.queue = s.dChoiceQueue; C.ahead = s.dChoiceAhead; C.counters = s.dChoiceCounters;
    return C;
}

}  // namespace

int SwarmSim::enqueueChoice(int in) {
    const ChoiceArgs C = choiceArgsOf(*this, in);
    const swarm_gpu::VenueArgs V = args(in).V;
    const int blocks = (n + 255) / 256;
    swarm_gpu::k_choice_prefix<<<choiceExits, swarm_gpu::CHOICE_PREFIX_THREADS, 0, stream>>>(C, V);
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
