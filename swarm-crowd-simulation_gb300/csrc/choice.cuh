// The queue-aware exit choice's stages as device functions (DedovSergei/swarm-crowd-simulation src/exit_choice.cpp:
// nav::evaluate :605-623, nav::switchThreshold :625-640, nav::apply :642-658, the prefix stage of nav::choiceStep
// :686-700; constants include/swarm/sim_params.hpp:412-427), run by choice.cu's stage kernels; every count is an
// integer sum, so any schedule of the agents gives the same integers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/swarm_cuda.h"
#include "device_math.cuh"
#include "step_args.cuh"

namespace swarm_gpu {

// The stages' arguments: the candidate table, the per-exit seconds per queued agent, each agent's assignment and
// pending switch, the per-exit histograms and counts (two parities)
struct ChoiceArgs {
    int32_t n, nExits, K;
    uint32_t step;
    int32_t evalStep;
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
    // a seated venue's own table (chIndex non-null: swarm_set_seated_choice; cExit / cDist unused): index words and
    // entries on the navigation grid, the estimate's seconds per model unit, the distance quantum, and the step-up
    // constants of the choice cell's surface rule
    const uint32_t* chIndex;
    const uint32_t* chEntries;
    int32_t* chCell;              // per agent: its choice cell this step (k_choice_cell)
    float sPerUnit, quantum;
    float suSample, suTol;
    int32_t suMax;
};

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

inline int choiceSteps(float dt) {
    const int k = int(double(CHOICE_T_S) / double(dt) + 0.5);
    return k > 1 ? k : 1;
}

__device__ __forceinline__ uint32_t aheadBin(float d) {
    return min(uint32_t(d * 2.0f), uint32_t(CHOICE_AHEAD_BINS - 1));
}

__device__ __forceinline__ float choiceEstimate(const ChoiceArgs& C, float d, uint32_t e, uint32_t queued) {
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
        const float e = choiceEstimate(C, d, ex, aRead[size_t(ex) * CHOICE_AHEAD_BINS + aheadBin(d)]);
        if (best < 0 || e < eBest) { best = k; eBest = e; }
    }
    return best;
}

// The agent's cell row of the table (the step's hash of its start-of-step position, NaN sanitised as the hash
// does), or -1 when it is evacuated
__device__ __forceinline__ long long choiceRow(const VenueArgs& V, const ChoiceArgs& C, int i) {
    float4 p = C.state[2 * size_t(i)];
    if (isnan(p.x)) p = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    if (p.w == 0.0f) return -1;
    const int x = sclamp(int((p.x - V.dminX) / V.dspanX * float(V.resX)), 0, V.resX - 1);
    const int y = sclamp(int((p.y - V.dminY) / V.dspanY * float(V.resY)), 0, V.resY - 1);
    return (long long)(x + y * V.resX) * C.K;
}

// The prefix stage for exit e, by a block of CHOICE_PREFIX_THREADS threads (4 bins each, one round trip): the read
// parity's queue-ahead histogram to exclusive prefix sums in place, the write parity's cleared
constexpr int CHOICE_PREFIX_THREADS = 256;
__device__ __forceinline__ void choicePrefixBlock(const ChoiceArgs& C, int e) {
    __shared__ uint32_t warpTot[CHOICE_PREFIX_THREADS / 32];
    const uint32_t par = C.step & 1u;
    uint32_t* aRead = C.ahead + (size_t(par) * CHOICE_STRIDE + size_t(e)) * CHOICE_AHEAD_BINS;
    uint32_t* aWrite = C.ahead + (size_t(1u - par) * CHOICE_STRIDE + size_t(e)) * CHOICE_AHEAD_BINS;
    constexpr int PER = CHOICE_AHEAD_BINS / CHOICE_PREFIX_THREADS;
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
}

// nav::evaluate for agent i
__device__ __forceinline__ void choiceEvalAgent(const VenueArgs& V, const ChoiceArgs& C, int i) {
    C.pending[i] = make_uint2(SWARM_CHOICE_NONE, 0u);
    const long long r = choiceRow(V, C, i);
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
    const float eCur = choiceEstimate(C, dCur, cur, aRead[size_t(cur) * CHOICE_AHEAD_BINS + aheadBin(dCur)]);
    const float gain = eCur - eBest;
    if (best != curK && gain > fmaxf(CHOICE_REL_MARGIN * eCur, CHOICE_ABS_MARGIN_S)) {
        const uint32_t bin = min(uint32_t(gain), uint32_t(CHOICE_GAIN_BINS - 1));
        C.pending[i] = make_uint2(uint32_t(C.cExit[row + size_t(best)]), bin);
        atomicAdd(C.hist + size_t(cur) * CHOICE_GAIN_BINS + bin, 1u);
        atomicAdd(C.counters + 1, 1u);
    }
}

// nav::switchThreshold for exit e, by one whole warp, then the exit's histogram cleared. The sequential rule (from the
// top bin down, accept bins while the accepted count stays within the cap; a top bin alone above the cap is taken
// anyway) is the lowest nonzero bin whose count with everything above it fits the cap, else the highest nonzero bin:
// suffix sums over the warp's 8 bins a lane.
__device__ __forceinline__ void choiceThrWarp(const ChoiceArgs& C, int e) {
    const unsigned lane = threadIdx.x & 31u;
    uint32_t* h = C.hist + size_t(e) * CHOICE_GAIN_BINS;
    const uint32_t queued = C.queue[(C.step & 1u) * CHOICE_STRIDE + uint32_t(e)];
    const uint32_t cap = max(CHOICE_MIN_SWITCHES, uint32_t(float(queued) * CHOICE_SWITCH_SHARE));
    constexpr int PER = CHOICE_GAIN_BINS / 32;
    uint32_t v[PER], suffix[PER];
#pragma unroll
    for (int j = 0; j < PER; ++j) v[j] = h[lane * PER + j];
    uint32_t run = 0;
#pragma unroll
    for (int j = PER - 1; j >= 0; --j) { run += v[j]; suffix[j] = run; }
    uint32_t above = run;   // this lane's bins and every higher lane's
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_down_sync(0xffffffffu, above, o);
        if (lane + unsigned(o) < 32u) above += u;
    }
    const uint32_t higher = above - run;
    uint32_t lowAccepted = 0xFFFFFFFFu, highNonzero = 0u;
    bool any = false;
#pragma unroll
    for (int j = 0; j < PER; ++j) {
        if (v[j] == 0u) continue;
        const uint32_t b = lane * PER + uint32_t(j);
        if (higher + suffix[j] <= cap) lowAccepted = min(lowAccepted, b);
        highNonzero = max(highNonzero, b);
        any = true;
    }
    lowAccepted = __reduce_min_sync(0xffffffffu, lowAccepted);
    highNonzero = __reduce_max_sync(0xffffffffu, any ? highNonzero + 1u : 0u);   // + 1: 0 means none
    if (lane == 0)
        C.threshold[e] = lowAccepted != 0xFFFFFFFFu ? lowAccepted : (highNonzero ? highNonzero - 1u : uint32_t(CHOICE_GAIN_BINS));
#pragma unroll
    for (int j = 0; j < PER; ++j) h[lane * PER + j] = 0u;
}

// nav::apply for agent i: its new assignment, its exit count added to the block's shared counts (sQueue), and the
// key of its queue-ahead count (exit x CHOICE_AHEAD_BINS + bin; all ones: none) for choiceAheadFlush
__device__ __forceinline__ uint32_t choiceApplyAgent(const VenueArgs& V, const ChoiceArgs& C, int i, uint32_t* sQueue) {
    const long long r = choiceRow(V, C, i);
    if (r < 0) return 0xFFFFFFFFu;
    const size_t row = size_t(r);
    const uint32_t* aRead = C.ahead + size_t(C.step & 1u) * CHOICE_STRIDE * CHOICE_AHEAD_BINS;
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
    if (ex == SWARM_CHOICE_NONE) return 0xFFFFFFFFu;
    atomicAdd(sQueue + ex, 1u);
    const int k = slotOf(C, row, ex);
    return k >= 0 ? ex * uint32_t(CHOICE_AHEAD_BINS) + aheadBin(C.cDist[row + size_t(k)]) : 0xFFFFFFFFu;
}

// The warp's queue-ahead counts: one atomic per distinct (exit, bin) (every lane of the warp calls it)
__device__ __forceinline__ void choiceAheadFlush(const ChoiceArgs& C, uint32_t key) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned valid = __ballot_sync(0xffffffffu, key != 0xFFFFFFFFu);
    if (key == 0xFFFFFFFFu) return;
    const unsigned peers = __match_any_sync(valid, key);
    if (int(lane) == __ffs(peers) - 1)
        atomicAdd(C.ahead + size_t(1u - (C.step & 1u)) * CHOICE_STRIDE * CHOICE_AHEAD_BINS + key, uint32_t(__popc(peers)));
}

// The block's exit counts into the write parity (after a block barrier)
__device__ __forceinline__ void choiceQueueFlush(const ChoiceArgs& C, const uint32_t* sQueue) {
    if (threadIdx.x < CHOICE_STRIDE && sQueue[threadIdx.x])
        atomicAdd(C.queue + (1u - (C.step & 1u)) * CHOICE_STRIDE + threadIdx.x, sQueue[threadIdx.x]);
}

}  // namespace swarm_gpu
