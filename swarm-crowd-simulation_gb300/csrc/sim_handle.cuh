// The handle behind the C ABI of include/swarm_cuda.h (swarm_api.cu; the adjoint's entry, adjoint_api.cu).
#pragma once

#include "../../include/swarm_cuda.h"
#include "step_args.cuh"

#include <cuda_runtime.h>

#include <cstdint>
#include <utility>
#include <string>
#include <vector>

struct SwarmAdjoint;   // the adjoint's buffers (adjoint_api.cu), made on first use
void swarm_adjoint_free(SwarmAdjoint* a);

struct SwarmSim {
    SwarmParams P{};
    SwarmVenue V{};
    int device = 0;
    int capacity = 0;
    int n = 0;
    int readIdx = 0;
    bool hasState = false;
    cudaStream_t ownStream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;
    // device buffers
    float4* state[2] = {nullptr, nullptr};
    float2* aparam = nullptr;
    float2* drive = nullptr;
    bool driveOn = false;
    uint8_t* contacts = nullptr;
    uint32_t *key = nullptr, *rank = nullptr, *count = nullptr, *start = nullptr, *sidTmp = nullptr, *sid = nullptr, *skey = nullptr;
    uint2* cells = nullptr;
    uint32_t* tileSums = nullptr;
    float4 *pos0 = nullptr, *vel0 = nullptr, *proj0 = nullptr, *proj1 = nullptr, *vel1 = nullptr, *plane = nullptr;
    float2* prm = nullptr;
    uint8_t* ctc = nullptr;
    uint4* rowsA = nullptr;
    uint2* rowsB = nullptr;
    float2* goal = nullptr;
    // the fused step's contact lists (a single instance; null on a batch): CLIST_MAX slot indices per slot, entry j of
    // slot s at j x n + s, the entries per slot, and the word that sends every slot back to its rows
    uint32_t* clist = nullptr;
    uint8_t* ccount = nullptr;
    float* clistRef = nullptr;
    int* listFlag = nullptr;
    int* errFlag = nullptr;
    int* errHost = nullptr;     // pinned host word: errFlag copied in stream order (swarm_step_host reads it after one sync)
    int* errHostDev = nullptr;  // its device view: the fused launch of a host-buffer call writes the flag there itself
    bool sumsZero = false;      // the scan-tile sums are all zero (cleared, or left so by a fused launch that counted nothing)
    unsigned* barrier = nullptr;
    unsigned long long* stamps = nullptr;
    bool fused = true;          // the whole step as one persistent kernel when the grid fits on the GPU
    int barrierExtra = 0;       // the timeout test's missing block (swarm_test_barrier_timeout)
    SwarmTuning tuning{1, 0, 0, 0.0f, 0};   // the launch configuration (swarm_autotune / swarm_set_tuning)
    bool counted = false;       // the counts hold the current state's keys (a fused step's final pass counted them)
    int countedTile = 0;        // the scan tile (cells) of the tile sums that counting left
    // swarm_step_host on the fused path with pinned buffers: the caller's input and output as the device sees them
    // (the first step reads hostIn, the last step copies its result to hostOut; null outside that call)
    const float4* hostIn = nullptr;
    float4* hostOut = nullptr;
    // safety metrics (swarm_metrics_enable)
    int metricRes = 0;
    uint32_t metricStep = 0;
    SwarmMetricCounters* mCounters = nullptr;
    uint32_t* mEvac = nullptr;
    uint2* mMass = nullptr;
    uint4* mThr = nullptr;
    SwarmMetricCell* mCells = nullptr;
    float4* mBoxes = nullptr;
    std::vector<float> exitBoxesHost;
    int enqueueMetrics(int in);
    // batched instances (swarm_batch_create)
    int instances = 0;
    swarm_gpu::VenueArgs* dVenueTable = nullptr;
    uint32_t* dInstAgent = nullptr;
    uint32_t* dInstSlot = nullptr;
    std::vector<int> instStart;   // first agent of each instance, + the total
    float *dSdf = nullptr, *dWall = nullptr, *dNav = nullptr, *dFloor = nullptr, *dSpeed = nullptr;
    SwarmSeatedLayout* dSeat = nullptr;  // seated venues: the layout (device copy)
    float4* dNavCells = nullptr;        //   and the navigation field's cells (null: drive table / router)
    float2* dWallFloor = nullptr;   // the wall SDF and floor heights interleaved (venues with a floor grid)
    uint8_t* dMask = nullptr;
    float speedMax = 1.0f;      // the largest of 1 and the venue's speed factors
    int ncells = 0;
    // execution
    bool useGraph = false;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};        // a whole step, per state half read
    cudaGraphExec_t stageGraph[2][4] = {};                  // its four stages (timing on)
    cudaGraphExec_t fusedGraph[2] = {nullptr, nullptr};     // one fused step from counted keys, per state half read
    bool timing = false;
    cudaEvent_t ev[6] = {};
    SwarmStageTimes times{};
    bool timesValid = false;
    int64_t launches = 0;
    std::vector<void*> allocs;
    SwarmAdjoint* adjoint = nullptr;
    // queue-aware exit choice (swarm_set_exit_choice, choice.cu): off while choiceExits == 0
    int choiceExits = 0, choiceK = 0;
    uint32_t choiceStep = 0;                // steps since the choice restarted (state upload or set)
    float* dExitFields = nullptr;           // choiceExits x nav nodes
    uint8_t* dChoiceExit = nullptr;         // ncells x choiceK candidate exits
    float* dChoiceDist = nullptr;           // ncells x choiceK candidate distances
    float* dChoiceInvCap = nullptr;         // per exit: seconds per queued agent
    uint32_t* dAssign = nullptr;            // per agent
    uint2* dPending = nullptr;              // per agent
    uint32_t *dChoiceHist = nullptr, *dChoiceThr = nullptr, *dChoiceQueue = nullptr, *dChoiceAhead = nullptr,
             *dChoiceCounters = nullptr;
    // a seated venue's own table (swarm_set_seated_choice): index words, entries, the estimate's terms, the steps
    // between evaluations (0: from dt, the grid venues' 3 s)
    uint32_t* dChIndex = nullptr;
    uint32_t* dChEntries = nullptr;
    int32_t* dChCell = nullptr;             // per agent: its choice cell this step
    float chSPerUnit = 0.0f, chQuantum = 0.0f;
    int32_t choiceEvery = 0;
    std::vector<void*> choiceAllocs;
    bool resetChoice();                     // no exit assigned, counts clear, step 0
    void freeChoice();                      // off, buffers freed
    int enqueueChoice(int in);              // the choice pass on state half `in`, before that step
    std::vector<std::pair<void*, size_t>> choiceLive() const;   // what a step changes (the evacuation runner's rollback)
    int64_t adjTapeBudget = int64_t(1) << 30;   // device bytes the adjoint may spend on kept segment tapes

    swarm_gpu::StepArgs args(int in) const;
    int fail(int code, const std::string& msg) { err = msg; return code; }
    void dropContactLists() {
        for (void* q : {static_cast<void*>(clist), static_cast<void*>(ccount), static_cast<void*>(clistRef),
                        static_cast<void*>(listFlag)}) {
            for (auto it = allocs.begin(); it != allocs.end(); ++it)
                if (*it == q) { cudaFree(q); allocs.erase(it); break; }
        }
        clist = nullptr;
        ccount = nullptr;
        clistRef = nullptr;
        listFlag = nullptr;
    }
    // The per-phase path hashes from zeroed counts: drop what a fused final pass counted ahead (and its scan-tile sums)
    bool clearCounts() {
        counted = false;
        sumsZero = cudaMemsetAsync(count, 0, (size_t(ncells) + 1) * 4, stream) == cudaSuccess &&
                   cudaMemsetAsync(tileSums, 0, (size_t(ncells) / 1024 + 2) * 4, stream) == cudaSuccess;
        return sumsZero;
    }
    void dropGraphs() {
        for (auto& g : graph) if (g) { cudaGraphExecDestroy(g); g = nullptr; }
        for (auto& row : stageGraph) for (auto& g : row) if (g) { cudaGraphExecDestroy(g); g = nullptr; }
        for (auto& g : fusedGraph) if (g) { cudaGraphExecDestroy(g); g = nullptr; }
    }
    // A set device error flag: clear it and the barrier words and counts a wait that gave up left behind, and report
    int deviceError(int flag);
    // The end of a host-buffer call: the error flag copied into errHost behind the step's work, one stream sync, then
    // the flag read from host memory (no second, blocking copy)
    int finishWithFlag() {
        if (cudaMemcpyAsync(errHost, errFlag, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
            cudaStreamSynchronize(stream) != cudaSuccess)
            return fail(SWARM_E_CUDA, "step sync");
        return *errHost ? deviceError(*errHost) : SWARM_OK;
    }
    // The same after a fused launch that mirrors the flag into errHost itself (set to ERR_PENDING before it): one
    // stream sync; a launch that ended early left the mirror pending, and the flag is then read from the device
    int finishWithMirror() {
        if (cudaStreamSynchronize(stream) != cudaSuccess) return fail(SWARM_E_CUDA, "step sync");
        int flag = *static_cast<volatile int*>(errHost);
        if (flag == swarm_gpu::ERR_PENDING && cudaMemcpy(&flag, errFlag, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
            return fail(SWARM_E_CUDA, "error flag");
        return flag ? deviceError(flag) : SWARM_OK;
    }
    int enqueueStages(int in, int s0, int s1);
    int captureStages(int in, int s0, int s1, cudaGraphExec_t* out);
    ~SwarmSim();
};

