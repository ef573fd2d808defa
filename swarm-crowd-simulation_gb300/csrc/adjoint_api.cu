// swarm_adjoint_run (include/swarm_cuda.h): the loss and its gradient by the adjoint of the step.
//
// Schedule, for T steps with checkpoints every C: a forward pass stores the state at the start of each of the S
// segments and tapes the last segment as it goes; then, for each segment from the last to the first, the segment is
// recomputed from its checkpoint with the tape on (all but the last) and its steps are reversed from the last to the
// first. Forward work 2T - C steps (T - C of them untaped), reverse work T steps, device memory C taped steps + S
// checkpoints. With a fused handle each forward step and each reverse step is one persistent cooperative launch. The handle's own state and buffers are not touched: the adjoint owns copies of
// every buffer a step writes.
#include "adjoint.cuh"
#include "sim_handle.cuh"
#include "step_kernels.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

using swarm_gpu::AdjArgs;
using swarm_gpu::StepArgs;
using swarm_gpu::TapeLayout;

// Words between consecutive steps' run starts on the tape: ncells + 1, rounded up to 4 so that each step's array
// starts 16-byte aligned (the scan writes it with 16-byte stores)
inline size_t startStride(int ncells) { return (size_t(ncells) + 1 + 3) / 4 * 4; }

struct SwarmAdjoint {
    int n = 0, K = 0, ckpt = 0, nseg = 0, steps = 0, ncells = 0;
    int keep = 1;                    // segments whose tapes the checkpoint pass keeps (the last ones): not recomputed
    double speedMax = 1.0;           // the venue's largest speed factor
    TapeLayout L{};
    std::vector<void*> allocs;
    int64_t bytes = 0;
    // forward
    float4* state[2] = {nullptr, nullptr};
    float4* ckptState = nullptr;     // nseg x 2n
    float4* tapeF4 = nullptr;        // keep x ckpt x L.f4PerStep() (the tape arrays hold keep x ckpt steps)
    float2* tapePrm = nullptr;       // ckpt x n
    uint32_t* tapeSid = nullptr;     // ckpt x n
    uint32_t* tapeSkey = nullptr;    // ckpt x n
    uint32_t* tapeStart = nullptr;   // ckpt x startStride (ncells + 1 run starts, padded to 16 bytes)
    uint8_t* tapeCtc = nullptr;      // ckpt x n
    uint32_t *key = nullptr, *rank = nullptr, *count = nullptr, *sidTmp = nullptr, *tileSums = nullptr;
    uint2* cells = nullptr;
    uint8_t* contacts = nullptr;
    int* err = nullptr;
    unsigned* barrier = nullptr;     // 8 words: the forward's (0 .. 3), the reverse's (4 .. 7)
    unsigned long long* stamps = nullptr;   // the fused reverse's phase spans
    uint4* rowsA = nullptr;
    uint2* rowsB = nullptr;
    float4* proj[2] = {nullptr, nullptr};
    // reverse
    float4* lamX[2] = {nullptr, nullptr};
    float4 *lamQ = nullptr, *lamPlane = nullptr, *lamNv = nullptr, *lamPOld = nullptr, *lamSep = nullptr, *lamP = nullptr,
           *lamV = nullptr;
    float2* lamC[2] = {nullptr, nullptr};
    float* lamR = nullptr;
    double *gR = nullptr, *gV0 = nullptr, *gTau = nullptr, *lossPart = nullptr;
    int lossBlocks = 0;

    ~SwarmAdjoint() { for (void* p : allocs) cudaFree(p); }
    template <class T>
    bool alloc(T** p, size_t count) {
        void* q = nullptr;
        const size_t b = std::max<size_t>(count, 1) * sizeof(T);
        if (cudaMalloc(&q, b) != cudaSuccess) return false;
        allocs.push_back(q);
        bytes += int64_t(b);
        *p = static_cast<T*>(q);
        return true;
    }
    size_t f4Step() const { return L.f4PerStep(); }
    float4* tape(int j) const { return tapeF4 + size_t(j) * f4Step(); }
    // the first tape slot of segment seg: a kept segment its own run of slots, a recomputed one the first run (the
    // kept segments are the last ones, reversed before any recomputed segment reuses their slots)
    int tapeBase(int seg) const { return seg >= nseg - keep ? (seg - (nseg - keep)) * ckpt : 0; }
};

void swarm_adjoint_free(SwarmAdjoint* a) { delete a; }

namespace {

bool ok(SwarmSim* h, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    h->err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

// Device bytes of one taped step: the float4 records, (r, v0), sorted ids and keys, run starts, contact bits
size_t tapeStepBytes(int n, int K, int ncells) {
    const TapeLayout L{n, K, std::max(K, 1)};
    return L.f4PerStep() * 16 + size_t(n) * (8 + 4 + 4 + 1) + startStride(ncells) * 4;
}

SwarmAdjoint* makeAdjoint(SwarmSim* h, int n, int K, int ckpt, int nseg, int steps, int keep) {
    SwarmAdjoint* a = new (std::nothrow) SwarmAdjoint();
    if (!a) return nullptr;
    a->n = n; a->K = K; a->ckpt = ckpt; a->nseg = nseg; a->steps = steps; a->ncells = h->ncells; a->keep = keep;
    a->speedMax = h->speedMax;
    a->L = TapeLayout{n, K, std::max(K, 1)};
    const size_t N = size_t(n), C = size_t(ckpt) * size_t(keep), NC = size_t(h->ncells) + 1;
    a->lossBlocks = std::max(swarm_gpu::adjFinalBlocks(n), swarm_gpu::adjFusedBlocks(n));
    const bool good =
        a->alloc(&a->state[0], 2 * N) && a->alloc(&a->state[1], 2 * N) && a->alloc(&a->ckptState, size_t(nseg) * 2 * N) &&
        a->alloc(&a->tapeF4, C * a->f4Step()) && a->alloc(&a->tapePrm, C * N) && a->alloc(&a->tapeSid, C * N) &&
        a->alloc(&a->tapeSkey, C * N) && a->alloc(&a->tapeStart, C * startStride(h->ncells)) && a->alloc(&a->tapeCtc, C * N) &&
        a->alloc(&a->key, N) && a->alloc(&a->rank, N) && a->alloc(&a->count, NC) && a->alloc(&a->sidTmp, N) &&
        a->alloc(&a->tileSums, size_t(h->ncells) / 1024 + 2) && a->alloc(&a->cells, NC) && a->alloc(&a->contacts, N) &&
        a->alloc(&a->err, 1) && a->alloc(&a->barrier, 8) && a->alloc(&a->stamps, 8) && a->alloc(&a->rowsA, N) && a->alloc(&a->rowsB, N) &&
        a->alloc(&a->proj[0], N) && a->alloc(&a->proj[1], N) &&
        a->alloc(&a->lamX[0], 2 * N) && a->alloc(&a->lamX[1], 2 * N) && a->alloc(&a->lamQ, N) && a->alloc(&a->lamPlane, N) &&
        a->alloc(&a->lamNv, N) && a->alloc(&a->lamPOld, N) && a->alloc(&a->lamSep, N) && a->alloc(&a->lamP, N) &&
        a->alloc(&a->lamV, N) && a->alloc(&a->lamC[0], N) && a->alloc(&a->lamC[1], N) && a->alloc(&a->lamR, N) &&
        a->alloc(&a->gR, N) && a->alloc(&a->gV0, N) && a->alloc(&a->gTau, N) &&
        a->alloc(&a->lossPart, size_t(steps) * size_t(a->lossBlocks));
    if (!good || cudaMemset(a->count, 0, NC * 4) != cudaSuccess || cudaMemset(a->err, 0, 4) != cudaSuccess ||
        cudaMemset(a->barrier, 0, 32) != cudaSuccess) {
        delete a;
        return nullptr;
    }
    return a;
}

// The step's arguments over the adjoint's buffers: state half `in`, tape slot j
StepArgs forwardArgs(const SwarmSim* h, const SwarmAdjoint* a, int in, int j) {
    StepArgs A = h->args(0);
    const TapeLayout& L = a->L;
    const size_t N = size_t(a->n);
    A.n = a->n;
    A.stateIn = a->state[in];
    A.stateOut = a->state[in ^ 1];
    A.drive = nullptr;
    A.contacts = a->contacts;
    A.key = a->key; A.rank = a->rank; A.count = a->count; A.cells = a->cells; A.tileSums = a->tileSums; A.sidTmp = a->sidTmp;
    A.sid = a->tapeSid + size_t(j) * N;
    A.skey = a->tapeSkey + size_t(j) * N;
    A.start = a->tapeStart + size_t(j) * startStride(a->ncells);
    float4* t = a->tape(j);
    A.pos0 = t + L.pos0();
    A.vel0 = t + L.vel0();
    A.vel1 = t + L.vel1();
    A.plane = t + L.plane();
    A.prm = a->tapePrm + size_t(j) * N;
    A.ctc = a->tapeCtc + size_t(j) * N;
    A.proj[0] = a->proj[0];
    A.proj[1] = a->proj[1];
    A.rowsA = a->rowsA; A.rowsB = a->rowsB;
    A.err = a->err;
    A.barrier = a->barrier;
    A.barrierExtra = 0;
    A.stamps = nullptr;
    A.hashed = 0;
    A.hashNext = 0;
    A.venueTable = nullptr; A.instAgent = nullptr; A.instSlot = nullptr;
    A.tapePred = A.tapeCorr = A.tapeQK = nullptr;
    return A;
}

}  // namespace

extern "C" int swarm_adjoint_set_tape_budget(SwarmHandle h, int64_t bytes) {
    if (!h || bytes < 0) return SWARM_E_INVALID;
    h->adjTapeBudget = bytes;
    return SWARM_OK;
}

extern "C" int swarm_adjoint_run(SwarmHandle h, const SwarmLossSpec* loss, int steps, int ckpt_every, double* loss_out,
                                 float* dL_dv0, float* dL_dr, float* dL_dtau, SwarmAdjointStats* stats) {
    if (!h || !loss || !loss_out || !dL_dv0 || !dL_dr || !dL_dtau) return SWARM_E_INVALID;
    if (loss->kind != SWARM_LOSS_NAV_DISTANCE) return h->fail(SWARM_E_INVALID, "unknown loss kind");
    if (h->V.kind != SWARM_VENUE_GRID || h->instances) return h->fail(SWARM_E_INVALID, "the adjoint runs on one grid venue");
    // a floor grid brings the step-up limit into the forward step, whose blocked moves have no reverse here
    if (h->dFloor) return h->fail(SWARM_E_INVALID, "the adjoint runs on flat venues (no floor grid: no step-up limit)");
    if (h->driveOn) return h->fail(SWARM_E_INVALID, "the adjoint follows e_goal: clear the drive table");
    if (h->choiceExits) return h->fail(SWARM_E_INVALID, "the adjoint follows the nearest-exit field: turn the exit choice off");
    if (!h->hasState) return h->fail(SWARM_E_STATE, "no state (upload one first)");
    if (steps < 1 || ckpt_every < 1) return h->fail(SWARM_E_INVALID, "steps and ckpt_every must be >= 1");
    const int K = h->P.proj_iterations;
    if (h->P.wall_passes < 0 || h->P.wall_passes > 5 || K > 64) return h->fail(SWARM_E_INVALID, "wall_passes <= 5 and K <= 64");
    const int n = h->n, C = std::min(ckpt_every, steps), nseg = (steps + C - 1) / C;
    // the last segment's tape always, and as many earlier segments' tapes as the tape budget holds
    const int64_t segBytes = int64_t(tapeStepBytes(n, K, h->ncells)) * C;
    const int keep = 1 + int(std::min<int64_t>(nseg - 1, h->adjTapeBudget / std::max<int64_t>(segBytes, 1)));
    SwarmAdjoint*& a = h->adjoint;
    if (!a || a->n != n || a->K != K || a->ckpt != C || a->nseg != nseg || a->steps != steps || a->ncells != h->ncells ||
        a->keep != keep) {
        delete a;
        a = makeAdjoint(h, n, K, C, nseg, steps, keep);
        if (!a) return h->fail(SWARM_E_OOM, "adjoint buffers (tape of " + std::to_string(C) + " steps)");
    }
    cudaStream_t st = h->stream;
    const size_t N = size_t(n);
    const TapeLayout& L = a->L;
    int64_t launches = 0;
    std::vector<cudaEvent_t> ev;
    if (stats) {
        ev.resize(2 + 3 * size_t(nseg));
        for (auto& e : ev) cudaEventCreate(&e);
        cudaEventRecord(ev[0], st);
    }
    bool good = ok(h, cudaMemcpyAsync(a->state[0], h->state[h->readIdx], N * 32, cudaMemcpyDeviceToDevice, st), "adjoint state") &&
                ok(h, cudaMemsetAsync(a->lamX[0], 0, N * 32, st), "adjoint clear") &&
                ok(h, cudaMemsetAsync(a->gR, 0, N * 8, st), "adjoint clear") &&
                ok(h, cudaMemsetAsync(a->gV0, 0, N * 8, st), "adjoint clear") &&
                ok(h, cudaMemsetAsync(a->gTau, 0, N * 8, st), "adjoint clear") &&
                ok(h, cudaMemsetAsync(a->err, 0, 4, st), "adjoint clear") &&
                ok(h, cudaMemsetAsync(a->lossPart, 0, size_t(steps) * size_t(a->lossBlocks) * 8, st), "adjoint clear") &&
                ok(h, cudaMemsetAsync(a->stamps, 0, 8 * 8, st), "adjoint clear");
    // the checkpoint pass; the kept segments (the last `keep`) are taped here, not recomputed
    int in = 0;
    std::vector<float4*> q(size_t(L.Kq)), corr(size_t(K) + 1, nullptr);
    // Fused steps run in chains, as the handle's stepping does: each final pass counts the next state's keys
    // (hashNext) for the next step of its chain (hashed); a chain's last step counts nothing, so the counts are clear
    // whenever a checkpoint is restored.
    bool counted = false;
    auto chain = [&](StepArgs& A, bool last) {
        // a chain's first step hashes from zero counts and zero scan-tile sums (the tile is the same along a chain:
        // the agent count, cell count and tuning do not change within the run)
        if (!counted) cudaMemsetAsync(a->tileSums, 0, (size_t(a->ncells) / 1024 + 2) * 4, st);
        A.hashed = counted ? 1 : 0;
        A.hashNext = last ? 0 : 1;
        counted = !last;
    };
    auto tapedStep = [&](int j, bool last) {
        StepArgs A = forwardArgs(h, a, in, j);
        float4* t = a->tape(j);
        if (h->fused) {   // one persistent launch writing the tape
            chain(A, last);
            A.proj[0] = t + L.q(0);
            A.tapeCorr = K > 0 ? t + L.corr(1) : nullptr;
            A.tapeQK = t + L.qK();
            A.tapePred = t + L.pred();
            launches += 1;
            return ok(h, swarm_gpu::launch_step_fused_taped(A, st), "adjoint recompute");
        }
        for (int k = 0; k < L.Kq; ++k) q[size_t(k)] = t + L.q(k);
        for (int k = 1; k <= K; ++k) corr[size_t(k)] = t + L.corr(k);
        swarm_gpu::launch_step_taped(A, q.data(), corr.data(), t + L.qK(), t + L.pred(), st, &launches);
        return ok(h, cudaGetLastError(), "adjoint recompute");
    };
    for (int seg = 0; good && seg < nseg; ++seg) {
        good = ok(h, cudaMemcpyAsync(a->ckptState + size_t(seg) * 2 * N, a->state[in], N * 32, cudaMemcpyDeviceToDevice, st), "checkpoint");
        if (seg >= nseg - a->keep) {   // a kept segment: taped now (one chain through the kept segments)
            const int cnt = std::min(C, steps - seg * C), base = a->tapeBase(seg);
            for (int j = 0; good && j < cnt; ++j) {
                good = tapedStep(base + j, seg == nseg - 1 && j == cnt - 1);
                in ^= 1;
            }
            continue;
        }
        if (h->fused) {   // the segment's C untaped steps in one persistent launch (a grid barrier between steps)
            if (!good) break;
            StepArgs A = forwardArgs(h, a, in, 0);
            chain(A, false);
            A.steps = C;
            good = ok(h, swarm_gpu::launch_step_fused(A, st), "adjoint forward");
            launches += 1;
            in ^= C & 1;
            continue;
        }
        for (int j = 0; good && j < C; ++j) {
            StepArgs A = forwardArgs(h, a, in, 0);
            {
                for (int s2 = 0; s2 < 4; ++s2) swarm_gpu::launch_stage(A, s2, st, &launches);
                good = ok(h, cudaGetLastError(), "adjoint forward");
            }
            in ^= 1;
        }
    }
    if (stats) cudaEventRecord(ev[1], st);
    // the segments, last to first: taped recompute, then the reverse steps
    const float gatherReach = float((2.0 * h->P.r_pair_max + std::max(double(h->P.sep_margin),
                                     double(h->P.v_max) * a->speedMax / double(h->P.headway_rate))) * 1.01);
    int lam = 0;
    for (int seg = nseg - 1; good && seg >= 0; --seg) {
        const int t0 = seg * C, cnt = std::min(C, steps - t0);
        if (stats) cudaEventRecord(ev[2 + 3 * size_t(seg)], st);
        if (seg < nseg - a->keep) {   // recompute the segment from its checkpoint, taped (tape slots from 0)
            good = ok(h, cudaMemcpyAsync(a->state[0], a->ckptState + size_t(seg) * 2 * N, N * 32, cudaMemcpyDeviceToDevice, st), "restore");
            in = 0;
            for (int j = 0; good && j < cnt; ++j) {
                good = tapedStep(j, j == cnt - 1);
                in ^= 1;
            }
        }
        if (stats) cudaEventRecord(ev[3 + 3 * size_t(seg)], st);
        const int base = a->tapeBase(seg);
        for (int j = cnt - 1; good && j >= 0; --j) {
            AdjArgs R{};
            const StepArgs A = forwardArgs(h, a, 0, base + j);
            R.P = A.P;
            R.V = A.V;
            R.L = L;
            R.f4 = a->tape(base + j);
            R.prm = A.prm;
            R.sid = A.sid;
            R.skey = A.skey;
            R.start = A.start;
            R.lamIn = a->lamX[lam];
            R.lamOut = a->lamX[lam ^ 1];
            R.lamQ = a->lamQ; R.lamC[0] = a->lamC[0]; R.lamC[1] = a->lamC[1]; R.lamPlane = a->lamPlane; R.lamNv = a->lamNv;
            R.lamPOld = a->lamPOld; R.lamSep = a->lamSep; R.lamP = a->lamP; R.lamV = a->lamV; R.lamR = a->lamR;
            R.gR = a->gR; R.gV0 = a->gV0; R.gTau = a->gTau;
            R.lossPart = a->lossPart + size_t(t0 + j) * size_t(a->lossBlocks);
            R.gatherReach = gatherReach;
            R.err = a->err;
            R.barrier = a->barrier + 4;
            R.stamps = stats ? a->stamps : nullptr;
            if (h->fused) {
                good = ok(h, swarm_gpu::launch_adjoint_step_fused(R, st), "adjoint reverse");
                launches += 1;
            } else {
                swarm_gpu::launch_adjoint_step(R, st, &launches);
                good = ok(h, cudaGetLastError(), "adjoint reverse");
            }
            lam ^= 1;
        }
        if (stats) cudaEventRecord(ev[4 + 3 * size_t(seg)], st);
    }
    if (!good) {
        cudaStreamSynchronize(st);
        for (auto& e : ev) cudaEventDestroy(e);
        return SWARM_E_CUDA;
    }
    std::vector<double> part(size_t(steps) * size_t(a->lossBlocks)), gr(N), gv(N), gt(N);
    int errFlag = 0;
    unsigned long long stampNs[8] = {};
    good = ok(h, cudaMemcpyAsync(part.data(), a->lossPart, part.size() * 8, cudaMemcpyDeviceToHost, st), "loss") &&
           ok(h, cudaMemcpyAsync(gr.data(), a->gR, N * 8, cudaMemcpyDeviceToHost, st), "gradient") &&
           ok(h, cudaMemcpyAsync(gv.data(), a->gV0, N * 8, cudaMemcpyDeviceToHost, st), "gradient") &&
           ok(h, cudaMemcpyAsync(gt.data(), a->gTau, N * 8, cudaMemcpyDeviceToHost, st), "gradient") &&
           ok(h, cudaMemcpyAsync(&errFlag, a->err, 4, cudaMemcpyDeviceToHost, st), "error flag") &&
           ok(h, cudaMemcpyAsync(stampNs, a->stamps, sizeof stampNs, cudaMemcpyDeviceToHost, st), "stamps") &&
           ok(h, cudaStreamSynchronize(st), "adjoint");
    if (good && stats) {
        float ms = 0.0f;
        *stats = SwarmAdjointStats{};
        cudaEventElapsedTime(&ms, ev[0], ev[1]);
        stats->ms_checkpoint = ms;
        for (int seg = 0; seg < nseg; ++seg) {
            cudaEventElapsedTime(&ms, ev[2 + 3 * size_t(seg)], ev[3 + 3 * size_t(seg)]);
            stats->ms_recompute += ms;
            cudaEventElapsedTime(&ms, ev[3 + 3 * size_t(seg)], ev[4 + 3 * size_t(seg)]);
            stats->ms_reverse += ms;
        }
        cudaEventElapsedTime(&ms, ev[0], ev[4 + 3 * 0]);   // segment 0 is reversed last
        stats->ms_total = ms;
        stats->launches = launches;
        stats->tape_bytes = a->bytes;
        stats->segments = nseg;
        stats->kept_segments = a->keep;
        stats->ms_rev_final = float(double(stampNs[0]) * 1e-6);
        stats->ms_rev_sweeps = float(double(stampNs[1]) * 1e-6);
        stats->ms_rev_predict = float(double(stampNs[2]) * 1e-6);
        stats->ms_rev_gather = float(double(stampNs[3]) * 1e-6);
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (!good) return SWARM_E_CUDA;
    if (errFlag & swarm_gpu::ERR_TIMEOUT) {
        cudaMemset(a->barrier, 0, 32);
        return h->fail(SWARM_E_TIMEOUT, "a grid barrier of the adjoint's forward timed out");
    }
    if (errFlag) return h->fail(SWARM_E_CUDA, "the adjoint's forward found its counts out of step with its keys");
    double L2 = 0.0, tau = 0.0;
    for (int t = 0; t < steps; ++t) {
        double s = 0.0;
        for (int b = 0; b < a->lossBlocks; ++b) s += part[size_t(t) * size_t(a->lossBlocks) + size_t(b)];
        L2 += double(h->P.dt) * s;
    }
    for (size_t i = 0; i < N; ++i) {
        dL_dr[i] = float(gr[i]);
        dL_dv0[i] = float(gv[i]);
        tau += gt[i];
    }
    *loss_out = L2;
    *dL_dtau = float(tau);
    return SWARM_OK;
}
