// The adjoint of one grid-venue step (adjoint.cu): the arguments of its kernels and the layout of a step's tape.
#pragma once

#include <cuda_runtime.h>

#include "step_args.cuh"

namespace swarm_gpu {

// One step's tape, in the step's slot order. The float4 block holds (2 + Kq + 4 + K) x n float4, Kq = max(K, 1):
//   0 start position, 1 start velocity, 2 .. 1 + Kq the sweeps' inputs q[0 .. Kq - 1] (q[0]: predict's result),
//   2 + Kq the last sweep's result, 3 + Kq predicted velocity, 4 + Kq wall plane, 5 + Kq predict's record
//   (sep.xy, sAhead, argmin slot), 6 + Kq .. 5 + Kq + K the sweeps' relaxed corrections and contact counts (k = 1 .. K)
struct TapeLayout {
    int n, K, Kq;
    __host__ __device__ size_t f4PerStep() const { return size_t(6 + Kq + K) * size_t(n); }
    __host__ __device__ size_t pos0() const { return 0; }
    __host__ __device__ size_t vel0() const { return size_t(n); }
    __host__ __device__ size_t q(int k) const { return size_t(2 + k) * size_t(n); }
    __host__ __device__ size_t qK() const { return size_t(2 + Kq) * size_t(n); }
    __host__ __device__ size_t vel1() const { return size_t(3 + Kq) * size_t(n); }
    __host__ __device__ size_t plane() const { return size_t(4 + Kq) * size_t(n); }
    __host__ __device__ size_t pred() const { return size_t(5 + Kq) * size_t(n); }
    __host__ __device__ size_t corr(int k) const { return size_t(5 + Kq + k) * size_t(n); }   // k = 1 .. K
};

struct AdjArgs {
    SwarmParams P;
    VenueArgs V;
    TapeLayout L;
    // the step's tape
    const float4* f4;
    const float2* prm;          // (radius, v0) per slot
    const uint32_t* sid;        // agent of each slot
    const uint32_t* skey;       // cell of each slot
    const uint32_t* start;      // the cells' run starts (ncells + 2)
    // the state adjoint per agent, 2 float4 each (position, velocity): after the step (in) and before it (out)
    const float4* lamIn;
    float4* lamOut;
    // per slot, within the step
    float4* lamQ;               // the position adjoint carried down the sweeps (xy, z)
    float2* lamC[2];            // the adjoint of each sweep's contact correction sum (ping-pong by sweep)
    float4* lamPlane;           // the wall plane's adjoint (normal.xy, offset), summed over the sweeps
    float4* lamNv;              // the predicted velocity's adjoint (from the final pass)
    float4* lamPOld;            // the start position's adjoint from the final pass
    float4* lamSep;             // predict's (separation.xy, sAhead) adjoints
    float4* lamP;               // predict's own start-position adjoint
    float4* lamV;               // predict's start-velocity adjoint
    float* lamR;                // the radius adjoint of this step
    // the gradients, per agent (summed over the steps)
    double* gR;
    double* gV0;
    double* gTau;
    double* lossPart;           // per block of the final pass: sum of D over its active outputs
    int sweep;                  // the sweep a k_adj_sweep launch reverses
    float gatherReach;          // the pair gather's disk: no pair farther apart has a separation force or is a
                                // headway argmin whose gap moves v_des (2 r_pair_max + max(sep_margin,
                                // v_max * largest speed factor / headway_rate), 1 % slack)
    int* err;                   // device error flags (ERR_TIMEOUT)
    unsigned* barrier;          // the fused reverse's grid barrier words (arrival word, exit counter)
    unsigned long long* stamps; // timing on: the fused reverse adds each phase's %globaltimer span (ns): final, sweeps,
                                // predict, gather (block 0's view; the gather ends when the last block leaves)
};

constexpr int ADJ_FINAL_THREADS = 128;
constexpr int ADJ_FUSED_THREADS = 512;
constexpr int ADJ_LANES = 4;    // lanes per slot in the fused reverse's neighbour gathers
inline int adjFinalBlocks(int n) { return (n + ADJ_FINAL_THREADS - 1) / ADJ_FINAL_THREADS; }

// Reverses one step: the final pass (and the last sweep's own terms, and the loss term of the step's result), the K
// sweeps, predict's local terms, predict's neighbour terms. K + 3 launches.
void launch_adjoint_step(AdjArgs& A, cudaStream_t st, int64_t* launches);
// The same as one cooperative persistent launch with K + 2 grid barriers
cudaError_t launch_adjoint_step_fused(AdjArgs& A, cudaStream_t st);
// The fused reverse's grid size for n agents (the blocks that write loss partials)
int adjFusedBlocks(int n);
int adjFusedThreads(int n);

}  // namespace swarm_gpu
