// The kernels of one crowd step (DedovSergei/swarm-crowd-simulation CrowdSim::step, src/crowd_sim.cpp:316-412;
// its CPU port CpuCrowdSim::step, src/cpu_crowd_sim.cpp:967-1088):
//
//   k_hash        per agent: cell key (calc_grid.comp / CpuCrowdSim::hash :983-993) and its arrival rank in the cell's
//                 counter (warp-aggregated atomics: one atomic per distinct cell per warp)
//   k_scan_*      exclusive scan of the per-cell counts (two tiled passes) -> run starts; the cell table; counts cleared
//   k_scatter     agent -> a slot in its cell's run (arrival order)
//   k_rank_gather per slot: the agent's rank by id among its cell's agents -> the final slot (the key order over
//                 unique (cell, id) keys = the reference's stable counting sort, CpuCrowdSim::sortCounting :997-1006);
//                 gathers the start-of-step state into slot order (reorder.comp)
//   k_predict     physics.comp PHYSICS_PASS 1 (cpu_crowd_sim.cpp:655-777)
//   k_project     one Jacobi sweep, PHYSICS_PASS 2 (cpu_crowd_sim.cpp:781-831), K - 1 launches
//   k_final       the last sweep, the final static contacts, the step-up limit, scatter to agent order (PHYSICS_PASS 3,
//                 cpu_crowd_sim.cpp:835-866)
//
// The inactive agents (evacuated) sort after every cell; they keep their scatter order in the tail, which no pass
// reads by position (the final pass copies each one's state by id). swarm_get_grid orders the tail by id on readout.
#include "step_kernels.cuh"

#include <type_traits>

#include <cuda/atomic>

#include "device_math.cuh"
#include "venue_grid.cuh"
#include "venue_seated.cuh"
#include "venue_stadium.cuh"

namespace swarm_gpu {

__device__ __forceinline__ uint32_t cellID(const VenueArgs& V, float4 p) {
    const int x = sclamp(int((p.x - V.dminX) / V.dspanX * float(V.resX)), 0, V.resX - 1);
    const int y = sclamp(int((p.y - V.dminY) / V.dspanY * float(V.resY)), 0, V.resY - 1);
    return V.cellOffset + uint32_t(x + y * V.resX);
}

// The venue of an agent / a slot: the handle's one venue, or its instance's in a batch
template <bool kB>
__device__ __forceinline__ const VenueArgs& venueOfAgent(const StepArgs& A, uint32_t i) {
    if constexpr (kB) return A.venueTable[A.instAgent[i]]; else return A.V;
}
template <bool kB>
__device__ __forceinline__ const VenueArgs& venueOfSlot(const StepArgs& A, int s) {
    if constexpr (kB) return A.venueTable[A.instSlot[s]]; else return A.V;
}

// Counts agent i's key in its cell's counter and records its arrival rank. Called by all 32 lanes of a warp together
// (warp-aggregated atomics: one atomic per distinct cell per warp); lanes with valid == false take no part.
// kTiles (the fused step): also the count of each scan tile of A.scanTile cells, into tileSums
template <bool kTiles = false>
__device__ __forceinline__ void countKey(const StepArgs& A, uint32_t i, uint32_t key, bool valid) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned mask = __ballot_sync(0xffffffffu, valid);
    if (!valid) return;
    const uint32_t bucket = key == INACTIVE_CELL ? uint32_t(A.V.ncells) : key;
    const unsigned peers = __match_any_sync(mask, bucket);
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (int(lane) == leader) base = atomicAdd(A.count + bucket, uint32_t(__popc(peers)));
    if constexpr (kTiles) {
        const uint32_t tile = bucket / uint32_t(A.scanTile);
        const unsigned tp = __match_any_sync(mask, tile);
        if (int(lane) == __ffs(tp) - 1) atomicAdd(A.tileSums + tile, uint32_t(__popc(tp)));
    }
    base = __shfl_sync(peers, base, leader);
    A.key[i] = key;
    A.rank[i] = base + uint32_t(__popc(peers & ((1u << lane) - 1u)));
}

// calc_grid.comp (CpuCrowdSim::hash, cpu_crowd_sim.cpp:983-993), with its NaN sanitiser. All lanes of a warp together.
template <bool kB, bool kTiles = false>
__device__ __forceinline__ void hashItem(const StepArgs& A, int i, float4* stateIn, const float4* hostIn) {
    const bool valid = i < A.n;
    uint32_t key = 0;
    if (valid) {
        float4 p;
        if (hostIn) {   // the state straight from the caller's host buffer: into the device half this step reads
            p = hostIn[2 * size_t(i)];
            stateIn[2 * size_t(i) + 1] = hostIn[2 * size_t(i) + 1];
            if (isnan(p.x)) p = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
            stateIn[2 * size_t(i)] = p;
        } else {
            p = stateIn[2 * size_t(i)];
            if (isnan(p.x)) { p = make_float4(0.0f, 0.0f, 0.0f, 1.0f); stateIn[2 * size_t(i)] = p; }
        }
        key = p.w == 0.0f ? INACTIVE_CELL : cellID(venueOfAgent<kB>(A, uint32_t(i)), p);
    }
    countKey<kTiles>(A, uint32_t(valid ? i : 0), key, valid);
}

template <bool kB>
__global__ void k_hash(StepArgs A) { hashItem<kB>(A, blockIdx.x * blockDim.x + threadIdx.x, A.stateIn, A.hostIn); }

// The exclusive scan of the ncells + 1 counts, in tiles of SCAN_TILE: k_scan_reduce writes each tile's total,
// k_scan_apply scans its tile on top of the totals of the tiles before it, writes the run starts and the cell table,
// and clears the counts for the next step. No block waits on another.
constexpr int SCAN_THREADS = 256, SCAN_ITEMS = 8, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr int FUSED_MAX_THREADS = 512;   // the fused kernel's largest block (one block per SM, sized to the state)
// the batched instantiation's largest block: a batch has many tiles per block and phase, and its phases are bound by
// the latency of the window loads and the neighbour loops, which more warps per SM hide (64 registers a thread)
constexpr int FUSED_MAX_THREADS_BATCH = 1024;

// Block-wide exclusive scan of one value per thread (any block size that is a multiple of 32, up to 1024)
__device__ __forceinline__ uint32_t blockExclusiveScan(uint32_t v, uint32_t* warpSums, uint32_t& total) {
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (int(lane) >= o) inc += u;
    }
    if (lane == 31) warpSums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nw ? warpSums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, w, o);
            if (int(lane) >= o) w += u;
        }
        if (lane < nw) warpSums[lane] = w;
    }
    __syncthreads();
    total = warpSums[nw - 1];
    return inc - v + (warp > 0 ? warpSums[warp - 1] : 0u);
}

// A thread's ITEMS consecutive counts of the scan (16-byte loads when the run lies inside the array and the array is
// 16-byte aligned: the run's start is a multiple of ITEMS >= 4 words)
__device__ __forceinline__ bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0u; }

template <int ITEMS>
__device__ __forceinline__ void loadCounts(const StepArgs& A, int base, int nb, uint32_t* c) {
    if (base + ITEMS <= nb && aligned16(A.count)) {
#pragma unroll
        for (int j = 0; j < ITEMS; j += 4) {
            const uint4 q = *reinterpret_cast<const uint4*>(A.count + base + j);
            c[j] = q.x; c[j + 1] = q.y; c[j + 2] = q.z; c[j + 3] = q.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) c[j] = base + j < nb ? A.count[base + j] : 0u;
    }
}

// Block-level: the total of tile `tile` (blockDim.x * ITEMS counts) into A.tileSums
template <int ITEMS = SCAN_ITEMS>
__device__ __forceinline__ void scanReduceTile(const StepArgs& A, int tile, uint32_t* warpSums) {
    const int nb = A.V.ncells + 1;
    const int base = tile * int(blockDim.x * ITEMS) + int(threadIdx.x) * ITEMS;
    uint32_t c[ITEMS];
    loadCounts<ITEMS>(A, base, nb, c);
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) sum += c[j];
    uint32_t total;
    blockExclusiveScan(sum, warpSums, total);
    if (threadIdx.x == 0) A.tileSums[tile] = total;
    __syncthreads();   // warpSums is reused by the next tile
}

// Block-level: scan tile `tile` on top of the totals of the tiles before it; run starts, cell table, counts cleared
template <int ITEMS = SCAN_ITEMS>
__device__ __forceinline__ void scanApplyTile(const StepArgs& A, int tile, uint32_t* warpSums, uint32_t* prefix) {
    const int nb = A.V.ncells + 1;
    uint32_t p = 0;
    for (int t = threadIdx.x; t < tile; t += blockDim.x) p += A.tileSums[t];
    for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
    if (threadIdx.x == 0) *prefix = 0;
    __syncthreads();
    if ((threadIdx.x & 31u) == 0 && p) atomicAdd(prefix, p);
    const int base = tile * int(blockDim.x * ITEMS) + int(threadIdx.x) * ITEMS;
    uint32_t c[ITEMS];
    loadCounts<ITEMS>(A, base, nb, c);
    uint32_t sum = 0;
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) sum += c[j];
    uint32_t total;
    uint32_t run = blockExclusiveScan(sum, warpSums, total);   // its barriers also order the prefix atomics
    run += *prefix;
    if (base + ITEMS < nb && aligned16(A.start) && aligned16(A.cells) && aligned16(A.count)) {
        // the whole run inside the cell table, every array 16-byte aligned: 16-byte stores
#pragma unroll
        for (int j = 0; j < ITEMS; j += 4) {
            uint32_t r[4];
            uint2 cl[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                r[q] = run;
                cl[q] = c[j + q] ? make_uint2(run, c[j + q]) : make_uint2(0u, 0u);
                run += c[j + q];
            }
            *reinterpret_cast<uint4*>(A.start + base + j) = make_uint4(r[0], r[1], r[2], r[3]);
            *reinterpret_cast<uint4*>(A.cells + base + j) = make_uint4(cl[0].x, cl[0].y, cl[1].x, cl[1].y);
            *reinterpret_cast<uint4*>(A.cells + base + j + 2) = make_uint4(cl[2].x, cl[2].y, cl[3].x, cl[3].y);
            *reinterpret_cast<uint4*>(A.count + base + j) = make_uint4(0u, 0u, 0u, 0u);   // ready for the next step's hash
        }
    } else {
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const int b = base + j;
            if (b >= nb) break;
            A.start[b] = run;
            if (b < A.V.ncells) A.cells[b] = c[j] ? make_uint2(run, c[j]) : make_uint2(0u, 0u);
            A.count[b] = 0u;   // ready for the next step's hash
            run += c[j];
        }
    }
    __syncthreads();   // prefix and warpSums are reused by the next tile
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(StepArgs A) {
    __shared__ uint32_t warpSums[32];
    scanReduceTile(A, blockIdx.x, warpSums);
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(StepArgs A) {
    __shared__ uint32_t warpSums[32];
    __shared__ uint32_t prefix;
    scanApplyTile(A, blockIdx.x, warpSums, &prefix);
}

__device__ __forceinline__ void scatterItem(const StepArgs& A, int i) {
    const uint32_t key = A.key[i];
    const uint32_t bucket = key == INACTIVE_CELL ? uint32_t(A.V.ncells) : key;
    const uint32_t slot = A.start[bucket] + A.rank[i];
    if (slot >= uint32_t(A.n)) { atomicOr(A.err, ERR_BOUNDS); return; }   // counts out of step with the keys
    A.sidTmp[slot] = uint32_t(i);
}

__global__ void k_scatter(StepArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < A.n) scatterItem(A, i);
}

template <class Venue>
__device__ __forceinline__ f2 goalOf(const StepArgs& A, const Venue& ven, f3 p, uint32_t id);

// The obstacle avoidance term at torso height (physics.comp:1315-1325 sceneDist / sceneNormal / calcGradient): a
// function of the start position alone
template <class Venue>
__device__ __forceinline__ f2 obstacleTerm(const SwarmParams& P, const Venue& ven, float4 p) {
    f2 aObs{0.0f, 0.0f};
    const f3 torso{p.x + 0.0f, p.y + 0.0f, p.z + P.torso_height};
    bool onFence = false;
    const float dTorso = ven.sceneDist(torso, onFence);
    if (dTorso < P.obstacle_range) {
        const f2 norm = ven.sceneNormal(torso, onFence);
        if (length(norm) > P.obstacle_min_normal)
            aObs = safeNormalize(norm, P.safe_eps) * (P.obstacle_range - dTorso) * P.w_obs * P.obstacle_gain;
    }
    return aObs;
}

// Venue (not void): also each slot's e_goal, for the fused step's predict window
template <bool kPerAgent, bool kB, class Venue = void>
__device__ __forceinline__ void rankGatherItem(const StepArgs& A, int s, float4* stateIn) {
    const int nActive = int(A.start[A.V.ncells]);
    const uint32_t me = A.sidTmp[s];
    if (me >= uint32_t(A.n)) { atomicOr(A.err, ERR_BOUNDS); return; }
    if (s >= nActive) { A.sid[s] = me; A.skey[s] = INACTIVE_CELL; return; }
    // The agent's own records (and its e_goal lookup) do not depend on its rank: every load comes before the first
    // store, so these overlap the cell lookup and the rank loop instead of following them
    float4 p = stateIn[2 * size_t(me)];
    const float4 v = stateIn[2 * size_t(me) + 1];
    const uint32_t c = A.key[me];
    float2 prm = make_float2(0.0f, 0.0f);
    if (kPerAgent) prm = A.aparam[me];
    uint32_t inst = 0;
    if (kB) inst = A.instAgent[me];
    const bool bad = isnan(p.x);
    if (bad) p = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    float2 goal = make_float2(0.0f, 0.0f);
    if constexpr (!std::is_void<Venue>::value) {
        const VenueArgs& V = kB ? A.venueTable[inst] : A.V;
        const f2 g = goalOf(A, Venue{A.P, V}, xyz(p), me);
        goal = make_float2(g.x, g.y);
    }
    if (c >= uint32_t(A.V.ncells)) { atomicOr(A.err, ERR_BOUNDS); return; }   // keys and counts out of step
    const uint2 cs = A.cells[c];
    if (uint64_t(cs.x) + cs.y > uint64_t(A.n)) { atomicOr(A.err, ERR_BOUNDS); return; }
    uint32_t r = 0;
    for (uint32_t j = cs.x; j < cs.x + cs.y; ++j) r += A.sidTmp[j] < me ? 1u : 0u;
    const uint32_t t = cs.x + r;
    A.sid[t] = me;
    A.skey[t] = c;
    if (bad) stateIn[2 * size_t(me)] = p;
    A.pos0[t] = p;
    A.vel0[t] = v;
    if (kPerAgent) A.prm[t] = prm;
    if (kB) A.instSlot[t] = inst;
    if constexpr (!std::is_void<Venue>::value) A.goal[t] = goal;
}

template <bool kPerAgent, bool kB>
__global__ void k_rank_gather(StepArgs A) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < A.n) rankGatherItem<kPerAgent, kB>(A, s, A.stateIn);
}

// ---- the physics passes ----
template <class Venue>
struct Body {
    // the reference's own venues: one body radius and free speed for every agent (model units)
    static constexpr bool kUniform = std::is_same<Venue, Stadium>::value || std::is_same<Venue, Seated>::value;
};

template <class Venue>
__device__ __forceinline__ f2 goalOf(const StepArgs& A, const Venue& ven, f3 p, uint32_t id) {
    if (A.drive) { const float2 d = A.drive[id]; return f2{d.x, d.y}; }
    if constexpr (std::is_same<Venue, GridVenue>::value) {
        if (A.choiceAssign) {   // the queue-aware exit choice: the assigned exit's own field
            const uint32_t e = A.choiceAssign[id];
            if (e != SWARM_CHOICE_NONE) return ven.goalIn(A.exitFields + size_t(e) * A.navNodes, p);
        }
    }
    if constexpr (std::is_same<Venue, Seated>::value) {
        // the reference's table: its goal whatever the assignment (none yet: no candidate matches, e_goal 0 but the
        // wall rule), in the choice cell the step's choice pass found for this position
        if (A.choiceAssign && ven.V.choiceIndex) return ven.choiceGoalCell(p, A.choiceAssign[id], A.choiceCell[id]);
    }
    return ven.goal(p);
}

__device__ __forceinline__ f2 separationForce(const SwarmParams& P, f3 offset, uint32_t self, uint32_t other, float rsep, float rsep2) {
    const float d2 = dot(offset, offset);
    if (d2 >= rsep2) return f2{0.0f, 0.0f};
    const float w = 1.0f - sqrtf(d2) / rsep;
    const float magnitude = P.k_sep * w * w;
    const float dxy2 = dot(xy(offset), xy(offset));
    if (dxy2 <= P.stacked_xy2) return magnitude * pairDirection(self, other, P.hash_to_radians);
    return magnitude * xy(offset) * (1.0f / sqrtf(dxy2));
}

// Where predict reads its neighbours: the slot buffers, or a tile's perception window staged in shared memory
struct PredGlobal {
    const StepArgs& A;
    template <class Venue>
    __device__ __forceinline__ f2 goal(uint32_t, const Venue& ven, f3 p, uint32_t id) const { return goalOf(A, ven, p, id); }
    template <class Venue>
    __device__ __forceinline__ f2 obstacle(uint32_t, const Venue& ven, float4 p) const { return obstacleTerm(A.P, ven, p); }
    __device__ __forceinline__ float4 pos(uint32_t k) const { return A.pos0[k]; }
    __device__ __forceinline__ uint32_t sid(uint32_t k) const { return A.sid[k]; }
    __device__ __forceinline__ float r(uint32_t k) const { return A.prm[k].x; }
};
struct PredWindow {
    const float4* pos_;
    const float* r_;
    const uint32_t* sid_;
    const float2* goal_;    // the gather phase's e_goal of each window slot
    const SwarmParams& P;
    uint32_t lo;
    template <class Venue>
    __device__ __forceinline__ f2 goal(uint32_t k, const Venue&, f3, uint32_t) const {
        const float2 g = goal_[k - lo];
        return f2{g.x, g.y};
    }
    template <class Venue>
    __device__ __forceinline__ f2 obstacle(uint32_t, const Venue& ven, float4 p) const { return obstacleTerm(P, ven, p); }
    __device__ __forceinline__ float4 pos(uint32_t k) const { return pos_[k - lo]; }
    __device__ __forceinline__ uint32_t sid(uint32_t k) const { return sid_[k - lo]; }
    __device__ __forceinline__ float r(uint32_t k) const { return r_[k - lo]; }
};

// The rest of predict once the neighbours are summed: desired speed, direction, obstacle avoidance, kinematics,
// the static contacts and the wall plane (cpu_crowd_sim.cpp:727-777)
template <class Venue, class Nbr>
__device__ __forceinline__ void predictFinish(const StepArgs& A, const Venue& ven, int s, float4 p, float4 v, f2 eGoal, f2 sep,
                                              float sAhead, float ri, const Nbr& nb) {
    constexpr bool kUniform = Body<Venue>::kUniform;
    const SwarmParams& P = A.P;
    uint32_t contact = 0;
    float vDes;
    if constexpr (std::is_same<Venue, Seated>::value) {
        vDes = ven.desiredSpeed(xy(p), eGoal, sAhead);   // the incline speed and stair spacing when on
    } else if (kUniform) {
        vDes = sclamp((sAhead - P.body_diam) * P.headway_rate, 0.0f, P.v_max) * length(eGoal);
    } else {
        const float vFree = A.prm[s].y * ven.speedFactor(xyz(p));
        vDes = sclamp(sAhead * P.headway_rate, 0.0f, vFree) * length(eGoal);
    }
    const f2 eDir = safeNormalize(eGoal + sep, P.safe_eps);

    // obstacle avoidance at torso height
    const f2 aObs = nb.obstacle(uint32_t(s), ven, p);

    // kinematics
    const f2 vEq = eDir * vDes + aObs * P.tau_relax;
    f3 nv = xyz(v);
    setXY(nv, vEq + (xy(nv) - vEq) * P.relax_step);
    const float along = dot(xy(nv), eGoal);
    if (along > vDes) setXY(nv, xy(nv) - eGoal * (along - vDes));
    nv.z -= P.gravity_dt;
    nv.z = smin(nv.z, 0.0f);
    if (length(xy(nv)) > P.v_max) setXY(nv, safeNormalize(xy(nv), P.safe_eps) * P.v_max);
    f3 np = xyz(p) + nv * P.dt;

    f3 wall;
    const bool grounded = ven.resolveStatic(xyz(p), np, nv, false, wall, contact, ri);
    if (wall.x == 0.0f && wall.y == 0.0f) wall = ven.wallPlaneProbe(np, ri);
    A.proj[0][s] = make_float4(np.x, np.y, np.z, 0.0f);
    A.vel1[s] = make_float4(nv.x, nv.y, nv.z, 0.0f);
    const f2 wn{wall.x, wall.y};
    A.plane[s] = make_float4(wn.x, wn.y, dot(xy(np), wn) - wall.z,
                             (nonzero(wn) ? PLANE_WALL : 0.0f) + (grounded ? PLANE_GROUNDED : 0.0f));
    A.ctc[s] = uint8_t(contact);
}

template <class Venue, bool kB, bool kTape = false, class Nbr = PredGlobal>
__device__ __forceinline__ void predictCore(const StepArgs& A, int s, const Nbr& nb) {
    constexpr bool kUniform = Body<Venue>::kUniform;
    const int nActive = int(A.start[A.V.ncells]);
    if (s >= nActive) return;
    const SwarmParams& P = A.P;
    const VenueArgs& V = venueOfSlot<kB>(A, s);
    const Venue ven{A.P, V};
    const uint32_t self = A.sid[s], cid = A.skey[s] - V.cellOffset;
    const float4 p = A.pos0[s], v = A.vel0[s];
    if (ven.exits(p)) {
        A.proj[0][s] = make_float4(P.park_coord, P.park_coord, P.park_coord, -1.0f);
        A.vel1[s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        A.ctc[s] = C_EXIT;
        if constexpr (kTape) A.tapePred[s] = make_float4(0.0f, 0.0f, 1e9f, __int_as_float(-1));
        return;
    }
    const f2 eGoal = nb.goal(uint32_t(s), ven, xyz(p), self);
    const float ri = kUniform ? P.body_radius : A.prm[s].x;
    const int resX = V.resX, resY = V.resY;
    const int cx = int(cid % uint32_t(resX)), cy = int(cid / uint32_t(resX));
    f2 sep{0.0f, 0.0f};
    float sAhead = 1e9f;
    int jstar = -1;   // the argmin's slot (taped forward only)
    const int R = P.perc_ring;
    // The neighbour rows: a row of cells is one contiguous run of slots, so each row is [start[a], start[b + 1]) and
    // walking it visits the reference's order (cells by x, agents by slot). Cells that cannot hold an agent within
    // R_PERC are left out of each row (every agent lies inside its cell, widened by `margin`): they contribute
    // nothing, and the nearest-agent-ahead minimum does not depend on the visiting order.
    const float csx = V.dspanX / float(resX), csy = V.dspanY / float(resY);
    const float margin = 0.01f * smax(csx, csy);
    // The search disk: R_PERC, or less where that cannot change the result. A neighbour farther than
    // (largest pair contact distance) + vFree * T_HEADWAY leaves a gap whose headway speed is above vFree, so it
    // cannot lower v_des; the separation ends at R_SEP_ij, nearer still. 1 % slack covers the float rounding.
    const float vFreeSelf = kUniform ? P.v_max : A.prm[s].y * ven.speedFactor(xyz(p));
    const float dcMax = kUniform ? P.body_diam : ri + P.r_pair_max;
    // (seated venues: the stair spacing's time gaps are longer than T_HEADWAY, its free speeds lower than V_MAX)
    float headway;
    if constexpr (std::is_same<Venue, Seated>::value) headway = vFreeSelf * ven.maxHeadwayTime();
    else headway = vFreeSelf / P.headway_rate;
    const float reach = smax(dcMax + headway, kUniform ? P.r_sep : dcMax + P.sep_margin) * 1.01f + margin;
    const float rPerc = smin(sqrtf(P.r_perc2) + margin, reach);
    const float reach2 = reach * reach;
    // every row's slot range first (independent loads, issued together), then the rows in order
    constexpr int MAXR = 2 * 4 + 1;   // PERC_RING <= 4
    uint32_t rk0[MAXR], rk1[MAXR];
#pragma unroll
    for (int j = 0; j < MAXR; ++j) {
        rk0[j] = rk1[j] = 0;
        const int y = j - R;
        const int ny = cy + y;
        if (y > R || ny < 0 || ny >= resY) continue;
        const float ylo = V.dminY + float(ny) * csy - margin, yhi = V.dminY + float(ny + 1) * csy + margin;
        const float dy = fmaxf(0.0f, fmaxf(ylo - p.y, p.y - yhi));
        if (dy >= rPerc) continue;
        const float w = sqrtf(rPerc * rPerc - dy * dy) + margin;
        const int xlo = max(max(cx - R, 0), int(floorf((p.x - w - V.dminX) / csx)));
        const int xhi = min(min(cx + R, resX - 1), int(floorf((p.x + w - V.dminX) / csx)));
        if (xlo > xhi) continue;
        rk0[j] = A.start[V.cellOffset + xlo + ny * resX];
        rk1[j] = A.start[V.cellOffset + xhi + 1 + ny * resX];
    }
#pragma unroll
    for (int j = 0; j < MAXR; ++j) {
        for (uint32_t k = rk0[j]; k < rk1[j]; k++) {
            if (int(k) == s) continue;
            const float4 op = nb.pos(k);
            const f3 offset = xyz(p) - xyz(op);
            const float dxy2 = dot(xy(offset), xy(offset));
            // beyond the search disk a neighbour adds a zero separation and no headway gap below vFree T (the rows'
            // argument, per agent): skipping it changes no bit (separation terms are +0, and +0 additions never
            // change a sum that starts at +0)
            if (dxy2 >= reach2) continue;
            const uint32_t other = nb.sid(k);
            const float rj = kUniform ? 0.0f : nb.r(k);
            if (dxy2 < P.r_perc2) {
                float dc, rs, rs2;
                if (kUniform) { dc = P.body_diam; rs = P.r_sep; rs2 = P.r_sep2; }
                else { dc = ri + rj; rs = dc + P.sep_margin; rs2 = rs * rs; }
                sep = sep + separationForce(P, offset, self, other, rs, rs2);
                const float ahead = -dot(xy(offset), eGoal);
                const float lateral = fabsf(offset.x * eGoal.y - offset.y * eGoal.x);
                const float dxy = sqrtf(dxy2);
                const float key = kUniform ? dxy : dxy - dc;
                if (ahead > 0.0f && lateral < dc && key < sAhead) {
                    const f2 eOther = nb.goal(k, ven, xyz(op), other);
                    const float aheadOther = dot(xy(offset), eOther);
                    const bool mutual = aheadOther > 0.0f && fabsf(offset.x * eOther.y - offset.y * eOther.x) < dc;
                    if (!mutual || ahead > aheadOther || (ahead == aheadOther && self > other)) {
                        sAhead = key;
                        if constexpr (kTape) jstar = int(k);
                    }
                }
            }
        }
    }
    if constexpr (kTape) A.tapePred[s] = make_float4(sep.x, sep.y, sAhead, __int_as_float(jstar));
    predictFinish<Venue>(A, ven, s, p, v, eGoal, sep, sAhead, ri, nb);
}

// predictCore by a group of G lanes per slot (G = 2, 4, 8, adjacent lanes; `sub` = the lane's index in its group):
// every lane of the group evaluates the slot's own terms, the lanes take the neighbour candidates in turn --
// candidate i of the rows' visiting order (rows y, then slots) by lane i mod G -- and in each round every lane adds
// the group's nonzero separation terms in candidate order (ballot, shuffles), so each lane sums exactly the
// reference's nonzero terms in the reference's order (a +0 or -0 term never changes a sum that starts at +0). The
// nearest agent ahead is the least key over the candidates that qualify (the sequential update takes key < sAhead
// under a condition that does not depend on sAhead): a minimum, reduced over the group. Lane 0 of the group writes.
// The whole warp calls it together (own: the lane has a slot below n); one instance, untaped.
template <class Venue, class Nbr>
__device__ __forceinline__ void predictLanes(const StepArgs& A, int s, bool own, const Nbr& nb, int G, int sub, int groupBase) {
    constexpr bool kUniform = Body<Venue>::kUniform;
    const SwarmParams& P = A.P;
    const VenueArgs& V = A.V;
    const Venue ven{A.P, V};
    const int nActive = int(A.start[V.ncells]);
    const bool live = own && s < nActive;
    uint32_t self = 0;
    float4 p = make_float4(0.0f, 0.0f, 0.0f, 0.0f), v = p;
    bool go = false;
    if (live) {
        self = A.sid[s];
        p = A.pos0[s];
        v = A.vel0[s];
        go = !ven.exits(p);
    }
    constexpr int MAXR = 2 * 4 + 1;   // PERC_RING <= 4
    uint32_t rk0[MAXR], rk1[MAXR];
    f2 eGoal{0.0f, 0.0f};
    float ri = 0.0f, reach2 = 0.0f;
#pragma unroll
    for (int j = 0; j < MAXR; ++j) rk0[j] = rk1[j] = 0;
    if (go) {   // predictCore's own terms and rows
        const uint32_t cid = A.skey[s] - V.cellOffset;
        eGoal = nb.goal(uint32_t(s), ven, xyz(p), self);
        ri = kUniform ? P.body_radius : A.prm[s].x;
        const int resX = V.resX, resY = V.resY;
        const int cx = int(cid % uint32_t(resX)), cy = int(cid / uint32_t(resX));
        const int R = P.perc_ring;
        const float csx = V.dspanX / float(resX), csy = V.dspanY / float(resY);
        const float margin = 0.01f * smax(csx, csy);
        const float vFreeSelf = kUniform ? P.v_max : A.prm[s].y * ven.speedFactor(xyz(p));
        const float dcMax = kUniform ? P.body_diam : ri + P.r_pair_max;
        float headway;
        if constexpr (std::is_same<Venue, Seated>::value) headway = vFreeSelf * ven.maxHeadwayTime();
        else headway = vFreeSelf / P.headway_rate;
        const float reach = smax(dcMax + headway, kUniform ? P.r_sep : dcMax + P.sep_margin) * 1.01f + margin;
        const float rPerc = smin(sqrtf(P.r_perc2) + margin, reach);
        reach2 = reach * reach;
#pragma unroll
        for (int j = 0; j < MAXR; ++j) {
            const int y = j - R;
            const int ny = cy + y;
            if (y > R || ny < 0 || ny >= resY) continue;
            const float ylo = V.dminY + float(ny) * csy - margin, yhi = V.dminY + float(ny + 1) * csy + margin;
            const float dy = fmaxf(0.0f, fmaxf(ylo - p.y, p.y - yhi));
            if (dy >= rPerc) continue;
            const float w = sqrtf(rPerc * rPerc - dy * dy) + margin;
            const int xlo = max(max(cx - R, 0), int(floorf((p.x - w - V.dminX) / csx)));
            const int xhi = min(min(cx + R, resX - 1), int(floorf((p.x + w - V.dminX) / csx)));
            if (xlo > xhi) continue;
            rk0[j] = A.start[V.cellOffset + xlo + ny * resX];
            rk1[j] = A.start[V.cellOffset + xhi + 1 + ny * resX];
        }
    }
    uint32_t total = 0;
#pragma unroll
    for (int j = 0; j < MAXR; ++j) total += rk1[j] - rk0[j];
    const uint32_t rounds = __reduce_max_sync(0xffffffffu, (total + uint32_t(G) - 1u) / uint32_t(G));
    const unsigned gmask = (G == 32 ? 0xffffffffu : (1u << G) - 1u) << groupBase;
    f2 sep{0.0f, 0.0f};
    float sAhead = 1e9f;
    for (uint32_t rd = 0; rd < rounds; ++rd) {
        const uint32_t i = rd * uint32_t(G) + uint32_t(sub);
        f2 c{0.0f, 0.0f};
        if (i < total) {
            uint32_t k = 0, acc = 0;   // candidate i's slot: the row whose run holds it
#pragma unroll
            for (int j = 0; j < MAXR; ++j) {
                const uint32_t len = rk1[j] - rk0[j];
                if (i >= acc && i < acc + len) k = rk0[j] + (i - acc);
                acc += len;
            }
            if (int(k) != s) {
                const float4 op = nb.pos(k);
                const f3 offset = xyz(p) - xyz(op);
                const float dxy2 = dot(xy(offset), xy(offset));
                if (dxy2 < reach2 && dxy2 < P.r_perc2) {
                    const uint32_t other = nb.sid(k);
                    const float rj = kUniform ? 0.0f : nb.r(k);
                    float dc, rs, rs2;
                    if (kUniform) { dc = P.body_diam; rs = P.r_sep; rs2 = P.r_sep2; }
                    else { dc = ri + rj; rs = dc + P.sep_margin; rs2 = rs * rs; }
                    c = separationForce(P, offset, self, other, rs, rs2);
                    const float ahead = -dot(xy(offset), eGoal);
                    const float lateral = fabsf(offset.x * eGoal.y - offset.y * eGoal.x);
                    const float dxy = sqrtf(dxy2);
                    const float key = kUniform ? dxy : dxy - dc;
                    if (ahead > 0.0f && lateral < dc && key < sAhead) {
                        const f2 eOther = nb.goal(k, ven, xyz(op), other);
                        const float aheadOther = dot(xy(offset), eOther);
                        const bool mutual = aheadOther > 0.0f && fabsf(offset.x * eOther.y - offset.y * eOther.x) < dc;
                        if (!mutual || ahead > aheadOther || (ahead == aheadOther && self > other)) sAhead = key;
                    }
                }
            }
        }
        // the group's nonzero separation terms of the round, lowest lane (= candidate order) first
        unsigned m = __ballot_sync(0xffffffffu, c.x != 0.0f || c.y != 0.0f) & gmask;
        while (m) {
            const int t = __ffs(m) - 1;
            const float cx = __shfl_sync(gmask, c.x, t);
            const float cy = __shfl_sync(gmask, c.y, t);
            sep = sep + f2{cx, cy};
            m &= m - 1u;
        }
    }
    for (int o = 1; o < G; o <<= 1) sAhead = fminf(sAhead, __shfl_xor_sync(0xffffffffu, sAhead, o));
    if (!live || sub != 0) return;
    if (!go) {   // it reached an exit: parked this step
        A.proj[0][s] = make_float4(P.park_coord, P.park_coord, P.park_coord, -1.0f);
        A.vel1[s] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        A.ctc[s] = C_EXIT;
        return;
    }
    predictFinish<Venue>(A, ven, s, p, v, eGoal, sep, sAhead, ri, nb);
}

template <class Venue, bool kB, bool kTape = false>
__device__ __forceinline__ void predictItem(const StepArgs& A, int s) {
    predictCore<Venue, kB, kTape>(A, s, PredGlobal{A});
}

template <class Venue, bool kB, bool kTape = false>
__global__ void __launch_bounds__(128) k_predict(StepArgs A) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < A.n) predictItem<Venue, kB, kTape>(A, s);
}

// Where a sweep reads its neighbours: the slot buffers in global memory (L2, and L1 for a block's reuse)
struct GlobalNbr {
    const float4* in;
    const float2* prm;
    __device__ __forceinline__ float4 pos(uint32_t k) const { return in[k]; }
    __device__ __forceinline__ float r(uint32_t k) const { return prm[k].x; }
};

// The 3 x 3 neighbour rows of slot s: slot ranges [rk0[j], rk1[j]) for the rows cy - 1 .. cy + 1
__device__ __forceinline__ void sweepRows(const StepArgs& A, const VenueArgs& V, uint32_t key, uint32_t* rk0, uint32_t* rk1) {
    const int resX = V.resX, resY = V.resY;
    const uint32_t cid = key - V.cellOffset;
    const int cx = int(cid % uint32_t(resX)), cy = int(cid / uint32_t(resX));
    const int xlo = max(cx - 1, 0), xhi = min(cx + 1, resX - 1);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const int ny = cy + j - 1;
        const bool ok = ny >= 0 && ny < resY;
        rk0[j] = ok ? A.start[V.cellOffset + xlo + ny * resX] : 0u;
        rk1[j] = ok ? A.start[V.cellOffset + xhi + 1 + ny * resX] : 0u;
    }
}

// One neighbour k of slot s at b in a sweep (cpu_crowd_sim.cpp:793-812): whether they touch, and k's push on s
// (op, rj: k's position and radius, loaded by the caller)
template <class Venue>
__device__ __forceinline__ bool pairPushAt(const StepArgs& A, float4 b, int s, float ri, uint32_t k, float4 op, float rj, f2& c) {
    constexpr bool kUniform = Body<Venue>::kUniform;
    const SwarmParams& P = A.P;
    const f3 offset = xyz(b) - xyz(op);
    float dc, dc2;
    if (kUniform) { dc = P.body_diam; dc2 = P.body_diam2; }
    else { dc = ri + rj; dc2 = dc * dc; }
    const float dxy2 = dot(xy(offset), xy(offset));
    if (!(op.w >= 0.0f && fabsf(offset.z) < dc && dxy2 < dc2)) return false;
    const float dxy = sqrtf(dxy2);
    const float shift = 0.5f * (dc - dxy);
    if (dxy2 <= P.stacked_xy2) c = shift * pairDirection(A.sid[s], A.sid[k], P.hash_to_radians);
    else c = shift * (xy(offset) / dxy);
    return true;
}
template <class Venue, class Nbr>
__device__ __forceinline__ bool pairPush(const StepArgs& A, float4 b, int s, float ri, uint32_t k, const Nbr& nb, f2& c) {
    constexpr bool kUniform = Body<Venue>::kUniform;
    return pairPushAt<Venue>(A, b, s, ri, k, nb.pos(k), kUniform ? 0.0f : nb.r(k), c);
}

// The contact lists' radius for slot s (its largest contact distance with any other + the margin), squared
template <class Venue>
__device__ __forceinline__ float listRadius2(const StepArgs& A, float ri) {
    constexpr bool kUniform = Body<Venue>::kUniform;
    const float rl = (kUniform ? A.P.body_diam : ri + A.P.r_pair_max) + A.listMargin;
    return rl * rl;
}

// The sweep's end for slot s (cpu_crowd_sim.cpp:813-822): the pushes' average relaxed, capped, the fence and the wall
// plane; w of the result: displacement
template <class Venue, bool kTape = false>
__device__ __forceinline__ float4 projectFinish(const StepArgs& A, const Venue& ven, float4 b, f2 corr, int nContacts,
                                               float4 plane, float4* corrOut) {
    const SwarmParams& P = A.P;
    corr = corr * (P.proj_relax / float(smax(nContacts, 1)));
    if constexpr (kTape) {
        if (corrOut) *corrOut = make_float4(corr.x, corr.y, float(nContacts), 0.0f);
    }
    const float len = length(corr);
    if (len > P.proj_max_shift) corr = corr * (P.proj_max_shift / len);
    f3 q = xyz(b);
    setXY(q, xy(q) + corr);
    ven.fenceProject(q);
    if (plane.w == PLANE_WALL || plane.w == PLANE_WALL + PLANE_GROUNDED) {   // fmod(w, 2) == PLANE_WALL, w in {0, 1, 2, 3}
        const float sd = plane.z - dot(xy(q), f2{plane.x, plane.y});
        if (sd > 0.0f) setXY(q, xy(q) + f2{plane.x, plane.y} * sd);
    }
    const f2 d = xy(q) - xy(b);
    return make_float4(q.x, q.y, b.z, b.w + length(d));
}

// One Jacobi sweep of an unparked slot s at b (cpu_crowd_sim.cpp:781-822 projectSlot); w of the result: displacement
template <class Venue, class Nbr, bool kTape = false>
__device__ __forceinline__ float4 projectCore(const StepArgs& A, const Venue& ven, float4 b, int s, float ri,
                                             const uint32_t* rk0, const uint32_t* rk1, float4 plane, const Nbr& nb,
                                             float4* corrOut = nullptr) {
    f2 corr{0.0f, 0.0f};
    int nContacts = 0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        for (uint32_t k = rk0[j]; k < rk1[j]; k++) {
            if (int(k) == s) continue;
            f2 c;
            if (pairPush<Venue>(A, b, s, ri, k, nb, c)) {
                corr = corr + c;
                ++nContacts;
            }
        }
    }
    return projectFinish<Venue, kTape>(A, ven, b, corr, nContacts, plane, corrOut);
}

// The first sweep of slot s with its contact list recorded (the fused step): projectCore's walk of the 3 x 3 rows,
// keeping, in visiting order, every unparked other slot nearer (xy) than the list radius; CLIST_NONE when the rows hold
// fewer than CLIST_MIN_CANDIDATES others or more than CLIST_MAX slots are near
template <class Venue>
__device__ __forceinline__ float4 projectBuild(const StepArgs& A, const Venue& ven, float4 b, int s, float ri,
                                              const uint32_t* rk0, const uint32_t* rk1, float4 plane, const GlobalNbr& nb) {
    constexpr bool kUniform = Body<Venue>::kUniform;
    const uint32_t total = (rk1[0] - rk0[0]) + (rk1[1] - rk0[1]) + (rk1[2] - rk0[2]);
    const bool keep = total > CLIST_MIN_CANDIDATES;   // (the rows hold slot s itself too)
    const float r2 = listRadius2<Venue>(A, ri);
    const size_t n = size_t(A.n);
    f2 corr{0.0f, 0.0f};
    int nContacts = 0;
    uint32_t cnt = 0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        for (uint32_t k = rk0[j]; k < rk1[j]; k++) {
            if (int(k) == s) continue;
            const float4 op = nb.pos(k);
            const float rj = kUniform ? 0.0f : nb.r(k);
            if (keep && op.w >= 0.0f) {
                const float dx = b.x - op.x, dy = b.y - op.y;
                if (dx * dx + dy * dy < r2) {
                    if (cnt < uint32_t(CLIST_MAX)) A.clist[size_t(cnt) * n + size_t(s)] = k;
                    ++cnt;
                }
            }
            f2 c;
            if (pairPushAt<Venue>(A, b, s, ri, k, op, rj, c)) {
                corr = corr + c;
                ++nContacts;
            }
        }
    }
    A.ccount[s] = keep && cnt <= uint32_t(CLIST_MAX) ? uint8_t(cnt) : CLIST_NONE;
    A.clistRef[s] = b.w;
    return projectFinish<Venue, false>(A, ven, b, corr, nContacts, plane, nullptr);
}

// A later sweep of slot s over its contact list of cnt slots (in the rows' visiting order: the same pushes in the
// same order as the rows, whose other slots cannot touch s while the lists hold)
template <class Venue>
__device__ __forceinline__ float4 projectList(const StepArgs& A, const Venue& ven, float4 b, int s, float ri, uint32_t cnt,
                                             float4 plane, const GlobalNbr& nb) {
    const size_t n = size_t(A.n);
    f2 corr{0.0f, 0.0f};
    int nContacts = 0;
    // the entries four at a time (their loads issued together, ahead of the neighbours' loads)
    for (uint32_t i0 = 0; i0 < cnt; i0 += 4) {
        uint32_t e[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) e[q] = i0 + uint32_t(q) < cnt ? A.clist[size_t(i0 + uint32_t(q)) * n + size_t(s)] : 0u;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (i0 + uint32_t(q) >= cnt) break;
            f2 c;
            if (pairPush<Venue>(A, b, s, ri, e[q], nb, c)) {
                corr = corr + c;
                ++nContacts;
            }
        }
    }
    return projectFinish<Venue, false>(A, ven, b, corr, nContacts, plane, nullptr);
}

// The same sweep by a group of G lanes (G = 2, 4, 8; the group's lanes adjacent, `sub` = the lane's index in it): the
// lanes take the slot's candidates in turn -- candidate i of the rows' visiting order (rows y, then slots) by lane
// i mod G -- and every lane folds the group's touching pushes of a round in candidate order (ballot, shuffles), so
// each lane adds the same pushes in the reference's order. The whole warp calls it together; go: the slot is unparked.
// kMode 0: the slot's 3 x 3 rows; 1: the rows, recording the contact list as projectBuild does (in candidate order:
// the group's recorded candidates of a round by lane); 2: its contact list of cnt slots (go: the list holds)
template <class Venue, class Nbr, int kMode = 0>
__device__ __forceinline__ void pairSumLanes(const StepArgs& A, float4 b, int s, float ri, const uint32_t* rk0,
                                             const uint32_t* rk1, const Nbr& nb, bool go, int G, int sub, int groupBase,
                                             f2& corr, int& nContacts, uint32_t cnt = 0) {
    constexpr bool kUniform = Body<Venue>::kUniform;
    uint32_t c0 = 0, c1 = 0, c2 = 0, total = 0;
    if constexpr (kMode == 2) {
        total = go ? cnt : 0u;
    } else {
        c0 = go ? rk1[0] - rk0[0] : 0u;
        c1 = go ? rk1[1] - rk0[1] : 0u;
        c2 = go ? rk1[2] - rk0[2] : 0u;
        total = c0 + c1 + c2;
    }
    const uint32_t rounds = __reduce_max_sync(0xffffffffu, (total + uint32_t(G) - 1u) / uint32_t(G));
    const unsigned gmask = (G == 32 ? 0xffffffffu : (1u << G) - 1u) << groupBase;
    const bool keep = kMode == 1 && total > CLIST_MIN_CANDIDATES;
    const float r2 = kMode == 1 ? listRadius2<Venue>(A, ri) : 0.0f;
    const size_t n = size_t(A.n);
    uint32_t kept = 0;
    corr = f2{0.0f, 0.0f};
    nContacts = 0;
    for (uint32_t r = 0; r < rounds; ++r) {
        const uint32_t i = r * uint32_t(G) + uint32_t(sub);
        f2 c{0.0f, 0.0f};
        int hit = 0, rec = 0;
        uint32_t k = 0;
        if (i < total) {
            if constexpr (kMode == 2) k = A.clist[size_t(i) * n + size_t(s)];
            else k = i < c0 ? rk0[0] + i : i < c0 + c1 ? rk0[1] + (i - c0) : rk0[2] + (i - c0 - c1);
            if (int(k) != s) {
                const float4 op = nb.pos(k);
                const float rj = kUniform ? 0.0f : nb.r(k);
                if (kMode == 1 && keep && op.w >= 0.0f) {
                    const float dx = b.x - op.x, dy = b.y - op.y;
                    rec = dx * dx + dy * dy < r2 ? 1 : 0;
                }
                if (pairPushAt<Venue>(A, b, s, ri, k, op, rj, c)) hit = 1;
            }
        }
        if constexpr (kMode == 1) {   // the group's recorded candidates of the round, in lane (= candidate) order
            const unsigned rm = __ballot_sync(0xffffffffu, rec != 0) & gmask;
            const uint32_t at = kept + uint32_t(__popc(rm & ((1u << (groupBase + sub)) - 1u)));
            if (rec && at < uint32_t(CLIST_MAX)) A.clist[size_t(at) * n + size_t(s)] = k;
            kept += uint32_t(__popc(rm));
        }
        // the group's touching candidates of the round, lowest lane (= candidate order) first; the loop is the same for
        // every lane of the group, so its shuffles name the group's lanes alone
        unsigned m = __ballot_sync(0xffffffffu, hit != 0) & gmask;
        while (m) {
            const int t = __ffs(m) - 1;
            const float cx = __shfl_sync(gmask, c.x, t);
            const float cy = __shfl_sync(gmask, c.y, t);
            corr = corr + f2{cx, cy};
            ++nContacts;
            m &= m - 1u;
        }
    }
    if (kMode == 1 && go && sub == 0) {
        A.ccount[s] = keep && kept <= uint32_t(CLIST_MAX) ? uint8_t(kept) : CLIST_NONE;
        A.clistRef[s] = b.w;
    }
}

// One Jacobi sweep for slot s reading `in` from global memory
template <class Venue, bool kTape = false>
__device__ __forceinline__ float4 projectSlot(const StepArgs& A, const VenueArgs& V, const Venue& ven, const float4* __restrict__ in, int s) {
    constexpr bool kUniform = Body<Venue>::kUniform;
    const float4 b = in[s];
    if (b.w < 0.0f) return b;   // parked this step
    uint32_t rk0[3], rk1[3];
    sweepRows(A, V, A.skey[s], rk0, rk1);
    const float ri = kUniform ? A.P.body_radius : A.prm[s].x;
    return projectCore<Venue, GlobalNbr, kTape>(A, ven, b, s, ri, rk0, rk1, A.plane[s], GlobalNbr{in, A.prm},
                                                kTape ? A.tapeCorr + s : nullptr);
}

template <class Venue, bool kB, bool kTape = false>
__device__ __forceinline__ void projectItem(const StepArgs& A, int s, int inBuf) {
    if (s >= int(A.start[A.V.ncells])) return;
    const VenueArgs& V = venueOfSlot<kB>(A, s);
    const Venue ven{A.P, V};
    A.proj[inBuf ^ 1][s] = projectSlot<Venue, kTape>(A, V, ven, A.proj[inBuf], s);
}

template <class Venue, bool kB, bool kTape = false>
__global__ void __launch_bounds__(128) k_project(StepArgs A, int inBuf) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < A.n) projectItem<Venue, kB, kTape>(A, s, inBuf);
}

// The final pass of an active slot whose last sweep gave b (cpu_crowd_sim.cpp:835-866)
// Returns the agent's cell key for the next step (INACTIVE_CELL once parked; a NaN position hashes as (0, 0, 0, 1))
template <class Venue>
__device__ __forceinline__ uint32_t finalActive(const StepArgs& A, const VenueArgs& V, const Venue& ven, int s, float4 b,
                                                float4* stateOut) {
    const SwarmParams& P = A.P;
    const uint32_t self = A.sid[s];
    if (b.w < 0.0f) {   // parked this step
        stateOut[2 * size_t(self)] = make_float4(P.park_coord, P.park_coord, P.park_coord, 0.0f);
        stateOut[2 * size_t(self) + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        A.contacts[self] = A.ctc[s];
        return INACTIVE_CELL;
    }
    constexpr bool kUniform = Body<Venue>::kUniform;
    const float ri = kUniform ? P.body_radius : A.prm[s].x;
    f3 np = xyz(b);
    f3 nv = xyz(A.vel1[s]);
    const f3 pOld = xyz(A.pos0[s]);
    uint32_t contact = A.ctc[s];
    if (b.w > 0.0f) {   // the projection moved it: the final static contacts
        contact |= C_AGENT;
        f3 wall;
        ven.resolveStatic(pOld, np, nv, A.plane[s].w >= PLANE_GROUNDED, wall, contact, ri);
    }
    if (ven.limitStepUp(pOld, np, nv, ri)) contact |= C_STEP_UP;
    const float4 out = make_float4(np.x, np.y, np.z, 1.0f);
    stateOut[2 * size_t(self)] = out;
    stateOut[2 * size_t(self) + 1] = make_float4(nv.x, nv.y, nv.z, length(nv));
    A.contacts[self] = uint8_t(contact);
    return cellID(V, isnan(out.x) ? make_float4(0.0f, 0.0f, 0.0f, 1.0f) : out);
}

// An agent evacuated before this step: carried over (its next key: inactive)
__device__ __forceinline__ void finalInactive(const StepArgs& A, int s, const float4* stateIn, float4* stateOut) {
    const uint32_t self = A.sid[s];
    stateOut[2 * size_t(self)] = stateIn[2 * size_t(self)];
    stateOut[2 * size_t(self) + 1] = stateIn[2 * size_t(self) + 1];
    A.contacts[self] = 0;
}

template <class Venue, bool kB, bool kTape = false>
__device__ __forceinline__ void finalItem(const StepArgs& A, int s, int inBuf) {
    if (s >= int(A.start[A.V.ncells])) { finalInactive(A, s, A.stateIn, A.stateOut); return; }
    const VenueArgs& V = venueOfSlot<kB>(A, s);
    const Venue ven{A.P, V};
    const float4 b = A.projectInFinal ? projectSlot<Venue, kTape>(A, V, ven, A.proj[inBuf], s) : A.proj[inBuf][s];
    if constexpr (kTape) A.tapeQK[s] = b;
    finalActive(A, V, ven, s, b, A.stateOut);
}

template <class Venue, bool kB, bool kTape = false>
__global__ void __launch_bounds__(128) k_final(StepArgs A, int inBuf) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < A.n) finalItem<Venue, kB, kTape>(A, s, inBuf);
}

// ---- the whole step as one persistent kernel ----
// Every block stays resident (a cooperative launch) and the phases are separated by grid barriers. A barrier is a
// counter and a generation word: the last block to arrive resets the counter and advances the generation (release);
// the others wait for the generation to move (acquire) for at most BARRIER_WAIT_NS of wall-clock time (%globaltimer),
// after which the block records ERR_TIMEOUT and leaves the kernel; a waiting block that finds ERR_TIMEOUT set leaves
// too, and a block that left never arrives at the next barrier, so no phase ever runs on data another block has not
// finished; the host reports SWARM_E_TIMEOUT and resets the barrier words.
constexpr uint64_t BARRIER_WAIT_NS = 1000000000ull;   // 1 s; a healthy barrier waits microseconds

__device__ __forceinline__ uint64_t globalNs() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The fused kernel's stage boundaries (timing on): block 0 records %globaltimer after each barrier
__device__ __forceinline__ void stamp(const StepArgs& A, int i) {
    if (A.stamps && blockIdx.x == 0 && threadIdx.x == 0) A.stamps[i] = globalNs();
}

// This block's share of an array of `bytes` bytes, prefetched into L2 by the copy engine (cp.async.bulk.prefetch: no
// registers, no wait). The shares are whole 16-byte units of the array, the last one ends at the array's last full
// 16-byte unit: every prefetched byte lies inside the array. A base that is not 16-byte aligned is skipped (a hint).
constexpr size_t PREFETCH_STATE_MAX = size_t(16) << 20;
constexpr uint32_t PREFETCH_CHUNK = 64u << 10;

__device__ __forceinline__ void bulkPrefetchShare(const void* base, size_t bytes) {
    if (!base || (reinterpret_cast<uintptr_t>(base) & 15u) != 0u) return;
    const size_t units = bytes / 16u;
    const size_t per = (units + gridDim.x - 1) / gridDim.x;
    const size_t u0 = size_t(blockIdx.x) * per, u1 = u0 + per < units ? u0 + per : units;
    const char* p = static_cast<const char*>(base);
    for (size_t u = u0; u < u1;) {
        const size_t take = u1 - u < PREFETCH_CHUNK / 16u ? u1 - u : PREFETCH_CHUNK / 16u;
        asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p + u * 16u), "r"(uint32_t(take * 16u)) : "memory");
        u += take;
    }
}

// One word per barrier: block 0 adds 2^31 - (expected - 1), every other block adds 1, so the word's top bit flips
// exactly when all `expected` blocks have arrived, and only the last arrival's add flips it: that block goes on at
// once (its add acquires what the earlier adds released), the others wait for the flip of the value they saw (the
// scheme of CUDA's cooperative groups grid sync). Nothing is read before the add: the error word is polled only while
// waiting, every BARRIER_ERR_POLLS polls.
// Returns false (the same in every thread of the block) when the block must leave the kernel.
constexpr unsigned BARRIER_ERR_POLLS = 64;

__device__ __forceinline__ bool gridBarrier(const StepArgs& A, unsigned expected) {
    __shared__ int leave;
    __syncthreads();
    if (threadIdx.x == 0) {
        cuda::atomic_ref<unsigned, cuda::thread_scope_device> word(A.barrier[0]);
        const unsigned add = blockIdx.x == 0 ? 0x80000000u - (expected - 1u) : 1u;
        const unsigned old = word.fetch_add(add, cuda::memory_order_acq_rel);
        int out = 0;
        if ((((old + add) ^ old) & 0x80000000u) == 0u) {
            cuda::atomic_ref<int, cuda::thread_scope_device> err(*A.err);
            const uint64_t t0 = globalNs();
            unsigned polls = 0;
            while (((word.load(cuda::memory_order_acquire) ^ old) & 0x80000000u) == 0u) {
                if (globalNs() - t0 > BARRIER_WAIT_NS) { err.fetch_or(ERR_TIMEOUT, cuda::memory_order_relaxed); out = 1; break; }
                if (++polls % BARRIER_ERR_POLLS == 0u && (err.load(cuda::memory_order_relaxed) & ERR_TIMEOUT)) { out = 1; break; }
            }
        }
        leave = out;
    }
    __syncthreads();
    return leave == 0;
}

// The sweeps' neighbour rows for the fused kernel, once per step: each active slot's 3 x 3 rows as slot ranges
template <bool kB>
__device__ __forceinline__ void prepareSweepItem(const StepArgs& A, int s) {
    const uint32_t cid = A.skey[s];
    const VenueArgs& V = venueOfSlot<kB>(A, s);
    uint32_t rk0[3], rk1[3];
    sweepRows(A, V, cid, rk0, rk1);
    A.rowsA[s] = make_uint4(rk0[0], rk1[0], rk0[1], rk1[1]);
    A.rowsB[s] = make_uint2(rk0[2], rk1[2]);
}

constexpr int WIN_CAP = 4096;   // slots predict's perception window may hold in shared memory (128 KB); larger windows read global memory

// The perception window of tile t (its active slots [t T, min((t + 1) T, nActive))): every slot within perc_ring cell
// rows and columns of its first and last cells, a contiguous range in key order; (0, 0) for a tile with no active slot.
// (A tile spanning batched instances: each slot's cells lie inside its own instance, within these bounds.)
template <bool kB>
__device__ __forceinline__ uint2 predWindow(const StepArgs& A, int t, int T, int nActive) {
    const int s0 = t * T;
    if (s0 >= nActive) return make_uint2(0u, 0u);
    const int s1 = min(s0 + T, nActive) - 1;
    const int R = A.P.perc_ring;
    const int c0 = int(A.skey[s0]), c1 = int(A.skey[s1]);
    const int res0 = venueOfSlot<kB>(A, s0).resX, res1 = venueOfSlot<kB>(A, s1).resX;
    return make_uint2(A.start[max(c0 - R * res0 - R, 0)], A.start[min(c1 + R * res1 + R + 1, A.V.ncells)]);
}

// kTape (the adjoint's recompute): sweep k reads q[k - 1] and writes q[k], q[k] = proj[0] + k n, with its relaxed
// corrections at tapeCorr + (k - 1) n; the final pass records the last sweep's result in tapeQK; predict its record
// kLanes: the instance for few agents on the reference's venues -- predict takes the sweeps' lane groups too (the
// other instances carry none of that code)
template <class Venue, bool kPerAgent, bool kB, bool kTape = false, bool kLanes = false>
__global__ void __launch_bounds__(kB ? FUSED_MAX_THREADS_BATCH : FUSED_MAX_THREADS, 1) k_step_fused(StepArgs A) {
    constexpr bool kUniform = Body<Venue>::kUniform;
    __shared__ uint32_t warpSums[32];
    __shared__ uint32_t prefix;
    extern __shared__ float4 smPos[];   // WIN_CAP positions, then WIN_CAP e_goals, WIN_CAP radii, WIN_CAP ids
    float2* smGoal = reinterpret_cast<float2*>(smPos + WIN_CAP);
    float* smR = reinterpret_cast<float*>(smGoal + WIN_CAP);
    uint32_t* smSid = reinterpret_cast<uint32_t*>(smR + WIN_CAP);
    const int n = A.n;
    const int T = int(blockDim.x);   // the tile of slots a block handles at a time
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    stamp(A, 0);
    // The per-agent records the gather phase reads in id order (state, keys, arrival ranks, radius and v0), prefetched
    // into L2 by the copy engine while the scan and the scatter run: one bulk prefetch per array and block, each block
    // a contiguous share. Only when the state is small beside L2 (a batch's state would evict its own working set).
    if (threadIdx.x == 0 && size_t(n) * 32u <= PREFETCH_STATE_MAX) {
        if (!A.hostIn) bulkPrefetchShare(A.stateIn, size_t(n) * 32u);   // (else the hash phase writes it)
        bulkPrefetchShare(A.key, size_t(n) * 4u);
        bulkPrefetchShare(A.rank, size_t(n) * 4u);
        if (kPerAgent) bulkPrefetchShare(A.aparam, size_t(n) * 8u);
    }
    // A.steps steps in this launch: the state halves swap after every step, each later step starts from the counts
    // the previous final pass left (one more grid barrier between steps), the host buffers serve the first and the
    // last step only
    float4* sIn = A.stateIn;
    float4* sOut = A.stateOut;
    const int steps = A.steps > 1 ? A.steps : 1;
    for (int step = 0; step < steps; ++step) {
        const bool last = step + 1 == steps;
        if (step > 0) {
            float4* t = sIn;
            sIn = sOut;
            sOut = t;
        }
        // The scan runs in tiles of A.scanTile cells (4 or 8 counts a thread, or 16 on sparse venues). Whoever counted the
        // keys -- the previous fused step's final pass, or the hash here -- also summed them per tile, so the scan starts
        // at its apply phase (the tile sums were zero before that counting: cleared below, or by the host).
        if (step == 0 && !A.hashed) {
            for (int base = tid - int(threadIdx.x & 31u); base < n; base += stride)
                hashItem<kB, true>(A, base + int(threadIdx.x & 31u), sIn, A.hostIn);
            if (!gridBarrier(A, gridDim.x)) return;
        }
        const bool wide = A.scanTile > T * SCAN_ITEMS, narrow = A.scanTile < T * SCAN_ITEMS;
        const int tiles = (A.V.ncells + 1 + A.scanTile - 1) / A.scanTile;
        for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
            if (wide) scanApplyTile<2 * SCAN_ITEMS>(A, t, warpSums, &prefix);
            else if (narrow) scanApplyTile<SCAN_ITEMS / 2>(A, t, warpSums, &prefix);
            else scanApplyTile<SCAN_ITEMS>(A, t, warpSums, &prefix);
        }
        // barrierExtra: the timeout test's block that never arrives
        if (!gridBarrier(A, gridDim.x + (step == 0 ? unsigned(A.barrierExtra) : 0u))) return;
        for (int t = tid; t < tiles; t += stride) A.tileSums[t] = 0u;   // read by every apply tile above; summed again below
        for (int i = tid; i < n; i += stride) scatterItem(A, i);
        if (!gridBarrier(A, gridDim.x)) return;
        for (int s = tid; s < n; s += stride) rankGatherItem<kPerAgent, kB, Venue>(A, s, sIn);
        if (!gridBarrier(A, gridDim.x)) return;
        stamp(A, 1);
        // the contact lists' flag of this step (read after the first sweep's barrier; the last step's final pass, which
        // read it, ended three barriers ago)
        if (!kB && !kTape && !std::is_same<Venue, GridVenue>::value && A.clist && blockIdx.x == 0 && threadIdx.x == 0)
            for (int w = 0; w < 3; ++w) cuda::atomic_ref<int, cuda::thread_scope_device>(A.listFlag[w]).store(0, cuda::memory_order_relaxed);
        const int nActive = int(A.start[A.V.ncells]);
        // predict, tile by tile: the tile's perception window staged in shared memory (global reads when it is larger);
        // in the lanes instance, with the sweeps' lane groups (few agents for the GPU), a group of lanes per slot here
        // too: tiles of T / G slots
        const int GP = kLanes ? A.sweepLanes : 1;
        const int TP = T / GP;
        const int allTilesP = (n + TP - 1) / TP;
        for (int t = blockIdx.x; t < allTilesP; t += gridDim.x) {
            const int s = t * TP + int(threadIdx.x) / GP;
            const uint2 win = predWindow<kB>(A, t, TP, nActive);
            const bool useWin = win.y > win.x && win.y - win.x <= uint32_t(WIN_CAP);
            if (useWin) {
                for (uint32_t k = win.x + threadIdx.x; k < win.y; k += blockDim.x) {
                    smPos[k - win.x] = A.pos0[k];
                    smGoal[k - win.x] = A.goal[k];
                    smR[k - win.x] = kUniform ? 0.0f : A.prm[k].x;
                    smSid[k - win.x] = A.sid[k];
                }
            }
            __syncthreads();
            if constexpr (kLanes) {
                if (GP > 1) {   // the whole warp together (its lanes' groups)
                    const int lane = int(threadIdx.x & 31u), sub = lane & (GP - 1);
                    if (useWin) predictLanes<Venue>(A, s, s < n, PredWindow{smPos, smR, smSid, smGoal, A.P, win.x}, GP, sub, lane - sub);
                    else predictLanes<Venue>(A, s, s < n, PredGlobal{A}, GP, sub, lane - sub);
                    if (sub == 0 && s < nActive) prepareSweepItem<kB>(A, s);
                    __syncthreads();   // the window is reused by the next tile
                    continue;
                }
            }
            if (s < n) {
                if (useWin) predictCore<Venue, kB, kTape>(A, s, PredWindow{smPos, smR, smSid, smGoal, A.P, win.x});
                else predictCore<Venue, kB, kTape>(A, s, PredGlobal{A});
                if (s < nActive) prepareSweepItem<kB>(A, s);
            }
            __syncthreads();   // the window is reused by the next tile
        }
        if (!gridBarrier(A, gridDim.x)) return;
        stamp(A, 2);
        const int K = A.P.proj_iterations;
        // the contact lists: the reference's venues (their K = 32 sweeps over dense rows), one instance, untaped (the
        // first sweep records them, the later ones walk them while the flags are clear; predict cleared the flags); the
        // grid venues' instances carry none of this code (their rows hold about 9 agents)
        constexpr bool kListable = !kB && !kTape && !std::is_same<Venue, GridVenue>::value;
        const bool lists = kListable && A.clist != nullptr;
        const float listHold = 0.4995f * A.listMargin;   // (half the margin, less the float rounding of the path length)
        int in = 0;
        for (int it = 1; it < K; ++it) {
            const float4* src = kTape ? A.proj[0] + size_t(it - 1) * size_t(n) : A.proj[in];
            float4* dst = kTape ? A.proj[0] + size_t(it) * size_t(n) : A.proj[in ^ 1];
            float4* corr = kTape ? A.tapeCorr + size_t(it - 1) * size_t(n) : nullptr;
            bool build = false, walk = false;
            if (lists) {
                const int f = it == 1 ? 1 : cuda::atomic_ref<int, cuda::thread_scope_device>(A.listFlag[(it - 1) % 3]).load(cuda::memory_order_relaxed);
                build = f != 0;
                walk = f == 0;
                if (blockIdx.x == 0 && threadIdx.x == 0)
                    cuda::atomic_ref<int, cuda::thread_scope_device>(A.listFlag[(it + 1) % 3]).store(0, cuda::memory_order_relaxed);
            }
            bool moved = false;   // a slot of this thread went beyond half the margin since its list was built
            // The sweeps read their neighbours straight from L2 (and L1, which catches a block's reuse): staging a
            // tile window in shared memory and its two block barriers cost more than they save
            if (!kB && A.sweepLanes > 1) {   // a group of lanes per slot (few agents for the GPU: the launcher's choice)
                const int G = A.sweepLanes, lane = int(threadIdx.x & 31u), sub = lane & (G - 1);
                const int per = 32 / G, warps = stride >> 5;
                for (int first = (tid >> 5) * per; first < nActive; first += warps * per) {   // warp-uniform
                    const int s = first + lane / G;
                    const bool own = s < nActive;
                    float4 b = own ? src[s] : make_float4(0.0f, 0.0f, 0.0f, -1.0f);
                    const bool go = own && b.w >= 0.0f;
                    uint32_t rk0[3] = {0u, 0u, 0u}, rk1[3] = {0u, 0u, 0u};
                    float ri = 0.0f;
                    uint32_t cnt = CLIST_NONE;
                    if (go) {
                        if (walk) cnt = A.ccount[s];
                        if (cnt == CLIST_NONE) {
                            const uint4 ra = A.rowsA[s];
                            const uint2 rb = A.rowsB[s];
                            rk0[0] = ra.x; rk0[1] = ra.z; rk0[2] = rb.x;
                            rk1[0] = ra.y; rk1[1] = ra.w; rk1[2] = rb.y;
                        }
                        ri = kUniform ? A.P.body_radius : A.prm[s].x;
                    }
                    f2 push;
                    int contacts;
                    // (warp-uniform choice: every lane of the warp takes the same path)
                    if (kListable && build) {
                        pairSumLanes<Venue, GlobalNbr, 1>(A, b, s, ri, rk0, rk1, GlobalNbr{src, A.prm}, go, G, sub, lane - sub, push, contacts);
                    } else if (kListable && walk && __any_sync(0xffffffffu, go && cnt != CLIST_NONE)) {
                        // the group's slot walks its list, or its rows (rk) when it keeps none: two passes, each lane
                        // group taking part in the pass of its own kind
                        f2 pl; int cl;
                        pairSumLanes<Venue, GlobalNbr, 2>(A, b, s, ri, rk0, rk1, GlobalNbr{src, A.prm}, go && cnt != CLIST_NONE, G, sub,
                                                          lane - sub, pl, cl, cnt);
                        f2 pr; int cr;
                        pairSumLanes<Venue, GlobalNbr, 0>(A, b, s, ri, rk0, rk1, GlobalNbr{src, A.prm}, go && cnt == CLIST_NONE, G, sub,
                                                          lane - sub, pr, cr);
                        push = cnt != CLIST_NONE ? pl : pr;
                        contacts = cnt != CLIST_NONE ? cl : cr;
                    } else {
                        pairSumLanes<Venue>(A, b, s, ri, rk0, rk1, GlobalNbr{src, A.prm}, go, G, sub, lane - sub, push, contacts);
                    }
                    if (go) {
                        const Venue ven{A.P, venueOfSlot<kB>(A, s)};
                        const float ref = lists ? (build ? b.w : A.clistRef[s]) : 0.0f;
                        b = projectFinish<Venue, kTape>(A, ven, b, push, contacts, A.plane[s],
                                                        kTape && sub == 0 ? corr + s : nullptr);
                        moved |= lists && b.w - ref > listHold;
                    }
                    if (own && sub == 0) dst[s] = b;
                }
            } else {
                for (int s = tid; s < nActive; s += stride) {
                    float4 b = src[s];
                    if (b.w >= 0.0f) {
                        const float ri = kUniform ? A.P.body_radius : A.prm[s].x;
                        const Venue ven{A.P, venueOfSlot<kB>(A, s)};
                        const uint32_t cnt = walk ? A.ccount[s] : CLIST_NONE;
                        const float ref = lists ? (build ? b.w : A.clistRef[s]) : 0.0f;
                        if (kListable && cnt != CLIST_NONE) {
                            b = projectList<Venue>(A, ven, b, s, ri, cnt, A.plane[s], GlobalNbr{src, A.prm});
                        } else {
                            const uint4 ra = A.rowsA[s];
                            const uint2 rb = A.rowsB[s];
                            const uint32_t rk0[3] = {ra.x, ra.z, rb.x}, rk1[3] = {ra.y, ra.w, rb.y};
                            if (kListable && build)
                                b = projectBuild<Venue>(A, ven, b, s, ri, rk0, rk1, A.plane[s], GlobalNbr{src, A.prm});
                            else
                                b = projectCore<Venue, GlobalNbr, kTape>(A, ven, b, s, ri, rk0, rk1, A.plane[s],
                                                                         GlobalNbr{src, A.prm}, kTape ? corr + s : nullptr);
                        }
                        moved |= lists && b.w - ref > listHold;
                    }
                    dst[s] = b;
                }
            }
            if (moved) cuda::atomic_ref<int, cuda::thread_scope_device>(A.listFlag[it % 3]).store(1, cuda::memory_order_relaxed);
            in ^= 1;
            if (!gridBarrier(A, gridDim.x)) return;
        }
        stamp(A, 3);
        // The final pass reads its neighbours from L2 too (warp-aligned slots: the next step's count is warp-collective)
        {
            const float4* src = kTape ? A.proj[0] + size_t(K > 0 ? K - 1 : 0) * size_t(n) : A.proj[in];
            const bool walk = lists && K > 1 &&
                              cuda::atomic_ref<int, cuda::thread_scope_device>(A.listFlag[(K - 1) % 3]).load(cuda::memory_order_relaxed) == 0;
            for (int base = tid - int(threadIdx.x & 31u); base < n; base += stride) {
                const int s = base + int(threadIdx.x & 31u);
                const bool own = s < nActive;
                float4 b = own ? src[s] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                uint32_t nextKey = INACTIVE_CELL;
                if (own) {
                    const VenueArgs& V = venueOfSlot<kB>(A, s);
                    const Venue ven{A.P, V};
                    if (A.projectInFinal && b.w >= 0.0f) {
                        const float ri = kUniform ? A.P.body_radius : A.prm[s].x;
                        const uint32_t cnt = walk ? A.ccount[s] : CLIST_NONE;
                        if (kListable && cnt != CLIST_NONE) {
                            b = projectList<Venue>(A, ven, b, s, ri, cnt, A.plane[s], GlobalNbr{src, A.prm});
                        } else {
                            const uint4 ra = A.rowsA[s];
                            const uint2 rb = A.rowsB[s];
                            const uint32_t rk0[3] = {ra.x, ra.z, rb.x}, rk1[3] = {ra.y, ra.w, rb.y};
                            b = projectCore<Venue, GlobalNbr, kTape>(A, ven, b, s, ri, rk0, rk1, A.plane[s], GlobalNbr{src, A.prm},
                                                                     kTape && K > 0 ? A.tapeCorr + size_t(K - 1) * size_t(n) + s : nullptr);
                        }
                    }
                    if (kTape) A.tapeQK[s] = b;
                    nextKey = finalActive(A, V, ven, s, b, sOut);
                } else if (s < n) {
                    finalInactive(A, s, sIn, sOut);
                }
                if (!last || A.hashNext) countKey<true>(A, s < n ? A.sid[s] : 0u, nextKey, s < n);
            }
        }
        if (!last && !gridBarrier(A, gridDim.x)) return;   // the next step reads these counts and this state
    }
    // The caller's host buffer: the finished state in agent order, copied in order after the last barrier (coalesced
    // 16-byte stores over the host link; the final pass's own writes go to agents in slot order, scattered)
    if (A.hostOut) {
        if (!gridBarrier(A, gridDim.x)) return;
        for (size_t k = size_t(tid); k < 2 * size_t(n); k += size_t(stride)) A.hostOut[k] = sOut[k];
    }
    if (A.stamps || A.errMirror) {   // the end: the last block out records it, and the launch's error flag
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            cuda::atomic_ref<unsigned, cuda::thread_scope_device> done(A.barrier[2]);
            if (done.fetch_add(1u, cuda::memory_order_acq_rel) == gridDim.x - 1) {
                if (A.stamps) A.stamps[4] = globalNs();
                if (A.errMirror) {
                    const int flag = cuda::atomic_ref<int, cuda::thread_scope_device>(*A.err).load(cuda::memory_order_relaxed);
                    cuda::atomic_ref<int, cuda::thread_scope_system>(*A.errMirror).store(flag, cuda::memory_order_release);
                }
                done.store(0u, cuda::memory_order_relaxed);
            }
        }
    }
}

// ---- host launchers ----
namespace {
inline int blocks(int n, int t) { return (n + t - 1) / t; }
}

template <bool kB>
static void sortImpl(const StepArgs& A, cudaStream_t st, int64_t* launches) {
    const int n = A.n;
    k_hash<kB><<<blocks(n, 256), 256, 0, st>>>(A);
    const int tiles = (A.V.ncells + 1 + SCAN_TILE - 1) / SCAN_TILE;
    k_scan_reduce<<<tiles, SCAN_THREADS, 0, st>>>(A);
    k_scan_apply<<<tiles, SCAN_THREADS, 0, st>>>(A);
    k_scatter<<<blocks(n, 256), 256, 0, st>>>(A);
    if (A.P.uniform_body) k_rank_gather<false, kB><<<blocks(n, 256), 256, 0, st>>>(A);
    else k_rank_gather<true, kB><<<blocks(n, 256), 256, 0, st>>>(A);
    *launches += 5;
}

void launch_sort(const StepArgs& A, cudaStream_t st, int64_t* launches) {
    if (A.venueTable) sortImpl<true>(A, st, launches);
    else sortImpl<false>(A, st, launches);
}

template <class Venue, bool kB>
static void stageImpl(const StepArgs& A, int stage, cudaStream_t st, int64_t* launches) {
    const int n = A.n, K = A.P.proj_iterations;
    if (stage == 1) {
        k_predict<Venue, kB><<<blocks(n, 128), 128, 0, st>>>(A);
        *launches += 1;
    } else if (stage == 2) {
        int in = 0;
        for (int it = 1; it < K; ++it) {
            k_project<Venue, kB><<<blocks(n, 128), 128, 0, st>>>(A, in);
            in ^= 1;
        }
        *launches += K > 1 ? K - 1 : 0;
    } else if (stage == 3) {
        k_final<Venue, kB><<<blocks(n, 128), 128, 0, st>>>(A, K > 1 ? (K - 1) & 1 : 0);
        *launches += 1;
    }
}

constexpr int FUSED_SMEM = WIN_CAP * (int(sizeof(float4)) + int(sizeof(float2)) + int(sizeof(float)) + int(sizeof(uint32_t)));

// The fused grid: one block per SM when the state fits (threads = n / SMs rounded up to a warp, 128..512; 128..1024
// for a batch), else as many blocks as stay resident, each taking several tiles per phase
// (The launch helpers' caches are per host thread and per device ordinal: handles stepped from several threads share
// none of them, and a thread that steps handles on several GPUs keeps each GPU's own.)
constexpr int MAX_DEVICES = 64;

static int currentDevice() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) dev = 0;
    return dev;
}

static int smCount() {
    static thread_local int sms[MAX_DEVICES] = {};
    const int dev = currentDevice();
    if (!sms[dev]) cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    return sms[dev];
}

// The block size, and the sweeps' lanes per slot: a group of 8, 4 or 2 lanes per slot when that many threads still fit
// one block per SM (few agents for the GPU: each slot's candidate walk split over its group), else one; a tuned block
// size keeps one lane per slot
static void fusedShape(const StepArgs& A, int& threads, int& lanes) {
    const int sms = smCount();
    const int cap = A.venueTable ? FUSED_MAX_THREADS_BATCH : FUSED_MAX_THREADS;
    lanes = 1;
    if (A.fusedThreads <= 0 && !A.venueTable) {
        for (int g = 8; g > 1; g >>= 1) {
            const long long t = ((static_cast<long long>(A.n) * g + sms - 1) / sms + 31) / 32 * 32;
            if (t <= cap) {
                lanes = g;
                threads = t < 128 ? 128 : int(t);
                return;
            }
        }
    }
    threads = A.fusedThreads > 0 ? A.fusedThreads : ((A.n + sms - 1) / sms + 31) / 32 * 32;
    const int floor = A.fusedThreads > 0 ? 64 : 128;   // a tuned block may be two warps (a scan tile of 16 x 64 cells)
    threads = threads < floor ? floor : (threads > cap ? cap : threads);
    threads = (threads + 31) / 32 * 32;
}

static int fusedThreads(const StepArgs& A) {
    int threads, lanes;
    fusedShape(A, threads, lanes);
    return threads;
}

// Counts a thread in the scan's apply phase: 4, 8 or 16, whichever gives the fewest counts on the busiest block (tiles
// per block, rounded up, x counts a thread: the phase's critical path), the larger on a tie; 4 only for a tile of at
// least 1 024 cells (as the tile sums' buffer assumes)
int fusedScanTile(const StepArgs& A) {
    const int T = fusedThreads(A);
    const int sms = smCount();
    int best = 0, bestCost = 0;
    for (int items = 2 * SCAN_ITEMS; items >= SCAN_ITEMS / 2; items /= 2) {
        if (T * items < 1024) continue;
        const int tiles = (A.V.ncells + 1 + T * items - 1) / (T * items);
        const int cost = (tiles + sms - 1) / sms * items;
        if (best == 0 || cost < bestCost) { best = items; bestCost = cost; }
    }
    return T * best;
}

template <class Venue, bool kPerAgent, bool kB, bool kTape = false, bool kLanes = false>
static cudaError_t fusedImpl(const StepArgs& A0, cudaStream_t st) {
    // the dynamic shared memory limit is a per-device attribute of the kernel: set once per device, kept only when set
    static thread_local bool smemSet[MAX_DEVICES] = {};
    const int dev = currentDevice();
    if (!smemSet[dev]) {
        const cudaError_t e = cudaFuncSetAttribute(k_step_fused<Venue, kPerAgent, kB, kTape, kLanes>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, FUSED_SMEM);
        if (e != cudaSuccess) return e;
        smemSet[dev] = true;
    }
    const int sms = smCount();
    StepArgs A = A0;
    int threads, lanes;
    fusedShape(A, threads, lanes);
    A.sweepLanes = lanes;
    A.scanTile = fusedScanTile(A);
    // the occupancy of the last block size asked for, per device
    static thread_local int occThreads[MAX_DEVICES], occPerSm[MAX_DEVICES];
    static thread_local bool occInit = false;
    if (!occInit) {
        for (int d = 0; d < MAX_DEVICES; ++d) occThreads[d] = -1;
        occInit = true;
    }
    if (occThreads[dev] != threads) {
        const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occPerSm[dev], k_step_fused<Venue, kPerAgent, kB, kTape, kLanes>,
                                                                            threads, FUSED_SMEM);
        if (e != cudaSuccess) return e;
        occThreads[dev] = threads;
    }
    int perSm = occPerSm[dev];
    if (A.fusedBlocksPerSm > 0 && A.fusedBlocksPerSm < perSm) perSm = A.fusedBlocksPerSm;
    const int resident = perSm * sms;
    if (resident <= 0) return cudaErrorCooperativeLaunchTooLarge;
    const int want = int((static_cast<long long>(A.n) * lanes + threads - 1) / threads);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(want < resident ? want : resident));
    cfg.blockDim = dim3(unsigned(threads));
    cfg.dynamicSmemBytes = FUSED_SMEM;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_step_fused<Venue, kPerAgent, kB, kTape, kLanes>, A);
}

cudaError_t launch_step_fused(const StepArgs& A, cudaStream_t st) {
    if (A.V.kind != SWARM_VENUE_GRID) {   // the reference's venues: the lanes instance when the sweeps take lane groups
        int threads, lanes;
        fusedShape(A, threads, lanes);
        if (A.V.kind == SWARM_VENUE_STADIUM)
            return lanes > 1 ? fusedImpl<Stadium, false, false, false, true>(A, st) : fusedImpl<Stadium, false, false>(A, st);
        return lanes > 1 ? fusedImpl<Seated, false, false, false, true>(A, st) : fusedImpl<Seated, false, false>(A, st);
    }
    if (A.venueTable) return fusedImpl<GridVenue, true, true>(A, st);
    return fusedImpl<GridVenue, true, false>(A, st);
}

// The adjoint's taped forward step (grid venue, one instance): the sort, then predict into q[0], sweep k from q[k - 1]
// into q[k] (k = 1 .. K - 1) with its corrections in corr[k], the final pass from q[K - 1] (q[0] when K = 0) with the
// last sweep's result in qK and its corrections in corr[K]
void launch_step_taped(const StepArgs& A, float4* const* q, float4* const* corr, float4* qK, float4* pred, cudaStream_t st,
                       int64_t* launches) {
    const int n = A.n, K = A.P.proj_iterations;
    launch_sort(A, st, launches);
    StepArgs B = A;
    B.proj[0] = q[0];
    B.tapePred = pred;
    k_predict<GridVenue, false, true><<<blocks(n, 128), 128, 0, st>>>(B);
    for (int it = 1; it < K; ++it) {
        B.proj[0] = q[it - 1];
        B.proj[1] = q[it];
        B.tapeCorr = corr[it];
        k_project<GridVenue, false, true><<<blocks(n, 128), 128, 0, st>>>(B, 0);
    }
    B.proj[0] = q[K > 0 ? K - 1 : 0];
    B.tapeCorr = K > 0 ? corr[K] : nullptr;
    B.tapeQK = qK;
    if (K > 0) k_final<GridVenue, false, true><<<blocks(n, 128), 128, 0, st>>>(B, 0);
    else k_final<GridVenue, false, false><<<blocks(n, 128), 128, 0, st>>>(B, 0);
    *launches += 2 + (K > 1 ? K - 1 : 0);
}

cudaError_t launch_step_fused_taped(const StepArgs& A, cudaStream_t st) {
    return fusedImpl<GridVenue, true, false, true>(A, st);
}

void launch_stage(const StepArgs& A, int stage, cudaStream_t st, int64_t* launches) {
    if (stage == 0) { launch_sort(A, st, launches); return; }
    if (A.V.kind == SWARM_VENUE_STADIUM) stageImpl<Stadium, false>(A, stage, st, launches);
    else if (A.V.kind == SWARM_VENUE_SEATED) stageImpl<Seated, false>(A, stage, st, launches);
    else if (A.venueTable) stageImpl<GridVenue, true>(A, stage, st, launches);
    else stageImpl<GridVenue, false>(A, stage, st, launches);
}

}  // namespace swarm_gpu
