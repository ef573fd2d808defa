// The arguments every kernel of the step takes (by value: kernel parameter space, so that handles with different
// venues and constants coexist in one process).
#pragma once

#include <cstdint>

#include "../../include/swarm_cuda.h"

namespace swarm_gpu {

constexpr uint32_t INACTIVE_CELL = 0xFFFFFFFFu;
constexpr float PLANE_WALL = 1.0f, PLANE_GROUNDED = 2.0f;
constexpr float WALL_NONE = 1e9f;
// ContactBits (reference include/swarm/cpu_crowd_sim.hpp:52-61)
enum : uint8_t { C_EXIT = 1, C_FENCE_CCD = 2, C_FENCE = 4, C_FLOOR = 8, C_WALL = 16, C_AGENT = 32, C_SWEEP = 64, C_STEP_UP = 128 };

// The fused step's contact lists (StepArgs::clist): entries per slot, the count of a slot that keeps none, and the
// fewest other slots in its 3 x 3 rows for which a slot keeps one
constexpr int CLIST_MAX = 24;
constexpr uint8_t CLIST_NONE = 0xFF;
constexpr uint32_t CLIST_MIN_CANDIDATES = 16;

// Device-side error flags (bit set by a kernel, read by the host after the step)
enum : int { ERR_TIMEOUT = 1, ERR_BOUNDS = 2 };
// errMirror's value before a launch that should write it: no combination of the flags above
constexpr int ERR_PENDING = 0x40000000;

struct VenueArgs {
    int32_t kind;
    int32_t resX, resY, ncells;
    float dminX, dminY, dspanX, dspanY, dmaxX, dmaxY;
    float exloX, exloY, exhiX, exhiY, exMaxZ;
    // stadium
    const float* sdf;
    int32_t sdfRes;
    float sdfMinX, sdfMinY, sdfMinZ, sdfSpacing, sdfInv;
    // grid
    const float* wall;
    int32_t wnx, wny;
    float wox, woy, winv;
    const float* nav;
    int32_t nnx, nny;
    float nox, noy, ninv;
    const float* floorH;
    const float2* wallFloor;    // optional: (wall SDF, floor height) per wall-grid node, one sector for both lookups
    const float* speedF;
    const uint8_t* exitMask;    // optional: nonzero at the nav nodes beyond an exit
    uint32_t cellOffset;    // batched instances: this instance's first cell in the shared key space (0 otherwise)
    // seated (the reference's analytic venues): the layout (a device copy); the navigation field's cells (anchor x,
    // anchor y, distance, info bits), navRes^2, x fastest
    const SwarmSeatedLayout* seatDev;
    const float4* navCells;
    int32_t navRes;
    float navOrigin, navCell, navInv;
    int32_t incline, stairHw;   // the incline speed; the stair spacing, with its time gaps up / down
    float stairTUp, stairTDown;
    // the queue-aware exit choice's candidate table on the navigation grid (null: off): index words, entries
    const uint32_t* choiceIndex;
    const uint32_t* choiceEntries;
};

struct StepArgs {
    SwarmParams P;
    VenueArgs V;
    int32_t n;              // agents in the state
    int32_t projectInFinal; // K > 0
    // agent order: the GpuBoid state (position, velocity interleaved: 2 float4 per agent); ping-pong by step
    float4* stateIn;
    float4* stateOut;
    // Host buffers the fused step reads and writes in place of copies (the caller's pinned GpuBoid arrays, as the
    // device sees them over the coherent host link; null otherwise): the hash phase loads the state from hostIn into
    // stateIn; after the final pass (one more grid barrier) the blocks copy stateOut to hostOut in order
    const float4* hostIn;
    float4* hostOut;
    // a pinned host word (device view; null: none) the last block to finish the launch sets to the error flag, so
    // that a host-buffer call reads the flag without a copy; a launch that ends early leaves it as it was
    int* errMirror;
    // queue-aware exit choice (null: off): each agent's assigned exit, whose own distance field (exitFields + exit x
    // navNodes, on the nav grid) gives its e_goal
    const uint32_t* choiceAssign;
    const int32_t* choiceCell;   // a seated venue's table: each agent's choice cell at the step's start (the choice pass's)
    const float* exitFields;
    uint32_t navNodes;
    const float2* aparam;   // (radius, v0) per agent
    const float2* drive;    // forced e_goal per agent, or null
    uint8_t* contacts;      // ContactBits per agent (the last step's)
    // sort
    uint32_t* key;          // cell of each agent (INACTIVE_CELL: evacuated)
    uint32_t* rank;         // arrival order of each agent in its cell's counter
    uint32_t* count;        // agents per cell; ncells + 1 buckets (the last: inactive)
    uint32_t* start;        // exclusive scan of count
    uint2* cells;           // (startIndex, agentCount) per cell, CpuCrowdSim::cells()
    uint32_t* tileSums;     // the scan's per-tile totals
    uint32_t* sidTmp;       // agent ids in scatter order (any order within a cell)
    uint32_t* sid;          // agent ids in slot order (ascending within a cell)
    uint32_t* skey;         // cell of each slot
    // slot order
    float4* pos0;           // start-of-step position (w: 1 active)
    float4* vel0;           // start-of-step velocity
    float2* prm;            // (radius, v0)
    float4* proj[2];        // projection state: xyz, w = displacement so far (>= 0) or -1 (parked this step)
    float4* vel1;           // predicted velocity
    float4* plane;          // wall plane (n.xy, offset) and flags
    uint8_t* ctc;           // the predict pass's contact bits
    uint4* rowsA;           // fused step: each slot's 3 x 3 neighbour rows (row 0 and row 1 ranges)
    uint2* rowsB;           //   (row 2 range)
    float2* goal;           // fused step: each active slot's e_goal, from the gather phase (predict's window reads it)
    int* err;
    unsigned* barrier;      // the fused kernel's grid barrier: arrival counter, generation
    int32_t barrierExtra;   // 0; 1 only in the timeout test: the first barrier waits for a block that never arrives
    unsigned long long* stamps;   // timing on: the fused kernel's stage boundaries (%globaltimer, ns), else null
    int32_t hashed;         // fused step: the keys and counts of this step's input were counted by the last final pass
    int32_t hashNext;       // fused step: count the next step's keys in the final pass (the launch's last step)
    int32_t steps;          // fused step: steps in this launch (0 or 1: one), a grid barrier between them
    int32_t sweepLanes;     // fused step: lanes per slot in the Jacobi sweeps (1, 2, 4, 8; set by the launcher)
    // fused step, one instance: contact lists (null: none). A sweep that builds them records, for each slot whose
    // 3 x 3 rows hold at least CLIST_MIN_CANDIDATES others, the unparked slots nearer (xy) than its largest contact
    // distance + listMargin, in visiting order (CLIST_NONE: none kept), and each slot's path length so far in clistRef;
    // the later sweeps and the final pass walk the lists. A sweep in which a slot's path since the build passes half the
    // margin sets its flag word, and the next sweep builds the lists again (a list can miss a contact only after two
    // slots have moved a margin towards each other). The first sweep of a step always builds. Three flag words in turn:
    // sweep k sets word k mod 3, sweep k + 1 reads it, sweep k + 2 clears it.
    uint32_t* clist;
    uint8_t* ccount;
    float* clistRef;
    int* listFlag;
    float listMargin;
    int32_t fusedThreads;   // fused step: threads per block (0: n / SMs rounded up to a warp, 128..512; 1024 a batch)
    int32_t fusedBlocksPerSm;   // fused step: at most this many blocks per SM (0: as many as fit)
    int32_t scanTile;       // fused step: cells per scan tile (set by the launcher: blockDim x 8, or x 16 on sparse
                            // venues); a fused pass that counts keys also sums them per tile into tileSums
    // batched instances (null otherwise): each instance's venue, the instance of each agent and of each slot
    const VenueArgs* venueTable;
    const uint32_t* instAgent;
    uint32_t* instSlot;
    // the adjoint's taped forward (null otherwise): predict's (sep.x, sep.y, sAhead, argmin slot as int bits, -1: none),
    // one sweep's (relaxed correction before the cap .xy, contact count), the last sweep's result in the final pass
    float4* tapePred;
    float4* tapeCorr;
    float4* tapeQK;
};

}  // namespace swarm_gpu
