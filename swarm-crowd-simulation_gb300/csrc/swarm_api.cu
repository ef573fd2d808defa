// The C ABI of include/swarm_cuda.h: one handle = one simulation on the current CUDA device.
//
// Stands in for the reference's CrowdSim (DedovSergei/swarm-crowd-simulation include/swarm/crowd_sim.hpp:53-194,
// src/crowd_sim.cpp) and mirrors its CPU port CpuCrowdSim (include/swarm/cpu_crowd_sim.hpp:30-169): upload writes the
// state, step runs hash -> key sort -> cell ranges + gather -> predict -> K - 1 sweeps -> final and swaps the state
// halves, the inspection calls return the last step's sorted pairs, cell table and contact bits.
// No exception crosses the boundary: every entry returns a status, swarm_last_error the message.

#include "../../include/swarm_cuda.h"
#include "metrics.cuh"
#include "sim_handle.cuh"
#include "step_kernels.cuh"
#include "venue_seated.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

using swarm_gpu::StepArgs;

namespace {

bool cudaOk(SwarmSim* h, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    h->err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

template <class T>
bool devAlloc(SwarmSim* h, T** p, size_t count) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T)) != cudaSuccess) return false;
    h->allocs.push_back(q);
    *p = static_cast<T*>(q);
    return true;
}

}  // namespace

SwarmSim::~SwarmSim() {
    dropGraphs();
    swarm_adjoint_free(adjoint);
    for (auto& e : ev) if (e) cudaEventDestroy(e);
    for (void* p : allocs) cudaFree(p);
    for (void* p : choiceAllocs) cudaFree(p);
    if (errHost) cudaFreeHost(errHost);
    if (ownStream) cudaStreamDestroy(ownStream);
}

int SwarmSim::deviceError(int flag) {
    cudaMemset(errFlag, 0, 4);
    cudaMemset(barrier, 0, 16);   // a barrier that gave up leaves its counter behind
    cudaMemset(count, 0, (size_t(ncells) + 1) * 4);
    counted = false;
    sumsZero = false;   // a launch that gave up may have left tile sums behind
    if (flag & 1) return fail(SWARM_E_TIMEOUT, "a device-side wait gave up (flag " + std::to_string(flag) + ")");
    return fail(SWARM_E_CUDA, "a device-side bounds check failed (flag " + std::to_string(flag) + ")");
}

StepArgs SwarmSim::args(int in) const {
    StepArgs A{};
    A.P = P;
    auto& v = A.V;
    v.kind = V.kind;
    v.resX = V.grid_res_x; v.resY = V.grid_res_y; v.ncells = ncells;
    v.dminX = V.domain_min_x; v.dminY = V.domain_min_y; v.dspanX = V.domain_span_x; v.dspanY = V.domain_span_y;
    v.dmaxX = V.domain_min_x + V.domain_span_x; v.dmaxY = V.domain_min_y + V.domain_span_y;
    v.exloX = V.exit_lo_x; v.exloY = V.exit_lo_y; v.exhiX = V.exit_hi_x; v.exhiY = V.exit_hi_y; v.exMaxZ = V.exit_max_z;
    v.sdf = dSdf; v.sdfRes = V.sdf_res;
    v.sdfMinX = V.sdf_origin[0]; v.sdfMinY = V.sdf_origin[1]; v.sdfMinZ = V.sdf_origin[2];
    v.sdfSpacing = V.sdf_spacing; v.sdfInv = V.sdf_spacing > 0.0f ? 1.0f / V.sdf_spacing : 0.0f;
    v.wall = dWall; v.wnx = V.wall_nx; v.wny = V.wall_ny; v.wox = V.wall_origin_x; v.woy = V.wall_origin_y;
    v.winv = V.wall_h > 0.0f ? 1.0f / V.wall_h : 0.0f;
    v.nav = dNav; v.nnx = V.nav_nx; v.nny = V.nav_ny; v.nox = V.nav_origin_x; v.noy = V.nav_origin_y;
    v.ninv = V.nav_h > 0.0f ? 1.0f / V.nav_h : 0.0f;
    v.floorH = dFloor; v.speedF = dSpeed; v.exitMask = dMask; v.wallFloor = dWallFloor;
    v.seatDev = dSeat;
    v.navCells = dNavCells;
    v.navRes = V.nav_res; v.navOrigin = V.nav_grid_origin; v.navCell = V.nav_grid_cell; v.navInv = V.nav_grid_inv_cell;
    // the stair spacing is part of the stair model: off without the incline speed (effectiveModelOptions,
    // src/exit_choice.cpp:60-64)
    v.incline = V.incline_speed ? 1 : 0;
    v.stairHw = V.incline_speed && V.stair_headway ? 1 : 0;
    v.stairTUp = V.stair_t_up; v.stairTDown = V.stair_t_down;
    v.choiceIndex = dChIndex;
    v.choiceEntries = dChEntries;
    A.n = n;
    A.projectInFinal = P.proj_iterations > 0 ? 1 : 0;
    A.stateIn = state[in];
    A.stateOut = state[in ^ 1];
    A.aparam = aparam;
    A.drive = driveOn ? drive : nullptr;
    A.contacts = contacts;
    A.key = key; A.rank = rank; A.count = count; A.start = start; A.cells = cells; A.tileSums = tileSums;
    A.sidTmp = sidTmp; A.sid = sid; A.skey = skey;
    A.pos0 = pos0; A.vel0 = vel0; A.prm = prm; A.proj[0] = proj0; A.proj[1] = proj1;
    // the contact lists where the crowd is dense for its hash cells: 9 cells of rows then hold 16 or more agents on
    // average (the reference's seated venues and terrace); sparser crowds (the benchmark halls and the bowl, about 9)
    // gain nothing from them and would pay their loads in every sweep
    const bool dense = clist && 9.0 * double(n) >= 16.0 * double(ncells);
    A.clist = dense ? clist : nullptr;
    A.ccount = ccount; A.clistRef = clistRef; A.listFlag = listFlag;
    // half the largest contact distance of a pair (model units: the uniform body's)
    A.listMargin = 0.5f * (V.kind == SWARM_VENUE_GRID ? 2.0f * P.r_pair_max : P.body_diam);
    A.vel1 = vel1; A.plane = plane; A.ctc = ctc; A.rowsA = rowsA; A.rowsB = rowsB; A.goal = goal; A.err = errFlag; A.barrier = barrier; A.barrierExtra = barrierExtra;
    A.stamps = timing ? stamps : nullptr;
    A.choiceAssign = choiceExits ? dAssign : nullptr;
    A.choiceCell = dChCell;
    A.exitFields = dExitFields;
    A.navNodes = uint32_t(size_t(V.nav_nx) * size_t(V.nav_ny));
    A.fusedThreads = tuning.threads;
    A.fusedBlocksPerSm = tuning.blocks_per_sm;
    A.venueTable = dVenueTable;
    A.instAgent = dInstAgent;
    A.instSlot = dInstSlot;
    return A;
}

int SwarmSim::enqueueMetrics(int in) {
    if (!metricRes) return SWARM_OK;
    swarm_gpu::MetricArgs M{};
    M.prev = state[in];
    M.cur = state[in ^ 1];
    M.n = n;
    M.res = metricRes;
    M.cellsPerUnit = P.metric_cells_per_unit;
    M.offset = float(0.5 * metricRes - 0.5);
    M.centerX = V.metric_center_x;
    M.centerY = V.metric_center_y;
    M.speedScale = P.metric_speed_scale;
    M.stadium = V.kind == SWARM_VENUE_STADIUM ? 1 : 0;
    M.avenueHalf = P.avenue_half;
    M.nExits = std::min(V.n_exits, 56);
    M.exitBoxes = mBoxes;
    M.counters = mCounters;
    M.evacStep = mEvac;
    M.mass = mMass;
    M.thresholds = mThr;
    M.cells = mCells;
    M.stepIndex = ++metricStep;
    swarm_gpu::launch_metrics(M, stream);
    launches += 2;
    return cudaOk(this, cudaGetLastError(), "metrics launch") ? SWARM_OK : SWARM_E_CUDA;
}

int SwarmSim::enqueueStages(int in, int s0, int s1) {
    const StepArgs A = args(in);
    for (int st = s0; st < s1; ++st) swarm_gpu::launch_stage(A, st, stream, &launches);
    return cudaOk(this, cudaGetLastError(), "kernel launch") ? SWARM_OK : SWARM_E_CUDA;
}

// A graph of stages [s0, s1) of a step reading state half `in`
int SwarmSim::captureStages(int in, int s0, int s1, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    if (!cudaOk(this, cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "capture")) return SWARM_E_CUDA;
    const int64_t saved = launches;
    const int rc = enqueueStages(in, s0, s1);
    launches = saved;
    if (!cudaOk(this, cudaStreamEndCapture(stream, &g), "capture end") || rc != SWARM_OK) return SWARM_E_CUDA;
    const bool inst = cudaOk(this, cudaGraphInstantiate(out, g, 0), "graph instantiate");
    cudaGraphDestroy(g);
    return inst ? SWARM_OK : SWARM_E_CUDA;
}

extern "C" {

int swarm_create(const SwarmParams* params, const SwarmVenue* venue, int n_capacity, SwarmHandle* out) {
    if (!params || !venue || !out || n_capacity <= 0) return SWARM_E_INVALID;
    *out = nullptr;
    SwarmSim* h = new (std::nothrow) SwarmSim();
    if (!h) return SWARM_E_OOM;
    h->P = *params;
    h->V = *venue;
    h->capacity = n_capacity;
    const SwarmVenue& V = *venue;
    auto bad = [&](const char* m) { delete h; (void)m; return SWARM_E_INVALID; };
    if (V.kind != SWARM_VENUE_STADIUM && V.kind != SWARM_VENUE_GRID && V.kind != SWARM_VENUE_SEATED) return bad("venue kind");
    if (V.kind == SWARM_VENUE_SEATED) {
        if (!V.seated || !params->uniform_body) return bad("seated layout");
        const SwarmSeatedLayout& L = *V.seated;
        if (L.rows < 1 || L.gangways < 1 || L.gangways > SWARM_SEATED_MAX_GANGWAYS || L.doors < 1 ||
            L.doors > SWARM_SEATED_MAX_DOORS || L.max_band_steps < 0 || !(L.row_depth > 0.0f))
            return bad("seated layout");
        if (V.nav_cells && (V.nav_res < 1 || !(V.nav_grid_cell > 0.0f) || !(V.nav_grid_inv_cell > 0.0f))) return bad("nav grid");
    }
    if (V.grid_res_x <= 0 || V.grid_res_y <= 0 || !(V.domain_span_x > 0.0f) || !(V.domain_span_y > 0.0f)) return bad("grid");
    if (params->proj_iterations < 0 || params->perc_ring < 1 || params->perc_ring > 4) return bad("params");   // the predict pass holds <= 9 rows
    if (V.kind == SWARM_VENUE_STADIUM && (!V.sdf || V.sdf_res < 2 || !(V.sdf_spacing > 0.0f))) return bad("sdf");
    if (V.kind == SWARM_VENUE_GRID && (!V.wall_sdf || !V.nav_dist || V.wall_nx < 2 || V.wall_ny < 2 || V.nav_nx < 2 || V.nav_ny < 2 ||
                                       !(V.wall_h > 0.0f) || !(V.nav_h > 0.0f)))
        return bad("grid fields");
    const double cells = double(V.grid_res_x) * double(V.grid_res_y);
    if (cells > 2.0e9) return bad("too many cells");
    h->ncells = int(cells);
    cudaGetDevice(&h->device);
    if (!cudaOk(h, cudaStreamCreateWithFlags(&h->ownStream, cudaStreamNonBlocking), "stream")) { delete h; return SWARM_E_CUDA; }
    h->stream = h->ownStream;
    const size_t N = size_t(n_capacity);
    bool ok = devAlloc(h, &h->state[0], 2 * N) && devAlloc(h, &h->state[1], 2 * N) && devAlloc(h, &h->aparam, N) &&
              devAlloc(h, &h->drive, N) && devAlloc(h, &h->contacts, N) && devAlloc(h, &h->key, N) && devAlloc(h, &h->rank, N) &&
              devAlloc(h, &h->count, size_t(h->ncells) + 1) && devAlloc(h, &h->start, size_t(h->ncells) + 1) &&
              devAlloc(h, &h->cells, size_t(h->ncells)) && devAlloc(h, &h->tileSums, size_t(h->ncells) / 1024 + 2) && devAlloc(h, &h->sidTmp, N) && devAlloc(h, &h->sid, N) &&
              devAlloc(h, &h->skey, N) && devAlloc(h, &h->pos0, N) && devAlloc(h, &h->vel0, N) && devAlloc(h, &h->proj0, N) &&
              devAlloc(h, &h->proj1, N) && devAlloc(h, &h->vel1, N) && devAlloc(h, &h->plane, N) && devAlloc(h, &h->prm, N) &&
              devAlloc(h, &h->ctc, N) && devAlloc(h, &h->rowsA, N) && devAlloc(h, &h->rowsB, N) &&
              devAlloc(h, &h->goal, N) && devAlloc(h, &h->errFlag, 1) &&
              devAlloc(h, &h->clist, N * swarm_gpu::CLIST_MAX) && devAlloc(h, &h->ccount, N) && devAlloc(h, &h->clistRef, N) &&
              devAlloc(h, &h->listFlag, 4) && devAlloc(h, &h->barrier, 4) && devAlloc(h, &h->stamps, 8) &&
              cudaHostAlloc(reinterpret_cast<void**>(&h->errHost), sizeof(int), cudaHostAllocMapped) == cudaSuccess &&
              cudaHostGetDevicePointer(reinterpret_cast<void**>(&h->errHostDev), h->errHost, 0) == cudaSuccess;
    if (ok && V.kind == SWARM_VENUE_STADIUM) {
        const size_t nv = size_t(V.sdf_res) * size_t(V.sdf_res) * size_t(V.sdf_res);
        ok = devAlloc(h, &h->dSdf, nv) && cudaMemcpy(h->dSdf, V.sdf, nv * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (ok && V.kind == SWARM_VENUE_SEATED) {   // the layout with its band and cell tables
        const std::vector<unsigned char> blob = swarm_gpu::seatedBlob(*V.seated);
        unsigned char* d = nullptr;
        ok = devAlloc(h, &d, blob.size()) && cudaMemcpy(d, blob.data(), blob.size(), cudaMemcpyHostToDevice) == cudaSuccess;
        h->dSeat = reinterpret_cast<SwarmSeatedLayout*>(d);
    }
    if (ok && V.kind == SWARM_VENUE_SEATED && V.nav_cells) {
        const size_t nc = size_t(V.nav_res) * size_t(V.nav_res);
        ok = devAlloc(h, &h->dNavCells, nc) &&
             cudaMemcpy(h->dNavCells, V.nav_cells, nc * sizeof(float4), cudaMemcpyHostToDevice) == cudaSuccess;
    }
    if (ok && V.kind == SWARM_VENUE_GRID) {
        const size_t nw = size_t(V.wall_nx) * size_t(V.wall_ny), nn = size_t(V.nav_nx) * size_t(V.nav_ny);
        ok = devAlloc(h, &h->dWall, nw) && cudaMemcpy(h->dWall, V.wall_sdf, nw * 4, cudaMemcpyHostToDevice) == cudaSuccess &&
             devAlloc(h, &h->dNav, nn) && cudaMemcpy(h->dNav, V.nav_dist, nn * 4, cudaMemcpyHostToDevice) == cudaSuccess;
        if (ok && V.floor_height) {
            ok = devAlloc(h, &h->dFloor, nw) && cudaMemcpy(h->dFloor, V.floor_height, nw * 4, cudaMemcpyHostToDevice) == cudaSuccess;
            // the step's wall and floor lookups at one point read both: interleaved, one 32-byte sector serves both
            std::vector<float2> wf(nw);
            for (size_t i = 0; i < nw; ++i) wf[i] = make_float2(V.wall_sdf[i], V.floor_height[i]);
            ok = ok && devAlloc(h, &h->dWallFloor, nw) && cudaMemcpy(h->dWallFloor, wf.data(), nw * 8, cudaMemcpyHostToDevice) == cudaSuccess;
        }
        if (ok && V.exit_mask)
            ok = devAlloc(h, &h->dMask, nn) && cudaMemcpy(h->dMask, V.exit_mask, nn, cudaMemcpyHostToDevice) == cudaSuccess;
        if (ok && V.speed_factor) {
            ok = devAlloc(h, &h->dSpeed, nw) && cudaMemcpy(h->dSpeed, V.speed_factor, nw * 4, cudaMemcpyHostToDevice) == cudaSuccess;
            for (size_t i = 0; i < nw; ++i) h->speedMax = std::max(h->speedMax, V.speed_factor[i]);
        }
    }
    if (V.n_exits > 0 && V.exit_boxes) h->exitBoxesHost.assign(V.exit_boxes, V.exit_boxes + 4 * size_t(V.n_exits));
    // host pointers of the venue are not kept
    h->V.sdf = nullptr; h->V.wall_sdf = nullptr; h->V.nav_dist = nullptr; h->V.floor_height = nullptr;
    h->V.speed_factor = nullptr; h->V.exit_boxes = nullptr; h->V.exit_mask = nullptr;
    h->V.seated = nullptr; h->V.nav_cells = nullptr;
    if (!ok) { delete h; return SWARM_E_OOM; }
    if (cudaMemset(h->count, 0, (size_t(h->ncells) + 1) * 4) != cudaSuccess || cudaMemset(h->errFlag, 0, 4) != cudaSuccess ||
        cudaMemset(h->barrier, 0, 16) != cudaSuccess ||
        cudaMemset(h->contacts, 0, N) != cudaSuccess) {
        delete h;
        return SWARM_E_CUDA;
    }
    // default per-agent parameters: the uniform body
    std::vector<float2> ap(N, make_float2(params->body_radius, params->v_max));
    cudaMemcpy(h->aparam, ap.data(), N * sizeof(float2), cudaMemcpyHostToDevice);
    for (auto& e : h->ev) cudaEventCreate(&e);
    *out = h;
    return SWARM_OK;
}

int swarm_batch_create(const SwarmParams* params, const SwarmVenue* venues, const int* counts, int m, SwarmHandle* out) {
    if (!params || !venues || !counts || !out || m <= 0) return SWARM_E_INVALID;
    *out = nullptr;
    if (params->proj_iterations < 0 || params->perc_ring < 1 || params->perc_ring > 4) return SWARM_E_INVALID;
    size_t total = 0, cells = 0, nWall = 0, nNav = 0;
    for (int i = 0; i < m; ++i) {
        const SwarmVenue& V = venues[i];
        if (V.kind != SWARM_VENUE_GRID || counts[i] <= 0 || !V.wall_sdf || !V.nav_dist || V.floor_height || V.speed_factor || V.exit_mask ||
            V.grid_res_x <= 0 || V.grid_res_y <= 0 || V.wall_nx < 2 || V.wall_ny < 2 || V.nav_nx < 2 || V.nav_ny < 2 ||
            !(V.wall_h > 0.0f) || !(V.nav_h > 0.0f) || !(V.domain_span_x > 0.0f) || !(V.domain_span_y > 0.0f))
            return SWARM_E_INVALID;   // plain grid venues only (no floor heights, speed factors or exit masks in a batch)
        total += size_t(counts[i]);
        cells += size_t(V.grid_res_x) * size_t(V.grid_res_y);
        nWall += size_t(V.wall_nx) * size_t(V.wall_ny);
        nNav += size_t(V.nav_nx) * size_t(V.nav_ny);
    }
    if (total > size_t(INT32_MAX) / 2 || cells > 2000000000u) return SWARM_E_INVALID;
    // the handle: a grid venue whose key space is every instance's cells, one after another
    SwarmVenue all = venues[0];
    all.grid_res_x = int(cells);
    all.grid_res_y = 1;
    all.floor_height = all.speed_factor = nullptr;
    all.exit_mask = nullptr;
    all.n_exits = 0;
    all.exit_boxes = nullptr;
    SwarmHandle h = nullptr;
    const int rc = swarm_create(params, &all, int(total), &h);
    if (rc != SWARM_OK) return rc;
    h->dropContactLists();   // (a batch's fused step walks its rows)
    // every instance's fields in two device buffers, and its venue record
    float *dWall = nullptr, *dNav = nullptr;
    if (!devAlloc(h, &dWall, nWall) || !devAlloc(h, &dNav, nNav) || !devAlloc(h, &h->dVenueTable, size_t(m)) ||
        !devAlloc(h, &h->dInstAgent, total) || !devAlloc(h, &h->dInstSlot, total)) {
        swarm_destroy(h);
        return SWARM_E_OOM;
    }
    std::vector<swarm_gpu::VenueArgs> table(static_cast<size_t>(m));
    std::vector<uint32_t> inst(total);
    size_t oWall = 0, oNav = 0, oAgent = 0;
    uint32_t oCell = 0;
    h->instStart.clear();
    for (int i = 0; i < m; ++i) {
        const SwarmVenue& V = venues[i];
        const size_t w = size_t(V.wall_nx) * size_t(V.wall_ny), nv = size_t(V.nav_nx) * size_t(V.nav_ny);
        if (cudaMemcpy(dWall + oWall, V.wall_sdf, w * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dNav + oNav, V.nav_dist, nv * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
            swarm_destroy(h);
            return SWARM_E_CUDA;
        }
        swarm_gpu::VenueArgs& a = table[size_t(i)];
        a = swarm_gpu::VenueArgs{};
        a.kind = SWARM_VENUE_GRID;
        a.resX = V.grid_res_x; a.resY = V.grid_res_y; a.ncells = V.grid_res_x * V.grid_res_y;
        a.dminX = V.domain_min_x; a.dminY = V.domain_min_y; a.dspanX = V.domain_span_x; a.dspanY = V.domain_span_y;
        a.dmaxX = V.domain_min_x + V.domain_span_x; a.dmaxY = V.domain_min_y + V.domain_span_y;
        a.exloX = V.exit_lo_x; a.exloY = V.exit_lo_y; a.exhiX = V.exit_hi_x; a.exhiY = V.exit_hi_y; a.exMaxZ = V.exit_max_z;
        a.wall = dWall + oWall; a.wnx = V.wall_nx; a.wny = V.wall_ny; a.wox = V.wall_origin_x; a.woy = V.wall_origin_y;
        a.winv = 1.0f / V.wall_h;
        a.nav = dNav + oNav; a.nnx = V.nav_nx; a.nny = V.nav_ny; a.nox = V.nav_origin_x; a.noy = V.nav_origin_y;
        a.ninv = 1.0f / V.nav_h;
        a.cellOffset = oCell;
        h->instStart.push_back(int(oAgent));
        for (int k = 0; k < counts[i]; ++k) inst[oAgent + size_t(k)] = uint32_t(i);
        oWall += w; oNav += nv; oAgent += size_t(counts[i]);
        oCell += uint32_t(V.grid_res_x * V.grid_res_y);
    }
    h->instStart.push_back(int(total));
    if (cudaMemcpy(h->dVenueTable, table.data(), table.size() * sizeof(table[0]), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->dInstAgent, inst.data(), total * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
        swarm_destroy(h);
        return SWARM_E_CUDA;
    }
    h->instances = m;
    *out = h;
    return SWARM_OK;
}

int swarm_destroy(SwarmHandle h) {
    if (!h) return SWARM_E_INVALID;
    cudaStreamSynchronize(h->stream);
    delete h;
    return SWARM_OK;
}

int swarm_set_stream(SwarmHandle h, void* s) {
    if (!h) return SWARM_E_INVALID;
    h->dropGraphs();
    h->stream = s ? static_cast<cudaStream_t>(s) : h->ownStream;
    return SWARM_OK;
}

int swarm_last_error(SwarmHandle h, char* buf, int len) {
    if (!h || !buf || len <= 0) return SWARM_E_INVALID;
    std::snprintf(buf, size_t(len), "%s", h->err.c_str());
    return SWARM_OK;
}

static int uploadImpl(SwarmHandle h, const float* boids, int n, cudaMemcpyKind kind) {
    if (!h || !boids) return SWARM_E_INVALID;
    if (h->instances && n != h->capacity) return h->fail(SWARM_E_INVALID, "a batch's state holds every instance's agents");
    if (n <= 0 || n > h->capacity) return h->fail(SWARM_E_INVALID, "agent count " + std::to_string(n) + " outside 1.." + std::to_string(h->capacity));
    if (n != h->n) h->dropGraphs();
    if (h->counted && !h->clearCounts()) return h->fail(SWARM_E_CUDA, "clearing the counts");
    h->n = n;
    h->readIdx = 0;
    const size_t bytes = size_t(n) * 32;
    // both halves, as CrowdSim::upload / CpuCrowdSim::setState
    if (!cudaOk(h, cudaMemcpyAsync(h->state[0], boids, bytes, kind, h->stream), "upload") ||
        !cudaOk(h, cudaMemcpyAsync(h->state[1], boids, bytes, kind, h->stream), "upload"))
        return SWARM_E_CUDA;
    h->hasState = true;
    if (!h->resetChoice()) return h->fail(SWARM_E_CUDA, "exit choice reset");
    return SWARM_OK;
}

int swarm_upload_state(SwarmHandle h, const float* boids, int n) { return uploadImpl(h, boids, n, cudaMemcpyHostToDevice); }
int swarm_upload_state_device(SwarmHandle h, const float* d, int n) { return uploadImpl(h, d, n, cudaMemcpyDeviceToDevice); }

static int downloadImpl(SwarmHandle h, float* boids, int n, cudaMemcpyKind kind) {
    if (!h || !boids) return SWARM_E_INVALID;
    if (!h->hasState) return h->fail(SWARM_E_STATE, "no state uploaded");
    if (n != h->n) return h->fail(SWARM_E_INVALID, "download size " + std::to_string(n) + " != state size " + std::to_string(h->n));
    if (!cudaOk(h, cudaMemcpyAsync(boids, h->state[h->readIdx], size_t(n) * 32, kind, h->stream), "download")) return SWARM_E_CUDA;
    if (kind == cudaMemcpyDeviceToHost) return swarm_synchronize(h);
    return SWARM_OK;
}

int swarm_download_state(SwarmHandle h, float* boids, int n) { return downloadImpl(h, boids, n, cudaMemcpyDeviceToHost); }
int swarm_download_state_device(SwarmHandle h, float* d, int n) { return downloadImpl(h, d, n, cudaMemcpyDeviceToDevice); }

int swarm_set_agent_params(SwarmHandle h, const float* radius, const float* v0, int n) {
    if (!h || !radius || !v0 || n <= 0 || n > h->capacity) return SWARM_E_INVALID;
    std::vector<float2> ap(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) {
        if (!(radius[i] > 0.0f) || radius[i] > h->P.r_pair_max || !(v0[i] >= 0.0f) || v0[i] > h->P.v_max)
            return h->fail(SWARM_E_INVALID, "agent " + std::to_string(i) + ": radius must lie in (0, r_pair_max] and v0 in [0, v_max]");
        ap[size_t(i)] = make_float2(radius[i], v0[i]);
    }
    if (!cudaOk(h, cudaMemcpyAsync(h->aparam, ap.data(), size_t(n) * sizeof(float2), cudaMemcpyHostToDevice, h->stream), "params"))
        return SWARM_E_CUDA;
    return cudaOk(h, cudaStreamSynchronize(h->stream), "params") ? SWARM_OK : SWARM_E_CUDA;
}

int swarm_set_iterations(SwarmHandle h, int k) {
    if (!h) return SWARM_E_INVALID;
    if (k < 0) return h->fail(SWARM_E_INVALID, "iterations must be >= 0");
    h->P.proj_iterations = k;
    h->dropGraphs();
    return SWARM_OK;
}

int swarm_set_drive_table(SwarmHandle h, const float* dirs, int n) {
    if (!h) return SWARM_E_INVALID;
    h->dropGraphs();
    if (!dirs) { h->driveOn = false; return SWARM_OK; }
    if (n != h->n) return h->fail(SWARM_E_INVALID, "the drive table must have one entry per agent");
    if (!cudaOk(h, cudaMemcpyAsync(h->drive, dirs, size_t(n) * sizeof(float2), cudaMemcpyHostToDevice, h->stream), "drive"))
        return SWARM_E_CUDA;
    h->driveOn = true;
    return cudaOk(h, cudaStreamSynchronize(h->stream), "drive") ? SWARM_OK : SWARM_E_CUDA;
}

int swarm_set_relaxation_time(SwarmHandle h, float tau) {
    if (!h) return SWARM_E_INVALID;
    if (!(tau > 0.0f)) return h->fail(SWARM_E_INVALID, "tau must be > 0");
    h->P.tau_relax = tau;
    h->P.relax_step = float(std::exp(-double(h->P.dt) / double(tau)));
    h->dropGraphs();
    return SWARM_OK;
}

int swarm_set_graph(SwarmHandle h, int enabled) {
    if (!h) return SWARM_E_INVALID;
    h->useGraph = enabled != 0;
    if (!h->useGraph) h->dropGraphs();
    return SWARM_OK;
}

int swarm_metrics_enable(SwarmHandle h, int res, const uint32_t* threshold_mass) {
    if (!h || !threshold_mass || res <= 0 || res % 16 != 0 || res > 4096) return SWARM_E_INVALID;
    if (h->instances) return h->fail(SWARM_E_INVALID, "metrics are per venue; a batch has many");
    if (!h->metricRes) {
        const size_t cells = size_t(res) * size_t(res), N = size_t(h->capacity);
        const size_t boxes = std::max<size_t>(h->exitBoxesHost.size() / 4, 1);
        if (!(devAlloc(h, &h->mCounters, 1) && devAlloc(h, &h->mEvac, N) && devAlloc(h, &h->mMass, cells) &&
              devAlloc(h, &h->mThr, cells) && devAlloc(h, &h->mCells, cells) && devAlloc(h, &h->mBoxes, boxes)))
            return h->fail(SWARM_E_OOM, "metrics buffers");
        if (!h->exitBoxesHost.empty() &&
            !cudaOk(h, cudaMemcpy(h->mBoxes, h->exitBoxesHost.data(), h->exitBoxesHost.size() * 4, cudaMemcpyHostToDevice), "boxes"))
            return SWARM_E_CUDA;
        h->metricRes = res;
    } else if (res != h->metricRes) {
        return h->fail(SWARM_E_INVALID, "the metric grid's resolution is fixed once enabled");
    }
    const size_t cells = size_t(res) * size_t(res);
    if (!cudaOk(h, cudaMemcpy(h->mThr, threshold_mass, cells * 16, cudaMemcpyHostToDevice), "thresholds")) return SWARM_E_CUDA;
    return swarm_metrics_reset(h);
}

int swarm_metrics_reset(SwarmHandle h) {
    if (!h) return SWARM_E_INVALID;
    if (!h->metricRes) return h->fail(SWARM_E_STATE, "metrics are not enabled");
    const size_t cells = size_t(h->metricRes) * size_t(h->metricRes);
    h->metricStep = 0;
    const bool ok = cudaMemsetAsync(h->mCounters, 0, sizeof(SwarmMetricCounters), h->stream) == cudaSuccess &&
                    cudaMemsetAsync(h->mEvac, 0, size_t(h->capacity) * 4, h->stream) == cudaSuccess &&
                    cudaMemsetAsync(h->mMass, 0, cells * 8, h->stream) == cudaSuccess &&
                    cudaMemsetAsync(h->mCells, 0, cells * sizeof(SwarmMetricCell), h->stream) == cudaSuccess;
    return ok ? SWARM_OK : h->fail(SWARM_E_CUDA, "metrics reset");
}

int swarm_metrics_read(SwarmHandle h, SwarmMetricCounters* counters, SwarmMetricCell* cells, uint32_t* evac_step, int n) {
    if (!h) return SWARM_E_INVALID;
    if (!h->metricRes) return h->fail(SWARM_E_STATE, "metrics are not enabled");
    if (!cudaOk(h, cudaStreamSynchronize(h->stream), "sync")) return SWARM_E_CUDA;
    if (counters) cudaMemcpy(counters, h->mCounters, sizeof *counters, cudaMemcpyDeviceToHost);
    if (cells) cudaMemcpy(cells, h->mCells, size_t(h->metricRes) * size_t(h->metricRes) * sizeof(SwarmMetricCell), cudaMemcpyDeviceToHost);
    if (evac_step) {
        if (n != h->n) return h->fail(SWARM_E_INVALID, "evac_step size mismatch");
        cudaMemcpy(evac_step, h->mEvac, size_t(n) * 4, cudaMemcpyDeviceToHost);
    }
    return cudaOk(h, cudaGetLastError(), "metrics read") ? SWARM_OK : SWARM_E_CUDA;
}

static int stepImpl(SwarmHandle h, int steps, bool countLast = true);

int swarm_set_tuning(SwarmHandle h, const SwarmTuning* t) {
    if (!h || !t || t->threads < 0 || t->blocks_per_sm < 0 || t->steps_per_launch < 0) return SWARM_E_INVALID;
    if (t->threads > (h->instances ? 1024 : 512))
        return h->fail(SWARM_E_INVALID, "threads above " + std::to_string(h->instances ? 1024 : 512) + " per block");
    // (the fused step's scan tiles hold at least 1 024 cells: 16 counts a thread of at least 64 threads)
    if (t->threads > 0 && t->threads < 64) return h->fail(SWARM_E_INVALID, "threads below 64 per block");
    h->tuning = *t;
    h->fused = t->fused != 0;
    h->dropGraphs();
    return SWARM_OK;
}

int swarm_autotune(SwarmHandle h, int steps, SwarmTuning* best) {
    if (!h || steps <= 0) return SWARM_E_INVALID;
    if (!h->hasState) return h->fail(SWARM_E_STATE, "autotune needs a state (upload one first)");
    // the candidates: the fused step at several block shapes, and the per-phase kernels replayed from graphs
    std::vector<SwarmTuning> cands;
    for (int threads : {0, 128, 256, 512, 768, 1024}) {
        if (threads > 512 && !h->instances) continue;   // wider blocks: the batched kernel only
        for (int bps : {0, 1, 2}) cands.push_back(SwarmTuning{1, threads, bps, 0.0f, 0});
    }
    cands.push_back(SwarmTuning{1, 0, 0, 0.0f, 1});   // a launch per step
    cands.push_back(SwarmTuning{0, 0, 0, 0.0f, 0});
    // snapshot of the state (and the metrics' running sums are not touched: the trials run with metrics off)
    float4* snap = nullptr;
    const size_t bytes = size_t(h->n) * 32;
    if (cudaMalloc(&snap, bytes) != cudaSuccess) return h->fail(SWARM_E_OOM, "autotune snapshot");
    cudaMemcpyAsync(snap, h->state[h->readIdx], bytes, cudaMemcpyDeviceToDevice, h->stream);
    const int metricRes = h->metricRes, choiceExits = h->choiceExits;
    const bool graph = h->useGraph, timing = h->timing;
    const SwarmTuning keep = h->tuning;
    h->metricRes = 0;
    h->choiceExits = 0;   // (the trials step without the exit choice: its state is not touched)
    h->useGraph = true;
    h->timing = false;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    SwarmTuning top{};
    top.ms_per_step = 1e30f;
    int rc = SWARM_OK;
    for (SwarmTuning c : cands) {
        h->tuning = c;
        h->fused = c.fused != 0;
        h->dropGraphs();
        cudaMemcpyAsync(h->state[h->readIdx], snap, bytes, cudaMemcpyDeviceToDevice, h->stream);
        if (h->counted && !h->clearCounts()) { rc = SWARM_E_CUDA; break; }
        if ((rc = stepImpl(h, 1)) != SWARM_OK) break;   // warm-up (graph capture)
        cudaEventRecord(e0, h->stream);
        if ((rc = stepImpl(h, steps)) != SWARM_OK) break;
        cudaEventRecord(e1, h->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) { rc = SWARM_E_CUDA; break; }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        c.ms_per_step = ms / float(steps);
        if (c.ms_per_step < top.ms_per_step) top = c;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // the state as it was, the best configuration in force
    cudaMemcpyAsync(h->state[h->readIdx], snap, bytes, cudaMemcpyDeviceToDevice, h->stream);
    if (h->counted) h->clearCounts();
    cudaStreamSynchronize(h->stream);
    cudaFree(snap);
    h->metricRes = metricRes;
    h->choiceExits = choiceExits;
    h->useGraph = graph;
    h->timing = timing;
    h->dropGraphs();
    if (rc != SWARM_OK) { h->tuning = keep; h->fused = keep.fused != 0; return rc; }
    h->tuning = top;
    h->fused = top.fused != 0;
    if (!h->fused) h->useGraph = true;   // the per-phase candidate was timed replaying graphs
    if (best) *best = top;
    return swarm_synchronize(h);
}

int swarm_test_barrier_timeout(SwarmHandle h) {
    if (!h) return SWARM_E_INVALID;
    h->barrierExtra = 1;
    return SWARM_OK;
}

int swarm_set_fused(SwarmHandle h, int enabled) {
    if (!h) return SWARM_E_INVALID;
    h->fused = enabled != 0;
    h->dropGraphs();
    return SWARM_OK;
}

int swarm_set_timing(SwarmHandle h, int enabled) {
    if (!h) return SWARM_E_INVALID;
    if (h->timing != (enabled != 0)) h->dropGraphs();   // the graphs hold the event records or not
    h->timing = enabled != 0;
    return SWARM_OK;
}

// One step = 4 stages. Timing on: an event before each stage and after the last, recorded on the stream between
// stage launches (or stage graphs), never inside a capture.
// countLast: the last fused step counts the next state's keys for the next call (false when the next call uploads a
// new state: the counts are then left clear, and nothing has to clear them)
static int stepImpl(SwarmHandle h, int steps, bool countLast) {
    h->launches = 0;
    const int perStep = 7 + std::max(h->P.proj_iterations - 1, 0);
    // steps one fused launch may run: all of them (or the tuning's steps_per_launch), unless something runs between
    // steps on the host's side (the exit choice's pass, the metrics) or each step is timed
    const bool chain = h->fused && !h->choiceExits && !h->metricRes && !h->timing;
    const int chunkMax = !chain ? 1 : (h->tuning.steps_per_launch > 0 ? h->tuning.steps_per_launch : std::max(steps, 1));
    for (int s = 0; s < steps;) {
        const int in = h->readIdx;
        const int chunk = h->fused ? std::min(chunkMax, steps - s) : 1;
        if (h->choiceExits && h->enqueueChoice(in) != SWARM_OK) return SWARM_E_CUDA;
        if (h->fused) {
            if (h->timing && !cudaOk(h, cudaEventRecord(h->ev[0], h->stream), "event")) return SWARM_E_CUDA;
            StepArgs A = h->args(in);
            // the counts (and their scan-tile sums) carried from the last fused step, if its tile matches this one's
            const int tile = swarm_gpu::fusedScanTile(A);
            if (h->counted && tile != h->countedTile && !h->clearCounts()) return SWARM_E_CUDA;
            if (!h->counted && !h->sumsZero) {
                if (!cudaOk(h, cudaMemsetAsync(h->tileSums, 0, (size_t(h->ncells) / 1024 + 2) * 4, h->stream), "tile sums"))
                    return SWARM_E_CUDA;
                h->sumsZero = true;
            }
            A.hashed = h->counted ? 1 : 0;
            A.hashNext = (countLast || s + chunk < steps) ? 1 : 0;
            A.steps = chunk;
            A.hostIn = s == 0 ? h->hostIn : nullptr;
            A.hostOut = s + chunk == steps ? h->hostOut : nullptr;
            A.errMirror = A.hostOut ? h->errHostDev : nullptr;
            if (A.hostIn && A.hashed) return h->fail(SWARM_E_STATE, "a host input needs the hash phase (counts left over)");
            // one step from counted keys, with counting, no host buffers and nothing timed: replayed from a graph
            // (one per state half) when graphs are on
            const bool steady = h->useGraph && !h->timing && chunk == 1 && A.hashed && A.hashNext && !A.hostIn &&
                                !A.hostOut && !A.barrierExtra;
            if (steady && !h->fusedGraph[in]) {
                cudaGraph_t g = nullptr;
                if (!cudaOk(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "capture")) return SWARM_E_CUDA;
                const cudaError_t le = swarm_gpu::launch_step_fused(A, h->stream);
                const cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
                if (!cudaOk(h, le, "fused step capture") || !cudaOk(h, ce, "capture end")) { if (g) cudaGraphDestroy(g); return SWARM_E_CUDA; }
                const bool inst = cudaOk(h, cudaGraphInstantiate(&h->fusedGraph[in], g, 0), "graph instantiate");
                cudaGraphDestroy(g);
                if (!inst) return SWARM_E_CUDA;
            }
            if (steady) {
                if (!cudaOk(h, cudaGraphLaunch(h->fusedGraph[in], h->stream), "graph launch")) return SWARM_E_CUDA;
            } else if (!cudaOk(h, swarm_gpu::launch_step_fused(A, h->stream), "fused step launch")) {
                return SWARM_E_CUDA;
            }
            h->barrierExtra = 0;
            h->counted = A.hashNext != 0;
            h->sumsZero = !h->counted;   // the launch clears the sums after its scans and adds none at its end
            h->countedTile = tile;
            if (h->timing && !cudaOk(h, cudaEventRecord(h->ev[4], h->stream), "event")) return SWARM_E_CUDA;
            h->launches += 1;
        } else {
            if (h->counted && !h->clearCounts()) return SWARM_E_CUDA;
            h->sumsZero = false;   // the per-phase scan writes tile sums
            if (h->useGraph && !h->timing) {
                if (!h->graph[in] && h->captureStages(in, 0, 4, &h->graph[in]) != SWARM_OK) return SWARM_E_CUDA;
                if (!cudaOk(h, cudaGraphLaunch(h->graph[in], h->stream), "graph launch")) return SWARM_E_CUDA;
                h->launches += perStep;
            } else {
                for (int st = 0; st < 4; ++st) {
                    if (h->timing && !cudaOk(h, cudaEventRecord(h->ev[st], h->stream), "event")) return SWARM_E_CUDA;
                    if (h->useGraph) {
                        if (!h->stageGraph[in][st] && h->captureStages(in, st, st + 1, &h->stageGraph[in][st]) != SWARM_OK)
                            return SWARM_E_CUDA;
                        if (!cudaOk(h, cudaGraphLaunch(h->stageGraph[in][st], h->stream), "graph launch")) return SWARM_E_CUDA;
                    } else {
                        const int rc = h->enqueueStages(in, st, st + 1);
                        if (rc != SWARM_OK) return rc;
                    }
                }
                if (h->timing && !cudaOk(h, cudaEventRecord(h->ev[4], h->stream), "event")) return SWARM_E_CUDA;
                if (h->useGraph) h->launches += perStep;
            }
        }
        if (h->metricRes && h->enqueueMetrics(in) != SWARM_OK) return SWARM_E_CUDA;
        h->readIdx ^= chunk & 1;
        s += chunk;
    }
    h->timesValid = false;
    return SWARM_OK;
}

int swarm_run_evacuation(SwarmHandle h, int max_steps, int32_t* active_out, SwarmEvacuation* out) {
    if (!h || !out || max_steps < 0) return SWARM_E_INVALID;
    if (!h->hasState) return h->fail(SWARM_E_STATE, "no state (upload one first)");
    constexpr int CHUNK = 256;   // steps between host checks; every step is counted on the device
    // What a step changes, saved at the start of every chunk: both state halves and, when on, the metrics'
    // accumulators. A chunk in which the crowd empties is rolled back and replayed up to that step, so the run stops
    // exactly there (the step is deterministic: the replay gives the same bits).
    std::vector<std::pair<void*, size_t>> live = {{h->state[0], size_t(h->n) * 32}, {h->state[1], size_t(h->n) * 32}};
    if (h->metricRes) {
        const size_t cells = size_t(h->metricRes) * size_t(h->metricRes);
        live.push_back({h->mCounters, sizeof(SwarmMetricCounters)});
        live.push_back({h->mEvac, size_t(h->capacity) * 4});
        live.push_back({h->mMass, cells * 8});
        live.push_back({h->mCells, cells * sizeof(SwarmMetricCell)});
    }
    for (const auto& l : h->choiceLive()) live.push_back(l);   // the exit choice's assignments and counts
    size_t saveBytes = 0;
    for (auto& l : live) saveBytes += (l.second + 255) / 256 * 256;
    uint32_t* dCounts = nullptr;
    char* dSave = nullptr;
    if (!cudaOk(h, cudaMalloc(&dCounts, (CHUNK + 1) * sizeof(uint32_t)), "evacuation counters")) return SWARM_E_OOM;
    if (!cudaOk(h, cudaMalloc(&dSave, saveBytes), "evacuation rollback copy")) { cudaFree(dCounts); return SWARM_E_OOM; }
    auto release = [&] { cudaFree(dCounts); cudaFree(dSave); };
    auto fail = [&](int code) { release(); return code; };
    auto copyLive = [&](bool save) {
        size_t off = 0;
        for (auto& l : live) {
            void* dst = save ? static_cast<void*>(dSave + off) : l.first;
            const void* src = save ? l.first : static_cast<const void*>(dSave + off);
            if (cudaMemcpyAsync(dst, src, l.second, cudaMemcpyDeviceToDevice, h->stream) != cudaSuccess) return false;
            off += (l.second + 255) / 256 * 256;
        }
        return true;
    };
    std::vector<uint32_t> counts(CHUNK + 1);
    std::vector<int32_t> series;
    int rc = SWARM_OK;
    int64_t launches = 0;
    // steps j = 0 .. c - 1 of a chunk, the active count after step j into dCounts[j]
    auto runChunk = [&](int c) -> int {
        if (!cudaOk(h, cudaMemsetAsync(dCounts, 0, size_t(c) * sizeof(uint32_t), h->stream), "evacuation counters"))
            return SWARM_E_CUDA;
        for (int j = 0; j < c; ++j) {
            const int r = stepImpl(h, 1);
            if (r != SWARM_OK) return r;
            swarm_gpu::launch_count_active(h->state[h->readIdx], h->n, dCounts + j, h->stream);
            launches += h->launches + 1;
        }
        if (!cudaOk(h, cudaMemcpyAsync(counts.data(), dCounts, size_t(c) * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                       h->stream), "count"))
            return SWARM_E_CUDA;
        return swarm_synchronize(h);
    };
    // the active agents before the first step
    if (!cudaOk(h, cudaMemsetAsync(dCounts, 0, sizeof(uint32_t), h->stream), "evacuation counters")) return fail(SWARM_E_CUDA);
    swarm_gpu::launch_count_active(h->state[h->readIdx], h->n, dCounts, h->stream);
    launches += 1;
    if (!cudaOk(h, cudaMemcpyAsync(counts.data(), dCounts, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream), "count") ||
        (rc = swarm_synchronize(h)) != SWARM_OK)
        return fail(rc != SWARM_OK ? rc : SWARM_E_CUDA);
    const int64_t initial = counts[0];
    int steps = 0;
    int64_t active = initial;
    while (steps < max_steps && active > 0) {
        const int c = std::min(CHUNK, max_steps - steps);
        const int readIdx = h->readIdx;
        const uint32_t metricStep = h->metricStep, choiceStep = h->choiceStep;
        if (!copyLive(true)) return fail(h->fail(SWARM_E_CUDA, "evacuation rollback copy"));
        if ((rc = runChunk(c)) != SWARM_OK) return fail(rc);
        int run = c;
        for (int j = 0; j < c; ++j)
            if (counts[size_t(j)] == 0) { run = j + 1; break; }
        if (run < c) {
            // the crowd emptied at step run of this chunk: back to the chunk's start, then exactly run steps
            if (!copyLive(false)) return fail(h->fail(SWARM_E_CUDA, "evacuation rollback copy"));
            h->readIdx = readIdx;
            h->metricStep = metricStep;
            h->choiceStep = choiceStep;
            if (!h->clearCounts()) return fail(h->fail(SWARM_E_CUDA, "clearing the counts"));
            if ((rc = runChunk(run)) != SWARM_OK) return fail(rc);
        }
        for (int j = 0; j < run; ++j) series.push_back(int32_t(counts[size_t(j)]));
        steps += run;
        active = counts[size_t(run - 1)];
    }
    release();
    SwarmEvacuation e{};
    e.steps = steps;
    e.initial_active = int32_t(initial);
    e.remaining = int32_t(active);
    int32_t* ts[3] = {&e.t50_step, &e.t90_step, &e.t100_step};
    const int pct[3] = {50, 90, 100};
    for (int q = 0; q < 3; ++q) {
        *ts[q] = -1;
        for (size_t t = 0; t < series.size(); ++t)
            if ((initial - series[t]) * 100 >= pct[q] * initial) { *ts[q] = int32_t(t + 1); break; }
    }
    e.t50_s = e.t50_step < 0 ? -1.0f : float(double(e.t50_step) * double(h->P.dt));
    e.t90_s = e.t90_step < 0 ? -1.0f : float(double(e.t90_step) * double(h->P.dt));
    e.t100_s = e.t100_step < 0 ? -1.0f : float(double(e.t100_step) * double(h->P.dt));
    *out = e;
    if (active_out) std::copy(series.begin(), series.end(), active_out);
    h->launches = launches;
    return SWARM_OK;
}

int swarm_step(SwarmHandle h, int steps) {
    if (!h) return SWARM_E_INVALID;
    if (!h->hasState) return h->fail(SWARM_E_STATE, "no state (upload one first)");
    if (steps < 0) return h->fail(SWARM_E_INVALID, "steps must be >= 0");
    return stepImpl(h, steps);
}

int swarm_step_host(SwarmHandle h, const float* in_boids, float* out_boids, int n, int steps) {
    if (!h || !in_boids || !out_boids) return SWARM_E_INVALID;
    if (n <= 0 || n > h->capacity) return h->fail(SWARM_E_INVALID, "agent count " + std::to_string(n) + " outside 1.." + std::to_string(h->capacity));
    if (steps < 0) return h->fail(SWARM_E_INVALID, "steps must be >= 0");
    if (n != h->n) h->dropGraphs();
    if (h->counted && !h->clearCounts()) return h->fail(SWARM_E_CUDA, "clearing the counts");
    h->n = n;
    h->hasState = true;
    if (!h->resetChoice()) return h->fail(SWARM_E_CUDA, "exit choice reset");
    const size_t bytes = size_t(n) * 32;
    // Pinned host buffers on the fused path: no copy operations. The first step's hash phase reads the input over the
    // coherent host link (into the device half it steps from), and the last step ends with its blocks copying the
    // result, in order, into the output. Pageable buffers, the per-phase path, or the exit choice (whose pass runs
    // before the kernel, on the device state): a copy each way.
    const float4* dIn = nullptr;
    float4* dOut = nullptr;
    if (h->fused && steps > 0 && !h->choiceExits) {
        cudaPointerAttributes ai{}, ao{};
        if (cudaPointerGetAttributes(&ai, in_boids) == cudaSuccess && ai.type == cudaMemoryTypeHost && ai.devicePointer &&
            cudaPointerGetAttributes(&ao, out_boids) == cudaSuccess && ao.type == cudaMemoryTypeHost && ao.devicePointer) {
            dIn = static_cast<const float4*>(ai.devicePointer);
            dOut = static_cast<float4*>(ao.devicePointer);
        }
        cudaGetLastError();   // (an unregistered pointer is not an error of this handle)
    }
    if (dIn && dOut) {
        h->hostIn = dIn;
        h->hostOut = dOut;
        *static_cast<volatile int*>(h->errHost) = swarm_gpu::ERR_PENDING;   // the last launch's last block sets it
        const int rc = stepImpl(h, steps, false);
        h->hostIn = nullptr;
        h->hostOut = nullptr;
        if (rc != SWARM_OK) return rc;
        // a barrier that gave up ends the launch before the output copy: the flag says so (read from the device when the
        // launch ended before it could write the mirror)
        return h->finishWithMirror();
    }
    // the read half only: the final pass writes every agent of the other half
    if (!cudaOk(h, cudaMemcpyAsync(h->state[h->readIdx], in_boids, bytes, cudaMemcpyHostToDevice, h->stream), "upload")) return SWARM_E_CUDA;
    const int rc = stepImpl(h, steps, false);
    if (rc != SWARM_OK) return rc;
    if (!cudaOk(h, cudaMemcpyAsync(out_boids, h->state[h->readIdx], bytes, cudaMemcpyDeviceToHost, h->stream), "download")) return SWARM_E_CUDA;
    return h->finishWithFlag();
}

int swarm_synchronize(SwarmHandle h) {
    if (!h) return SWARM_E_INVALID;
    if (!cudaOk(h, cudaStreamSynchronize(h->stream), "synchronize")) return SWARM_E_CUDA;
    int flag = 0;
    cudaMemcpy(&flag, h->errFlag, 4, cudaMemcpyDeviceToHost);
    return flag ? h->deviceError(flag) : SWARM_OK;
}

int swarm_get_grid(SwarmHandle h, uint32_t* grid_id, uint32_t* boid_id, int n) {
    if (!h || !grid_id || !boid_id) return SWARM_E_INVALID;
    if (n != h->n) return h->fail(SWARM_E_INVALID, "grid size mismatch");
    if (!cudaOk(h, cudaStreamSynchronize(h->stream), "sync")) return SWARM_E_CUDA;
    cudaMemcpy(grid_id, h->skey, size_t(n) * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(boid_id, h->sid, size_t(n) * 4, cudaMemcpyDeviceToHost);
    // the evacuated tail, in id order (CpuCrowdSim's stable counting sort)
    int first = n;
    while (first > 0 && grid_id[first - 1] == 0xFFFFFFFFu) --first;
    std::sort(boid_id + first, boid_id + n);
    return SWARM_OK;
}

int swarm_get_cells(SwarmHandle h, uint32_t* start_count, int n_cells) {
    if (!h) return SWARM_E_INVALID;
    if (!start_count) return h->ncells;
    if (n_cells != h->ncells) return h->fail(SWARM_E_INVALID, "cell count mismatch");
    if (!cudaOk(h, cudaStreamSynchronize(h->stream), "sync")) return SWARM_E_CUDA;
    return cudaOk(h, cudaMemcpy(start_count, h->cells, size_t(n_cells) * 8, cudaMemcpyDeviceToHost), "cells") ? SWARM_OK : SWARM_E_CUDA;
}

int swarm_get_contacts(SwarmHandle h, uint8_t* bits, int n) {
    if (!h || !bits) return SWARM_E_INVALID;
    if (n != h->n) return h->fail(SWARM_E_INVALID, "contacts size mismatch");
    if (!cudaOk(h, cudaStreamSynchronize(h->stream), "sync")) return SWARM_E_CUDA;
    return cudaOk(h, cudaMemcpy(bits, h->contacts, size_t(n), cudaMemcpyDeviceToHost), "contacts") ? SWARM_OK : SWARM_E_CUDA;
}

int swarm_stage_times(SwarmHandle h, SwarmStageTimes* out) {
    if (!h || !out) return SWARM_E_INVALID;
    if (!h->timing) return h->fail(SWARM_E_STATE, "timing is off (swarm_set_timing)");
    if (!h->timesValid && h->fused) {
        if (!cudaOk(h, cudaEventSynchronize(h->ev[4]), "timing")) return SWARM_E_CUDA;
        float total = 0;
        cudaEventElapsedTime(&total, h->ev[0], h->ev[4]);
        unsigned long long st[5] = {};
        cudaMemcpy(st, h->stamps, sizeof st, cudaMemcpyDeviceToHost);
        auto ms = [&](int a, int b) { return st[b] > st[a] ? float(double(st[b] - st[a]) * 1e-6) : 0.0f; };
        h->times = SwarmStageTimes{0.0f, ms(0, 1), 0.0f, ms(1, 2), ms(2, 3), ms(3, 4), total};
        h->timesValid = true;
    }
    if (!h->timesValid) {
        if (!cudaOk(h, cudaEventSynchronize(h->ev[4]), "timing")) return SWARM_E_CUDA;
        float sort = 0, pred = 0, proj = 0, fin = 0;
        cudaEventElapsedTime(&sort, h->ev[0], h->ev[1]);
        cudaEventElapsedTime(&pred, h->ev[1], h->ev[2]);
        cudaEventElapsedTime(&proj, h->ev[2], h->ev[3]);
        cudaEventElapsedTime(&fin, h->ev[3], h->ev[4]);
        h->times = SwarmStageTimes{0.0f, sort, 0.0f, pred, proj, fin, sort + pred + proj + fin};
        h->timesValid = true;
    }
    *out = h->times;
    return SWARM_OK;
}

int swarm_launch_count(SwarmHandle h, int64_t* out) {
    if (!h || !out) return SWARM_E_INVALID;
    *out = h->launches;
    return SWARM_OK;
}

}  // extern "C"
