// Test infrastructure only: a C entry layer over the UNMODIFIED reference CPU step (swarm::CpuCrowdSim,
// src/cpu_crowd_sim.cpp of DedovSergei/swarm-crowd-simulation), compiled from the reference tree by
// oracle/Makefile into oracle/_ref/libswarm_ref.so. Nothing in the product links or loads it; the tests use
// it to pin the oracle restatement (oracle/swarm_oracle.cpp) and to generate golden fixtures.
//
// The reference's spawn and SDF loader go through loadSDFTexture3D (src/sdf.cpp:109-130), which also uploads an
// OpenGL texture. No GL context exists here, so the four GL entry points it calls are pointed at no-op
// functions before the call; the CPU copy of the volume (sdfVolumeCPU) is all the CPU step uses.

#include <swarm/cpu_crowd_sim.hpp>
#include <swarm/crowd_sim.hpp>
#include <swarm/metrics.hpp>
#include <swarm/sdf.hpp>
#include <swarm/venue.hpp>

#include <glad/glad.h>

// the seated venues' test scenarios (header-only harness code of the reference: the dense forced scenario's plans and
// drive directions) and this project's C ABI types (the export format of the layout and the navigation table)
#include <tools/venue_s.hpp>
#include <swarm/nav_field.hpp>
#include <swarm/exit_choice.hpp>
#include "../include/swarm_cuda.h"

#include <cstdint>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

namespace {

void APIENTRY noGenTextures(GLsizei n, GLuint* t) { for (GLsizei i = 0; i < n; ++i) t[i] = 1u + GLuint(i); }
void APIENTRY noBindTexture(GLenum, GLuint) {}
void APIENTRY noTexParameteri(GLenum, GLenum, GLint) {}
void APIENTRY noTexImage3D(GLenum, GLint, GLint, GLsizei, GLsizei, GLsizei, GLint, GLenum, GLenum, const void*) {}

std::string g_err;

struct RefSim {
    swarm::CpuCrowdSim sim;
    std::vector<swarm::GpuBoid> scratch;
    std::vector<glm::vec2> drive;   // the forced e_goal table (setDriveTable keeps a pointer to it)
};

swarm::CpuCrowdSim::SortMode sortMode(int m) {
    return m == 1 ? swarm::CpuCrowdSim::SortMode::GpuBitonic : swarm::CpuCrowdSim::SortMode::Counting;
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// Loads stadium.sdf into the reference's CPU copy (sampleSDF_CPU / sdfVolumeCPU). 0 on success.
int ref_load_sdf(const char* path) {
    glad_glGenTextures = noGenTextures;
    glad_glBindTexture = noBindTexture;
    glad_glTexParameteri = noTexParameteri;
    glad_glTexImage3D = noTexImage3D;
    return swarm::loadSDFTexture3D(path) != 0 ? 0 : -1;
}

// spawnBleacherCrowd(n, seed) (src/crowd_sim.cpp:601-645) into out[n * 8] (GpuBoid: pos.xyzw, vel.xyzw)
int ref_spawn_terrace(int n, unsigned seed, float* out) {
    try {
        const std::vector<swarm::GpuBoid> b = swarm::spawnBleacherCrowd(n, seed);
        std::memcpy(out, b.data(), b.size() * sizeof(swarm::GpuBoid));
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

// spawnSeatedCrowd(venueByName(name), n, load, seed) (src/crowd_sim.cpp:673-690)
int ref_spawn_seated(const char* venue, int n, double load, unsigned seed, float* out) {
    try {
        const std::vector<swarm::GpuBoid> b = swarm::spawnSeatedCrowd(swarm::venueByName(venue), n, load, seed);
        std::memcpy(out, b.data(), b.size() * sizeof(swarm::GpuBoid));
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

// CpuCrowdSim on venue `venue` ("terrace" | "S" | "M" | "L") with the venue's default model options
void* ref_create(const char* venue, int sort, int threads) {
    try {
        const swarm::Venue& v = swarm::venueByName(venue);
        std::vector<float> sdf = v.seated() ? std::vector<float>{} : swarm::sdfVolumeCPU();
        return new RefSim{ swarm::CpuCrowdSim(v, std::move(sdf), threads, sortMode(sort)), {}, {} };
    } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}

// CpuCrowdSim with explicit ModelOptions (include/swarm/exit_choice.hpp:82-90): exit_choice 0 nearest / 1 queue-aware,
// incline 0/1, stair 0 off / 1 empirical / 2 conservative
void* ref_create_opts(const char* venue, int sort, int threads, int exit_choice, int incline, int stair) {
    try {
        const swarm::Venue& v = swarm::venueByName(venue);
        std::vector<float> sdf = v.seated() ? std::vector<float>{} : swarm::sdfVolumeCPU();
        swarm::ModelOptions o;
        o.exitChoice = exit_choice ? swarm::ExitChoice::QueueAware : swarm::ExitChoice::Nearest;
        o.inclineSpeed = incline != 0;
        o.stairFlow = stair == 1 ? swarm::StairFlow::Empirical : stair == 2 ? swarm::StairFlow::Conservative : swarm::StairFlow::Off;
        return new RefSim{ swarm::CpuCrowdSim(v, o, std::move(sdf), threads, sortMode(sort)), {}, {} };
    } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}

// setDriveTable: e_goal of agent i = dirs[2i..2i+1] from the next step on; NULL: the venue's own goal
int ref_set_drive(void* h, const float* dirs, int n) {
    try {
        RefSim* r = static_cast<RefSim*>(h);
        if (!dirs) { r->sim.setDriveTable(nullptr); return 0; }
        r->drive.resize(size_t(n));
        std::memcpy(r->drive.data(), dirs, size_t(n) * sizeof(glm::vec2));
        r->sim.setDriveTable(&r->drive);
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

// A seated venue's layout in the C ABI's format, and its neighbour grid and exit test
int ref_seated_layout(const char* venue, SwarmSeatedLayout* out, int* grid_res, float* domain_min, float* domain_span,
                      float* exit_depth, float* exit_max_z) {
    try {
        const swarm::Venue& v = swarm::venueByName(venue);
        if (!v.seated()) { g_err = "not a seated venue"; return -1; }
        const swarm::SeatedLayout& L = v.layout;
        SwarmSeatedLayout o{};
        o.stand_front = L.standFront; o.row0 = L.row0; o.row_depth = L.rowDepth; o.clearway = L.clearway; o.rows = L.rows;
        o.conc_front = L.concFront; o.conc_back = L.concBack; o.outer_face = L.outerFace; o.landing_end = L.landingEnd;
        o.avenue_half = L.avenueHalf; o.lat0 = L.lat0; o.gangway_lo = L.gangwayLo; o.gangway_hi = L.gangwayHi;
        o.exit_lo = L.exitLo; o.exit_hi = L.exitHi; o.corner_inset = L.cornerInset; o.seat_inset = L.seatInset;
        o.face_margin = L.faceMargin; o.wall_above = L.wallAbove; o.wall_clear = L.wallClear;
        o.first_row = L.firstRow; o.row_rise = L.rowRise; o.seat_top = L.seatTop; o.barrier_top = L.barrierTop;
        o.concourse_z = L.concourseZ; o.wall_top = L.wallTop; o.rake = L.rake; o.max_band_steps = L.maxBandSteps;
        o.gangways = L.gangways;
        for (int i = 0; i < SWARM_SEATED_MAX_GANGWAYS; ++i) {
            o.gw_lo[i] = L.gwLo[size_t(i)]; o.gw_hi[i] = L.gwHi[size_t(i)];
            o.gw_row[i] = L.gwRow[size_t(i)]; o.gw_seated[i] = L.gwSeated[size_t(i)];
        }
        o.doors = L.doors;
        for (int i = 0; i < SWARM_SEATED_MAX_DOORS; ++i) { o.door_lo[i] = L.doorLo[size_t(i)]; o.door_hi[i] = L.doorHi[size_t(i)]; }
        o.corner_door_lo = L.cornerDoorLo;
        *out = o;
        *grid_res = v.gridRes; *domain_min = v.domainMin; *domain_span = v.domainSpan;
        *exit_depth = v.exitDepth; *exit_max_z = v.exitMaxZ;
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

// sim_params.hpp's incline and stair constants: V_STAIR_UP, V_STAIR_DOWN, INCLINE_INV_REF_SLOPE, T_HEADWAY,
// T_HEADWAY_STAIR_UP, T_HEADWAY_STAIR_DOWN, T_HEADWAY_STAIR_UP_CONSERVATIVE, T_HEADWAY_STAIR_DOWN_CONSERVATIVE
int ref_incline_constants(float* out8) {
    const float v[8] = {swarm::V_STAIR_UP, swarm::V_STAIR_DOWN, swarm::INCLINE_INV_REF_SLOPE, swarm::T_HEADWAY,
                        swarm::T_HEADWAY_STAIR_UP, swarm::T_HEADWAY_STAIR_DOWN, swarm::T_HEADWAY_STAIR_UP_CONSERVATIVE,
                        swarm::T_HEADWAY_STAIR_DOWN_CONSERVATIVE};
    std::memcpy(out8, v, sizeof v);
    return 0;
}

// The venue's navigation field as its GPU table (nav::gpuCells of nav::forVenue: built, or read from the cache
// directory SWARM_NAV_CACHE); returns the grid's res (cells per axis), writes its origin, cell and 1 / cell
int ref_nav_table(const char* venue, SwarmNavCell* out, int capacity, float* origin, float* cell, float* inv_cell) {
    try {
        const swarm::Venue& v = swarm::venueByName(venue);
        const swarm::nav::Field& f = swarm::nav::forVenue(v);
        const std::vector<swarm::GpuNavCell> cells = swarm::nav::gpuCells(f);
        if (out) {
            if (capacity < int(cells.size())) { g_err = "capacity"; return -1; }
            std::memcpy(out, cells.data(), cells.size() * sizeof(swarm::GpuNavCell));
        }
        *origin = f.grid.origin; *cell = f.grid.cell; *inv_cell = f.grid.invCell;
        return f.grid.res;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

// The queue-aware exit choice's candidate table of a seated venue (nav::choiceForVenue, src/exit_choice.cpp:445-474;
// built, or read from the cache directory SWARM_NAV_CACHE): per grid cell its index word into index_out (cells words,
// when non-null), the entries (GpuNavChoiceCell: 24 slot words, 12 distance words) into entries_out (when non-null,
// at most max_entries), meta = {exitCount, secondsPerUnit, distQuantum, invCapS[0 .. exitCount)}. Returns the entry
// count; *grid_res: the table grid's cells per axis.
long long ref_choice_table(const char* venue, uint32_t* index_out, long long cells, uint32_t* entries_out, long long max_entries,
                           float* meta, int* grid_res) {
    try {
        const swarm::Venue& v = swarm::venueByName(venue);
        const swarm::nav::ChoiceTable& t = swarm::nav::choiceForVenue(v);
        *grid_res = t.grid.res;
        meta[0] = float(t.exitCount);
        meta[1] = t.secondsPerUnit;
        meta[2] = t.distQuantum;
        for (int e = 0; e < t.exitCount; ++e) meta[3 + e] = t.invCapS[size_t(e)];
        if (index_out) {
            if (cells < (long long)t.index.size()) { g_err = "index capacity"; return -1; }
            std::memcpy(index_out, t.index.data(), t.index.size() * 4);
        }
        if (entries_out) {
            if (max_entries < (long long)t.entries.size()) { g_err = "entry capacity"; return -1; }
            std::memcpy(entries_out, t.entries.data(), t.entries.size() * sizeof(swarm::GpuNavChoiceCell));
        }
        return (long long)t.entries.size();
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

// The exit choice's state of a queue-aware CpuCrowdSim (cpu_crowd_sim.hpp:97-103): each agent's assigned exit,
// GpuChoiceCounters (132 words) and the choice step
int ref_choice_state(void* h, uint32_t* assign, int n, uint32_t* counters, uint32_t* step) {
    try {
        const swarm::CpuCrowdSim& s = static_cast<RefSim*>(h)->sim;
        const std::vector<uint32_t>& a = s.assignedExits();
        if (n < int(a.size())) { g_err = "capacity"; return -1; }
        std::memcpy(assign, a.data(), a.size() * 4);
        std::memcpy(counters, &s.choiceCounters(), sizeof(swarm::GpuChoiceCounters));
        *step = s.choiceStep();
        return int(a.size());
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

// The reference's own seated-venue functions, point by point (the harness's counterpart, same op codes):
// 0 seated::floorHeight | 1 cellKey | 2 sdfGrad | 3 wall | 4 stepUpScan | 5 floorSlope | 6 nav::goal (forVenue's field)
int ref_seated_eval(const char* venue, int op, int n, const float* in, float* out) {
    try {
        const swarm::Venue& v = swarm::venueByName(venue);
        const swarm::SeatedLayout& L = v.layout;
        const swarm::nav::Field* f = op == 6 ? &swarm::nav::forVenue(v) : nullptr;
        for (int i = 0; i < n; ++i) {
            switch (op) {
            case 0: out[i] = swarm::seated::floorHeight(L, glm::vec2(in[2 * i], in[2 * i + 1])); break;
            case 1: { const glm::vec2 k = swarm::seated::cellKey(L, glm::vec2(in[2 * i], in[2 * i + 1])); out[2 * i] = k.x; out[2 * i + 1] = k.y; break; }
            case 2: {
                const glm::vec4 g = swarm::seated::sdfGrad(L, glm::vec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]));
                out[4 * i] = g.x; out[4 * i + 1] = g.y; out[4 * i + 2] = g.z; out[4 * i + 3] = g.w;
                break;
            }
            case 3: {
                const glm::vec3 w = swarm::seated::wall(L, glm::vec3(in[4 * i], in[4 * i + 1], in[4 * i + 2]), in[4 * i + 3]);
                out[3 * i] = w.x; out[3 * i + 1] = w.y; out[3 * i + 2] = w.z;
                break;
            }
            case 4: {
                glm::vec2 nn;
                const float t = swarm::seated::stepUpScan(L, glm::vec2(in[5 * i], in[5 * i + 1]), glm::vec2(in[5 * i + 2], in[5 * i + 3]), in[5 * i + 4], nn);
                out[3 * i] = t; out[3 * i + 1] = nn.x; out[3 * i + 2] = nn.y;
                break;
            }
            case 5: out[i] = swarm::seated::floorSlope(L, glm::vec2(in[4 * i], in[4 * i + 1]), glm::vec2(in[4 * i + 2], in[4 * i + 3])); break;
            case 6: {
                const glm::vec2 e = swarm::nav::goal(*f, L, glm::vec3(in[3 * i], in[3 * i + 1], in[3 * i + 2]));
                out[2 * i] = e.x; out[2 * i + 1] = e.y;
                break;
            }
            default: return -1;
            }
        }
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

// The dense forced scenario of the reference's venue tests (tools/venue_s.hpp denseSetup): every seat occupied, padded
// with parked agents to a power of two; returns the agent count
int ref_dense_setup(const char* venue, float* boids, int capacity) {
    try {
        const swarm::Venue& v = swarm::venueByName(venue);
        const swarm::venue_s::Setup st = swarm::venue_s::denseSetup(v.layout);
        if (boids) {
            if (capacity < int(st.boids.size())) { g_err = "capacity"; return -1; }
            std::memcpy(boids, st.boids.data(), st.boids.size() * sizeof(swarm::GpuBoid));
        }
        return int(st.boids.size());
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

// Its drive table for a state (tools/venue_s.hpp driveTable over denseSetup's plans): out[2i..2i+1] = e_goal of agent i
int ref_dense_drive(const char* venue, const float* state, int n, float* out) {
    try {
        const swarm::Venue& v = swarm::venueByName(venue);
        static std::vector<swarm::venue_s::Plan> plans;
        static std::string plansOf;
        if (plansOf != venue) { plans = swarm::venue_s::denseSetup(v.layout).plans; plansOf = venue; }
        std::vector<swarm::GpuBoid> s(static_cast<size_t>(n));
        std::memcpy(s.data(), state, size_t(n) * sizeof(swarm::GpuBoid));
        std::vector<glm::vec2> t;
        swarm::venue_s::driveTable(v.layout, plans, s, t);
        std::memcpy(out, t.data(), t.size() * sizeof(glm::vec2));
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

void ref_destroy(void* h) { delete static_cast<RefSim*>(h); }

int ref_set_state(void* h, const float* boids, int n) {
    try {
        RefSim* r = static_cast<RefSim*>(h);
        r->scratch.resize(size_t(n));
        std::memcpy(r->scratch.data(), boids, size_t(n) * sizeof(swarm::GpuBoid));
        r->sim.setState(r->scratch);
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

int ref_set_iterations(void* h, int k) {
    try { static_cast<RefSim*>(h)->sim.setProjectionIterations(k); return 0; }
    catch (const std::exception& e) { g_err = e.what(); return -1; }
}

int ref_step(void* h, int steps) {
    try {
        RefSim* r = static_cast<RefSim*>(h);
        for (int i = 0; i < steps; ++i) r->sim.step();
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

int ref_get_state(void* h, float* out) {
    const auto& s = static_cast<RefSim*>(h)->sim.state();
    std::memcpy(out, s.data(), s.size() * sizeof(swarm::GpuBoid));
    return 0;
}

// grid(): the last step's sorted (gridID, boidID) pairs
int ref_get_grid(void* h, uint32_t* grid_id, uint32_t* boid_id) {
    const auto& g = static_cast<RefSim*>(h)->sim.grid();
    for (size_t i = 0; i < g.size(); ++i) { grid_id[i] = g[i].gridID; boid_id[i] = g[i].boidID; }
    return 0;
}

// cells(): (startIndex, agentCount) per cell; returns the cell count
int ref_get_cells(void* h, uint32_t* start_count, int capacity) {
    const auto& c = static_cast<RefSim*>(h)->sim.cells();
    const int n = int(c.size());
    for (int i = 0; i < n && i < capacity; ++i) { start_count[2 * i] = c[size_t(i)].startIndex; start_count[2 * i + 1] = c[size_t(i)].agentCount; }
    return n;
}

int ref_get_contacts(void* h, uint8_t* out) {
    const auto& c = static_cast<RefSim*>(h)->sim.contacts();
    std::memcpy(out, c.data(), c.size());
    return 0;
}

// timings(): hash, sort, cells, physics, total (ms, wall clock of the last step)
int ref_timings(void* h, double* out5) {
    const auto& t = static_cast<RefSim*>(h)->sim.timings();
    out5[0] = t.hash; out5[1] = t.sort; out5[2] = t.cells; out5[3] = t.physics; out5[4] = t.total;
    return 0;
}

int ref_num_threads(void* h) { return static_cast<RefSim*>(h)->sim.numThreads(); }

// The terrace venue's grid: gridRes, domainMin, domainSpan
int ref_venue_grid(const char* venue, int* grid_res, float* domain_min, float* domain_span, float* exit_depth, float* exit_max_z) {
    try {
        const swarm::Venue& v = swarm::venueByName(venue);
        *grid_res = v.gridRes; *domain_min = v.domainMin; *domain_span = v.domainSpan;
        *exit_depth = v.exitDepth; *exit_max_z = v.exitMaxZ;
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

// ---- safety metrics: MetricsReference (src/metrics.cpp:429-476), the CPU mirror of metrics_deposit/finalize.comp ----

// The terrace's metric cell table (computeMetricVenue, src/metrics.cpp:122): per cell thresholdMass[4], walkable m^2
int ref_metrics_terrace_cells(uint32_t* threshold_mass, float* walkable_m2, int capacity) {
    try {
        const swarm::metrics::MetricVenue mv = swarm::metrics::computeMetricVenue(swarm::sdfVolumeCPU());
        const std::vector<swarm::GpuMetricCellInfo> info = mv.cellInfo();
        const int n = int(info.size());
        for (int c = 0; c < n && c < capacity; ++c) {
            for (int k = 0; k < 4; ++k) threshold_mass[4 * c + k] = info[size_t(c)].thresholdMass[k];
            walkable_m2[c] = info[size_t(c)].walkableM2;
        }
        return n;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

void* ref_metrics_create(int n, const uint32_t* threshold_mass, int cells) {
    try {
        std::vector<swarm::GpuMetricCellInfo> info(size_t(cells), swarm::GpuMetricCellInfo{});
        for (int c = 0; c < cells; ++c)
            for (int k = 0; k < 4; ++k) info[size_t(c)].thresholdMass[k] = threshold_mass[4 * c + k];
        return new swarm::metrics::MetricsReference(n, std::move(info));
    } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
}
void ref_metrics_destroy(void* h) { delete static_cast<swarm::metrics::MetricsReference*>(h); }

int ref_metrics_record(void* h, const float* prev, const float* cur, int n) {
    try {
        std::vector<swarm::GpuBoid> a(static_cast<size_t>(n)), b(static_cast<size_t>(n));
        std::memcpy(a.data(), prev, size_t(n) * sizeof(swarm::GpuBoid));
        std::memcpy(b.data(), cur, size_t(n) * sizeof(swarm::GpuBoid));
        static_cast<swarm::metrics::MetricsReference*>(h)->record(a, b);
        return 0;
    } catch (const std::exception& e) { g_err = e.what(); return -1; }
}

// counters: 784 bytes (GpuMetricCounters); cells: 64 bytes each (GpuMetricCell); evac_step: n
int ref_metrics_read(void* h, void* counters, void* cells, uint32_t* evac_step) {
    auto* m = static_cast<swarm::metrics::MetricsReference*>(h);
    std::memcpy(counters, &m->counters, sizeof m->counters);
    std::memcpy(cells, m->cells.data(), m->cells.size() * sizeof(swarm::GpuMetricCell));
    std::memcpy(evac_step, m->evacStep.data(), m->evacStep.size() * sizeof(uint32_t));
    return 0;
}

}  // extern "C"
