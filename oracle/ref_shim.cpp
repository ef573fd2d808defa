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
        return new RefSim{ swarm::CpuCrowdSim(v, std::move(sdf), threads, sortMode(sort)), {} };
    } catch (const std::exception& e) { g_err = e.what(); return nullptr; }
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
