// swarm_gb300.hpp -- header-only C++ host class over the C ABI (swarm_cuda.h), shaped like the reference's
// swarm::CpuCrowdSim (DedovSergei/swarm-crowd-simulation include/swarm/cpu_crowd_sim.hpp:30-169) and
// swarm::CrowdSim (include/swarm/crowd_sim.hpp:53-194): setState/upload, step, state, grid, cells, contacts,
// setProjectionIterations, setDriveTable. Errors become the reference's exception types (std::invalid_argument for a
// bad argument, std::runtime_error otherwise). Link with libswarm_gb300.so.
#pragma once

#include "swarm_cuda.h"

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace swarm_gb300 {

// The reference's GpuBoid (include/swarm/gpu_types.hpp:17-20)
struct Boid { float position[4]; float velocity[4]; };
static_assert(sizeof(Boid) == 32, "GpuBoid is 32 bytes");
struct GridInfo { uint32_t gridID, boidID; };
struct CellData { uint32_t startIndex, agentCount; };

class CudaCrowdSim {
public:
    // One simulation on the current CUDA device. `capacity`: the largest state it will hold.
    CudaCrowdSim(const SwarmParams& params, const SwarmVenue& venue, int capacity) {
        check(swarm_create(&params, &venue, capacity, &h_), "swarm_create");
    }
    ~CudaCrowdSim() { if (h_) swarm_destroy(h_); }
    CudaCrowdSim(const CudaCrowdSim&) = delete;
    CudaCrowdSim& operator=(const CudaCrowdSim&) = delete;

    static SwarmParams referenceParams() { SwarmParams p; swarm_params_reference(&p); return p; }
    static SwarmParams siParams() { SwarmParams p; swarm_params_si(&p); return p; }

    // CpuCrowdSim::setState / CrowdSim::upload: writes both state halves
    void setState(const std::vector<Boid>& boids) {
        check(swarm_upload_state(h_, &boids[0].position[0], int(boids.size())), "setState");
        n_ = int(boids.size());
    }
    void setAgentParams(const std::vector<float>& radius, const std::vector<float>& v0) {
        if (radius.size() != v0.size()) throw std::invalid_argument("setAgentParams: radius and v0 differ in size");
        check(swarm_set_agent_params(h_, radius.data(), v0.data(), int(radius.size())), "setAgentParams");
    }
    void step(int steps = 1) { check(swarm_step(h_, steps), "step"); }
    void setProjectionIterations(int k) { check(swarm_set_iterations(h_, k), "setProjectionIterations"); }
    // CpuCrowdSim::setDriveTable: e_goal of agent i is (*table)[i]; nullptr: the venue's direction
    void setDriveTable(const std::vector<float>* xy) {
        check(swarm_set_drive_table(h_, xy ? xy->data() : nullptr, xy ? int(xy->size() / 2) : 0), "setDriveTable");
    }
    void setGraph(bool on) { check(swarm_set_graph(h_, on ? 1 : 0), "setGraph"); }
    int numBoids() const { return n_; }

    std::vector<Boid> state() const {
        std::vector<Boid> out(static_cast<size_t>(n_));
        check(swarm_download_state(h_, &out[0].position[0], n_), "state");
        return out;
    }
    std::vector<GridInfo> grid() const {
        std::vector<uint32_t> g(static_cast<size_t>(n_)), b(static_cast<size_t>(n_));
        check(swarm_get_grid(h_, g.data(), b.data(), n_), "grid");
        std::vector<GridInfo> out(static_cast<size_t>(n_));
        for (size_t i = 0; i < out.size(); ++i) out[i] = {g[i], b[i]};
        return out;
    }
    std::vector<CellData> cells() const {
        const int nc = swarm_get_cells(h_, nullptr, 0);
        std::vector<CellData> out(static_cast<size_t>(nc));
        check(swarm_get_cells(h_, &out[0].startIndex, nc), "cells");
        return out;
    }
    std::vector<uint8_t> contacts() const {
        std::vector<uint8_t> out(static_cast<size_t>(n_));
        check(swarm_get_contacts(h_, out.data(), n_), "contacts");
        return out;
    }
    SwarmHandle handle() const { return h_; }

private:
    void check(int rc, const char* what) const {
        if (rc == SWARM_OK) return;
        char msg[512] = {0};
        if (h_) swarm_last_error(h_, msg, sizeof msg);
        const std::string text = std::string(what) + ": " + msg;
        if (rc == SWARM_E_INVALID) throw std::invalid_argument(text);
        throw std::runtime_error(text);
    }
    SwarmHandle h_ = nullptr;
    int n_ = 0;
};

}  // namespace swarm_gb300
