// ORACLE -- test infrastructure only (see swarm_oracle.cpp). C entry points of the CPU restatement.
#pragma once
#include "../include/swarm_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif
const char* oracle_last_error(void);
void* oracle_create(const SwarmParams* p, const SwarmVenue* v, int threads);
void oracle_destroy(void* h);
int oracle_set_state(void* h, const float* boids, int n);
int oracle_set_agent_params(void* h, const float* radius, const float* v0, int n);
int oracle_set_iterations(void* h, int k);
int oracle_set_threads(void* h, int threads);
int oracle_set_drive_table(void* h, const float* dirs, int n);
int oracle_set_exit_choice(void* h, int n_exits, int k, const float* fields, const float* inv_cap, const uint8_t* c_exit,
                           const float* c_dist);
int oracle_get_exit_choice(void* h, uint32_t* assigned, uint32_t* counters);
int oracle_step(void* h, int steps);
int oracle_get_state(void* h, float* out);
int oracle_get_grid(void* h, uint32_t* grid_id, uint32_t* boid_id);
int oracle_get_cells(void* h, uint32_t* start_count, int capacity);
int oracle_get_contacts(void* h, uint8_t* out);
int oracle_max_threads(void);
#ifdef __cplusplus
}
#endif
