/*
 * swarm_cuda.h -- C ABI of the GB300-native SWARM crowd step (libswarm_gb300.so).
 *
 * One handle = one simulation on one GPU: the agent state, the neighbour grid, the venue and a CUDA stream.
 * Every entry point returns SWARM_OK (0) or a negative status; swarm_last_error() gives the message.
 * Threads: handles share no state, so different handles may be driven from different host threads at once; the calls
 * on one handle must not overlap (as for the reference's CrowdSim object).
 * No C++ exception, no torch type and no CUDA type crosses this boundary (streams are passed as void*).
 *
 * Reference interface replaced (DedovSergei/swarm-crowd-simulation, paths within that project):
 *   class swarm::CrowdSim        include/swarm/crowd_sim.hpp:53-194  (GPU step / state API, OpenGL compute)
 *   class swarm::CpuCrowdSim     include/swarm/cpu_crowd_sim.hpp:30-169 (its CPU mirror)
 * Each declaration below names the member it stands in for.
 *
 * State format: the reference's GpuBoid (include/swarm/gpu_types.hpp:17-20), 8 floats per agent:
 *   position.xyz, position.w (1 = active, 0 = evacuated / parked), velocity.xyz, velocity.w (speed).
 * Agent ids are the indices into that array (the reference's boidID).
 */
#ifndef SWARM_CUDA_H
#define SWARM_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
enum {
    SWARM_OK = 0,
    SWARM_E_INVALID = -1,  /* bad argument (std::invalid_argument in the reference) */
    SWARM_E_CUDA = -2,     /* a CUDA call failed */
    SWARM_E_OOM = -3,      /* device allocation failed */
    SWARM_E_TIMEOUT = -4,  /* a bounded device-side wait gave up (the kernel returned instead of hanging) */
    SWARM_E_STATE = -5     /* call out of order (e.g. step before a state was uploaded) */
};

/* ---- venue kinds ---- */
enum {
    /* The reference's baked terrace (venue "terrace"): stadium.sdf (130^3 float32, [x][y][z] z fastest), the analytic
     * pitch fence and the egress router, model units, uniform body radius (include/swarm/sim_params.hpp). */
    SWARM_VENUE_STADIUM = 0,
    /* A plan venue on grids, SI units, per-agent radius and desired speed: a horizontal wall SDF, a geodesic
     * distance-to-exit field whose negative normalised gradient is the walking direction, an optional floor
     * heightfield and stair speed factors. The synthetic halls and the seated bowl are built as these. */
    SWARM_VENUE_GRID = 1,
    /* The reference's analytic seated venues (venues S, M and L: swarm::SeatedLayout, include/swarm/venue.hpp:99-138),
     * model units, uniform body: a closed-form heightfield of square-ring rows, gangway inclines, barrier, concourse and
     * walls, evaluated exactly (src/venue.cpp:411-908, shaders/venue_seated.glsl), the pitch fence of the terrace, and
     * e_goal from the reference's navigation field (its GpuNavCell table) or the drive table. */
    SWARM_VENUE_SEATED = 2
};

/* swarm::SeatedLayout (include/swarm/venue.hpp:99-138): the seated venue's breakpoints in model units, as the reference's
 * buildSeatedLayout computes them (src/venue.cpp:170-327) -- the values its shader preamble emits (VS_* literals). In the
 * folded frame lat = min(|x|, |y|), dep = max(|x|, |y|). */
#define SWARM_SEATED_MAX_GANGWAYS 8
#define SWARM_SEATED_MAX_DOORS 8
typedef struct SwarmSeatedLayout {
    float stand_front, row0, row_depth, clearway;
    int32_t rows;
    float conc_front, conc_back, outer_face, landing_end;
    float avenue_half, lat0, gangway_lo, gangway_hi, exit_lo, exit_hi, corner_inset;
    float seat_inset, face_margin, wall_above, wall_clear;
    float first_row, row_rise, seat_top, barrier_top, concourse_z, wall_top, rake;
    int32_t max_band_steps;
    int32_t gangways;                                   /* straight gangways per wing */
    float gw_lo[SWARM_SEATED_MAX_GANGWAYS], gw_hi[SWARM_SEATED_MAX_GANGWAYS];
    int32_t gw_row[SWARM_SEATED_MAX_GANGWAYS], gw_seated[SWARM_SEATED_MAX_GANGWAYS];
    int32_t doors;                                      /* concourse doors per wing */
    float door_lo[SWARM_SEATED_MAX_DOORS], door_hi[SWARM_SEATED_MAX_DOORS];
    float corner_door_lo;                               /* >= 1e8: no corner door */
} SwarmSeatedLayout;

/* The reference's GpuNavCell (include/swarm/gpu_types.hpp:42-46): one cell of a seated venue's navigation field -- the
 * anchor (the first vertex of the cell's shortest any-angle path to an exit), the distance, and info = the exit id
 * (bits 0-7) | SWARM_NAV_FIT | SWARM_NAV_REACHABLE. */
typedef struct SwarmNavCell { float anchor_x, anchor_y, dist; uint32_t info; } SwarmNavCell;
#define SWARM_NAV_FIT 0x100u
#define SWARM_NAV_REACHABLE 0x200u

/* Every model constant of the step (the reference's include/swarm/sim_params.hpp, including its folded constant
 * expressions). swarm_params_reference() fills the reference's values (model units, K = 32);
 * swarm_params_si() the SI preset of the grid venues (dt 0.05 s, K = 8, per-agent radius and v0). */
typedef struct SwarmParams {
    /* step */
    float dt;                     /* DT */
    int32_t proj_iterations;      /* PROJ_ITERATIONS: Jacobi sweeps per step, the last one in the final pass */
    int32_t perc_ring;            /* PERC_RING: cells searched to each side in the predict pass */
    int32_t uniform_body;         /* 1: every agent is BODY_RADIUS / V_MAX (stadium); 0: per-agent radius and v0 */
    /* body model */
    float body_radius;            /* BODY_RADIUS (uniform body; the default radius otherwise) */
    float body_diam, body_diam2;  /* BODY_DIAM, BODY_DIAM * BODY_DIAM (folded) */
    float r_sep, r_sep2;          /* R_SEP, R_SEP * R_SEP (uniform body) */
    float sep_margin;             /* per-agent body: the separation support of a pair is r_i + r_j + sep_margin */
    float k_sep;                  /* K_SEP */
    float r_perc2;                /* R_PERC * R_PERC */
    float v_max;                  /* V_MAX: the free speed (uniform body) and the |v_xy| clamp */
    float headway_rate;           /* 1 / T_HEADWAY */
    float relax_step;             /* exp(-DT / TAU_RELAX) */
    float tau_relax;              /* TAU_RELAX */
    float gravity_dt;             /* GRAVITY * DT */
    float proj_relax, proj_max_shift;   /* PROJ_RELAX, PROJ_MAX_SHIFT */
    float safe_eps;               /* SAFE_NORMALIZE_EPS */
    float stacked_xy2;            /* SEP_STACKED_XY2 */
    float hash_to_radians;        /* 2 pi / 2^32 */
    float goal_deadzone;          /* GOAL_DEADZONE */
    /* obstacle avoidance */
    float torso_height, obstacle_range, w_obs, obstacle_gain, obstacle_min_normal, obstacle_grad_h, obstacle_grad_scale;
    /* static contacts */
    int32_t feeler_count, wall_root_steps, wall_recast_steps, wall_passes;
    int32_t floor_search_cells, sweep_bisections, fence_ccd_bisections, pad0;
    float feeler_reach, plane_probe_reach, wall_recast_tol, wall_max_nz, centre_grad_min, floor_settle_reach;
    float feeler_dir[16][2], feeler_off[16][2], probe_off[16][2];
    /* step-up limit */
    float max_step_up, step_up_tol, step_up_floor_reach, step_up_sample;
    int32_t step_up_bisections, step_up_max_samples, step_up_slide_tries, pad1;
    float step_up_slide[3][2];
    /* analytic pitch fence (stadium) */
    float fence_center[2], fence_half_mid[2], fence_half_thk_coll;
    /* egress router (stadium) */
    float avenue_half, walkway_min, walkway_max, walkway_centre, aisle_max, aisle_centre;
    float avenue_target_depth, pitch_recovery_depth;
    float park_coord;             /* PARK_COORD */
    /* metrics (fixed-point cloud-in-cell density; include/swarm/metrics.hpp) */
    float metric_cells_per_unit;  /* metric cells per length unit */
    float metric_speed_scale;     /* m/s per speed unit */
    float r_pair_max;             /* per-agent body: the largest radius any agent may have (bounds the search disk) */
    /* incline speed and stair spacing on seated venues (sim_params.hpp:429-480): V_STAIR_UP, V_STAIR_DOWN,
     * 1 / INCLINE_REF_SLOPE, T_HEADWAY (model units) */
    float v_stair_up, v_stair_down, incline_inv_ref_slope, t_headway;
    float pad2[1];
} SwarmParams;

/* The venue: the neighbour grid, the exit test, and the static fields of its kind. Host pointers; swarm_create
 * copies them to the device. */
typedef struct SwarmVenue {
    int32_t kind;                 /* SWARM_VENUE_* */
    int32_t grid_res_x, grid_res_y;   /* neighbour (hash) grid cells per axis */
    int32_t n_exits;              /* exits listed in exit_boxes (grid venues; metrics) */
    float domain_min_x, domain_min_y, domain_span_x, domain_span_y;   /* the hash grid's extent */
    /* exit test: an agent is parked (evacuated) when it leaves [exit_lo, exit_hi] below exit_max_z, or the domain.
     * Stadium: max(|x|, |y|) > exit_hi_x (EXIT_DEPTH) below exit_max_z (EXIT_MAX_Z). */
    float exit_lo_x, exit_lo_y, exit_hi_x, exit_hi_y, exit_max_z;
    /* stadium: the baked volume */
    const float* sdf;             /* sdf_res^3 floats */
    int32_t sdf_res;
    float sdf_origin[3];          /* SDF_ORIGIN: world position of sample index 1 */
    float sdf_spacing;            /* SDF_SPACING */
    /* grid venues: node (i, j) of every field sits at origin + (i, j) * h; arrays x fastest */
    const float* wall_sdf;        /* horizontal signed distance to the walls (< 0 inside a wall) */
    int32_t wall_nx, wall_ny;
    float wall_origin_x, wall_origin_y, wall_h;
    const float* nav_dist;        /* geodesic distance to the nearest exit (walls: a large value) */
    int32_t nav_nx, nav_ny;
    float nav_origin_x, nav_origin_y, nav_h;
    const float* floor_height;    /* optional (NULL: a flat floor at z = 0), on the wall grid */
    const float* speed_factor;    /* optional (NULL: 1), on the wall grid: the desired-speed factor (stairs) */
    const float* exit_boxes;      /* n_exits x (lo_x, lo_y, hi_x, hi_y): the metric's exit attribution */
    /* metrics: the 1 m floor grid, metric_res^2 cells centred on metric_center */
    int32_t metric_res;
    float metric_center_x, metric_center_y;
    /* grid venues, optional: nav_nx x nav_ny bytes, nonzero at the nodes beyond an exit. When set, an agent is
     * parked when the nav node nearest to it is an exit node (or it leaves the domain) instead of by the exit
     * rectangle: exits anywhere in the plan, such as vomitories inside a seating bowl. */
    const uint8_t* exit_mask;
    /* seated venues (SWARM_VENUE_SEATED): the layout; the navigation field (nav_res x nav_res cells, x fastest, cell
     * (i, j) covering origin + [i, i + 1) x cell: nav::Grid, include/swarm/nav_field.hpp:69-79; NULL: e_goal comes from
     * the drive table alone, zero without one); the model options (ModelOptions, include/swarm/exit_choice.hpp:82-90):
     * incline_speed = the free speed by the slope along e_goal, stair_headway = the headway time gap by the slope, with
     * stair_t_up / stair_t_down its values on a full-slope incline (T_HEADWAY_STAIR_UP / _DOWN, model time) */
    const SwarmSeatedLayout* seated;
    const SwarmNavCell* nav_cells;
    int32_t nav_res;
    float nav_grid_origin, nav_grid_cell, nav_grid_inv_cell;
    int32_t incline_speed, stair_headway;
    float stair_t_up, stair_t_down;
} SwarmVenue;

typedef struct SwarmSim* SwarmHandle;

/* Per-stage device time of the last timed step, milliseconds (CpuCrowdSim::StageTimesMs,
 * include/swarm/cpu_crowd_sim.hpp:76; CrowdSim::readTimings, src/crowd_sim.cpp:449-478). */
typedef struct SwarmStageTimes {
    float hash, sort, cells, predict, project, final_pass, total;
} SwarmStageTimes;

/* ---- parameters ---- */
/* sim_params.hpp's values, folded as the reference folds them (include/swarm/sim_params.hpp:28-54, 499-512). */
int swarm_params_reference(SwarmParams* out);
/* The SI preset of the grid venues: dt 0.05 s, K = 8 sweeps, tau 0.5 s, per-agent radius and v0. */
int swarm_params_si(SwarmParams* out);

/* ---- lifecycle ----
 * swarm_create: CrowdSim(shaderDir, numBoids, venue) (src/crowd_sim.cpp:96-202) / CpuCrowdSim(venue, sdf)
 *   (src/cpu_crowd_sim.cpp:918-927). n_capacity: the agent buffer size (no power-of-two rule: the key sort has none). */
int swarm_create(const SwarmParams* params, const SwarmVenue* venue, int n_capacity, SwarmHandle* out);
int swarm_destroy(SwarmHandle h);
/* Batched instances: m independent grid venues (no floor heights or speed factors) with counts[i] agents each, packed
 * into one handle. The state is every instance's agents one after another (instance i's first agent follows the
 * counts before it); each instance keeps its own hash grid, in one shared key space, so one sort and one step cover
 * them all and no instance sees another's agents: each instance's result is bit-identical to running it alone.
 * Every other entry point works on the batch as on one simulation (metrics excepted). */
int swarm_batch_create(const SwarmParams* params, const SwarmVenue* venues, const int* counts, int m, SwarmHandle* out);
/* Optional: run on the caller's stream (a cudaStream_t) instead of the handle's own. */
int swarm_set_stream(SwarmHandle h, void* cuda_stream);
int swarm_last_error(SwarmHandle h, char* buf, int len);

/* ---- state I/O ----
 * swarm_upload_state: CrowdSim::upload (src/crowd_sim.cpp:285-309) / CpuCrowdSim::setState. boids: n x 8 floats
 *   (GpuBoid). Sets the active agent count to n (<= capacity). Host memory. */
int swarm_upload_state(SwarmHandle h, const float* boids, int n);
/* The latest state, n x 8 floats (CpuCrowdSim::state(); CrowdSim::currentStateBuffer readback). */
int swarm_download_state(SwarmHandle h, float* boids, int n);
/* Per-agent radius and desired speed (grid venues): n floats each. Default: body_radius and v_max. */
int swarm_set_agent_params(SwarmHandle h, const float* radius, const float* v0, int n);
/* Device-resident variants: pointers to device memory on the handle's device, same layouts. */
int swarm_upload_state_device(SwarmHandle h, const float* d_boids, int n);
int swarm_download_state_device(SwarmHandle h, float* d_boids, int n);

/* ---- stepping ----
 * swarm_step: `steps` x CrowdSim::step (src/crowd_sim.cpp:316-412) = hash, key sort, cell ranges + gather,
 *   predict, K - 1 Jacobi sweeps, final pass; asynchronous on the handle's stream. */
int swarm_step(SwarmHandle h, int steps);
/* One call for callers holding the state in host memory: in_boids (n x 8 floats) into the device state, `steps`
 * steps, the result into out_boids, and waits for it. With pinned (page-locked, device-mapped) buffers and the fused
 * step there are no copy operations: the first step's hash phase reads in_boids over the coherent host link, and the
 * last step's kernel ends by writing its result into out_boids (the device state holds it too); otherwise (or with
 * the exit choice on) one copy each way. in_boids may equal out_boids. Like swarm_synchronize it reads the device
 * error flag before it returns: SWARM_E_TIMEOUT when a grid barrier gave up (out_boids then holds no result). */
int swarm_step_host(SwarmHandle h, const float* in_boids, float* out_boids, int n, int steps);
/* CpuCrowdSim::setProjectionIterations / CrowdSim::setProjectionIterations (src/crowd_sim.cpp:480-483). */
int swarm_set_iterations(SwarmHandle h, int k);
/* CpuCrowdSim::setDriveTable (include/swarm/cpu_crowd_sim.hpp:114): e_goal of agent i is dirs[2i..2i+1];
 * NULL restores the venue's router / navigation field. */
int swarm_set_drive_table(SwarmHandle h, const float* dirs, int n);
/* Captures one step in a CUDA graph and replays it (1) or launches kernel by kernel (0, the default). */
int swarm_set_graph(SwarmHandle h, int enabled);
/* 1 (the default): each step is one persistent cooperative kernel whose phases are separated by grid barriers (the
 * grid is sized to stay resident); 0: one kernel per phase (hash, scan x2, scatter, rank + gather, predict, K - 1
 * sweeps, final), replayed from CUDA graphs when swarm_set_graph is on. Both give the same bits. */
int swarm_set_fused(SwarmHandle h, int enabled);
/* The launch configuration: the fused persistent kernel (fused = 1) with `threads` per block (0: the state size over
 * the SMs, rounded up to a warp, 128..512, or 128..1024 for a batch; else 64..512, 64..1024 for a batch, rounded up to
 * a warp; below 64 is SWARM_E_INVALID) and at most `blocks_per_sm` blocks per SM (0: as many as fit; fewer blocks
 * mean more agents per thread), or one kernel per phase (fused = 0: one Jacobi sweep per launch). steps_per_launch
 * (fused only): the steps of one swarm_step call that one persistent launch runs, with one more grid barrier between
 * steps (0: all of them; 1: a launch per step); steps with the exit choice, the metrics or stage timing on take a
 * launch each. Every configuration gives the same bits. */
typedef struct SwarmTuning { int32_t fused, threads, blocks_per_sm; float ms_per_step; int32_t steps_per_launch; } SwarmTuning;
int swarm_set_tuning(SwarmHandle h, const SwarmTuning* tuning);
/* Times `steps` steps of each candidate configuration from the current state (restored after every trial and at the
 * end), keeps the fastest in force and returns it. The results of every configuration are the same bits. */
int swarm_autotune(SwarmHandle h, int steps, SwarmTuning* best);
/* Failure-path test: the next fused step's first grid barrier waits for one block more than the launch has, runs
 * out its 1 s limit, records the timeout and ends the launch early; the next swarm_synchronize (or download)
 * returns SWARM_E_TIMEOUT and the handle stays usable. For tests only. */
int swarm_test_barrier_timeout(SwarmHandle h);
int swarm_synchronize(SwarmHandle h);

/* ---- inspection (the reference's parity tests read these) ----
 * swarm_get_grid: CpuCrowdSim::grid() -- the last step's sorted (gridID, boidID) pairs, n each. */
int swarm_get_grid(SwarmHandle h, uint32_t* grid_id, uint32_t* boid_id, int n);
/* CpuCrowdSim::cells(): (startIndex, agentCount) per cell, 2 x n_cells; returns the cell count if the buffer is NULL. */
int swarm_get_cells(SwarmHandle h, uint32_t* start_count, int n_cells);
/* CpuCrowdSim::contacts(): the ContactBits per agent of the last step. */
int swarm_get_contacts(SwarmHandle h, uint8_t* bits, int n);
/* Records CUDA events around the stages of every following step (0: off, the default); swarm_stage_times waits for
 * and returns the last step's stage times. */
int swarm_set_timing(SwarmHandle h, int enabled);
int swarm_stage_times(SwarmHandle h, SwarmStageTimes* out);
/* Kernel launches the last swarm_step issued (evidence for benchmarks). */
int swarm_launch_count(SwarmHandle h, int64_t* out);

/* ---- synthetic venues and spawns (host code; inputs of the step, built once) ----
 * A rectangular hall centred on the origin: interior size_x x size_y metres, walls of wall_thickness around it with
 * door gaps, the exit line exit_depth beyond the walls' outer faces (agents past it are evacuated), a margin of open
 * ground around that. The walls' horizontal SDF is exact (boxes); the navigation field is the first-order fast-marching
 * geodesic distance, through the free nodes, to the free nodes beyond the exit line. */
typedef struct SwarmHallSpec {
    float size_x, size_y;         /* interior, metres */
    float wall_thickness;         /* metres */
    float exit_depth;             /* exit line beyond the walls' outer faces */
    float margin;                 /* open ground beyond the exit line */
    float wall_h, nav_h, cell;    /* wall SDF spacing (0.05), nav spacing (0.1), hash cell (0.5) */
    int32_t n_doors;              /* <= 8 */
    int32_t door_wall[8];         /* 0: the -x wall, 1: +x, 2: -y, 3: +y */
    float door_center[8];         /* along the wall, from the wall's midpoint */
    float door_width[8];
} SwarmHallSpec;

/* Fills every scalar of *venue (grid sizes, origins, domain, exit test) and leaves its array pointers NULL; the
 * array sizes are wall_nx * wall_ny and nav_nx * nav_ny floats, and 4 * n_exits for the exit boxes. */
int swarm_hall_layout(const SwarmHallSpec* spec, SwarmVenue* venue);
/* Fills the arrays of a layout made by swarm_hall_layout (caller-allocated). */
int swarm_hall_fields(const SwarmHallSpec* spec, const SwarmVenue* venue, float* wall_sdf, float* nav_dist, float* exit_boxes);

/* A seated bowl (the generated venue of the seated-bowl workload): `sectors` straight blocks of `rows` rows x `seats`
 * seats around a regular polygon, rising `rise` per row of depth `row_pitch`; each row is a tread between thin walls
 * (its front and back edges; the first row opens onto a flat cross-aisle along the pitch wall), so agents walk
 * along their row to the gangways between blocks; gangways are stairs of rise / 2 steps (speed factor stair_speed)
 * from the cross-aisle up to a flat concourse of depth concourse behind the top row; a vomitory (an exit portal vomitory_width wide) lies across every gangway at row vomitory_row;
 * perimeter_exits gaps of perimeter_exit_width in the concourse's outer wall, evenly spaced, lead out. The floor
 * heightfield and the speed factors are on the wall grid; the nav field is the speed-weighted travel distance to the
 * nearest exit (one plan-view field: the levels never overlap in plan). Its wall nodes (walls and their clearance)
 * within 1 m of a reached node hold the nearest reached node's value + 3 per metre of distance, so that e_goal beside
 * a wall keeps the route's direction with a push away from the wall; farther wall nodes and free nodes no exit
 * reaches hold the largest reached value + 10 m. All lengths in metres. */
typedef struct SwarmBowlSpec {
    int32_t sectors, rows, seats;       /* 32, 32, 62 */
    float seat_width, row_pitch, rise;  /* 0.5, 0.8, 0.4 */
    float gangway;                      /* width at the pitch wall (the gap between blocks widens upward): 1.2 */
    float vomitory_width;               /* 2.4 */
    int32_t vomitory_row;               /* 16 (0-based) */
    int32_t perimeter_exits;            /* 8 */
    float perimeter_exit_width;         /* 4 */
    float concourse;                    /* 4 */
    float aisle;                        /* the cross-aisle in front of the first row (the pitch wall beyond it): 1.2 */
    float stair_speed;                  /* 0.6 */
    float clearance;                    /* the nav field treats nodes this close to a wall as walls: 0.25 (the
                                           largest body radius) */
    float wall_h, nav_h, cell;          /* 0.05, 0.1, 0.5 */
} SwarmBowlSpec;
/* Fills every scalar of *venue; array sizes as swarm_hall_layout, plus the exit mask (nav_nx * nav_ny bytes) and the
 * floor heights and speed factors (wall_nx * wall_ny floats each); n_exits = sectors + perimeter_exits. */
int swarm_bowl_layout(const SwarmBowlSpec* spec, SwarmVenue* venue);
/* Fills the arrays of a layout made by swarm_bowl_layout (caller-allocated); exit_boxes: each exit's bounding box. */
int swarm_bowl_fields(const SwarmBowlSpec* spec, const SwarmVenue* venue, float* wall_sdf, float* nav_dist,
                      float* floor_height, float* speed_factor, uint8_t* exit_mask, float* exit_boxes);
/* ---- the navigation field solver ----
 * The first-order fast-marching travel distance (the nav_dist of every grid venue above) on an nx x ny grid of spacing
 * h: kind per node 0 free, 1 source (distance 0), 3 wall; speed per node (NULL: 1) divides the local step h. Walls and
 * unreached nodes get the largest reached distance + 10 m. The host builders use fast marching on the CPU unless
 * swarm_set_nav_solver(SWARM_NAV_GPU) selected the GPU solver, which gives the same floats node for node (the fixed
 * point of the same FP64 update). No counterpart in the reference (its seated venues build Lazy Theta* fields on the
 * CPU, src/nav_field.cpp:268-344). */
typedef struct SwarmNavFieldStats {
    int32_t passes;       /* tile passes run (launched in groups of 8) */
    int32_t tiles;        /* 32 x 32-node tiles of the grid */
    int64_t tile_runs;    /* tile relaxations over all passes */
    float ms;             /* wall-clock time of the call, allocation, uploads and downloads included */
    float ms_solve;       /* the passes alone (CUDA events) */
} SwarmNavFieldStats;
enum { SWARM_NAV_CPU = 0, SWARM_NAV_GPU = 1 };
int swarm_nav_field_gpu(int nx, int ny, double h, const uint8_t* kind, const float* speed, float* out,
                        SwarmNavFieldStats* stats);
int swarm_nav_field_cpu(int nx, int ny, double h, const uint8_t* kind, const float* speed, float* out);
/* The solver the venue builders use from now on (process-wide); returns the previous one, or SWARM_E_INVALID. */
int swarm_set_nav_solver(int solver);

/* ---- queue-aware exit choice (the reference's ExitChoice::QueueAware: physics.comp PHYSICS_PASS 0,
 * nav::choiceStep, src/exit_choice.cpp:580-790; constants include/swarm/sim_params.hpp:395-427) ----
 * Every agent holds an assigned exit and steers on that exit's own distance field; it estimates its time to leave
 * through each candidate exit e of its cell, E_e = d_e / V_FREE + A_e x 60 / (w_e J) seconds (d_e the cell's walking
 * distance to e, A_e the agents assigned to e in nearer 0.5 m distance bins, w_e the clear width, J = 83.6 persons per
 * metre per minute). Every 3 s of simulated time all agents re-evaluate on the same counts: an agent may switch to its
 * best candidate if that gains more than max(10 % of E_current, 5 s), and per exit at most max(1, 10 % of its
 * assigned agents) switch, the largest gains first (1 s gain bins). An agent whose exit is no candidate of its cell
 * takes the best candidate at once. Integer histograms and counts throughout: deterministic.
 * Exit types of the candidate rule: every cell's candidates hold its 2 nearest exits of type 0 (avenues: a bowl's
 * vomitories) and its nearest of type 1 (doors: a bowl's perimeter exits, a hall's doors), then the nearest others. */
#define SWARM_CHOICE_MAX_EXITS 63
#define SWARM_CHOICE_MAX_CANDIDATES 24
#define SWARM_CHOICE_EMPTY 0xFF          /* an empty candidate slot */
#define SWARM_CHOICE_NONE 0xFFFFFFFFu    /* an agent with no exit assigned yet */
typedef struct SwarmExitChoiceSpec {
    int32_t n_exits;              /* 1 .. SWARM_CHOICE_MAX_EXITS */
    int32_t candidates;           /* per cell, 1 .. SWARM_CHOICE_MAX_CANDIDATES */
    const float* fields;          /* n_exits x nav_nx x nav_ny: each exit's walking distance on the venue's nav grid */
    const float* width_m;         /* n_exits: clear widths, metres */
    const uint8_t* type;          /* n_exits: 0 avenue, 1 door */
} SwarmExitChoiceSpec;
/* Per-exit distance fields of the generated venues, solved as their nav_dist (same walls, speeds, solver) with one
 * exit's sources each (the other exits' sources blocked); fields: n_exits x nav_nx x nav_ny floats, width_m and type:
 * n_exits each (halls: n_doors doors of type 1; bowls: the sectors' vomitories, type 0, then the perimeter exits;
 * a bowl's fields fill their wall band as its nav_dist does, each from its own reached nodes). */
int swarm_hall_exit_fields(const SwarmHallSpec* spec, const SwarmVenue* venue, float* fields, float* width_m, uint8_t* type);
int swarm_bowl_exit_fields(const SwarmBowlSpec* spec, const SwarmVenue* venue, float* fields, float* width_m, uint8_t* type);
/* The candidate table on the venue's hash cells (grid_res_x x grid_res_y cells, `candidates` slots each): per cell the
 * reachable nav node nearest its centre stands for it; the slots hold exits (SWARM_CHOICE_EMPTY: none) and their
 * distances there, ascending (ties: the lower exit id). Host code; swarm_set_exit_choice builds the same table. */
int swarm_exit_choice_table(const SwarmVenue* venue, const SwarmExitChoiceSpec* spec, uint8_t* exits, float* dists);
/* Queue-aware exit choice on (spec) or off (NULL: e_goal from the venue's nearest-exit field, the default). Grid venues,
 * one instance; the handle's choice restarts (no exit assigned, step 0) here and at every state upload. */
int swarm_set_exit_choice(SwarmHandle h, const SwarmExitChoiceSpec* spec);
/* The assigned exit of each agent (SWARM_CHOICE_NONE: none yet) and the counters since the choice restarted:
 * evaluations, eligible agents, switches, forced choices (4 values; either pointer may be NULL). */
int swarm_get_exit_choice(SwarmHandle h, uint32_t* assigned, int n, uint32_t* counters);

/* The seated venues' queue-aware exit choice on the reference's own candidate table (nav::ChoiceTable,
 * include/swarm/exit_choice.hpp:146-168, as nav::choiceForVenue builds or caches it, src/exit_choice.cpp:445-474; the
 * choice pass nav::choiceStep :683-790, e_goal nav::choiceGoal :568-578 = physics.comp navChoiceGoal). The table lives
 * on the navigation field's grid: per cell an index word (SWARM_CHOICE_INDEX_FIT: the cell's class; the low bits: its
 * entry + 1, 0 without candidates) and, per entry, the reference's GpuNavChoiceCell: 24 slots (anchor cell index bits
 * 0-24, exit id bits 25-30 (63: empty), the class bit 31) and the candidates' walking distances in 16-bit quanta (two
 * a word; 0xFFFF: empty). The stages are those of swarm_set_exit_choice on the table's numbers: E = q x quantum x
 * seconds_per_unit + A x inv_cap_s[e], the queue ahead's bins q >> 6. */
#define SWARM_CHOICE_INDEX_FIT 0x80000000u
#define SWARM_CHOICE_INDEX_MASK 0x7FFFFFFFu
typedef struct SwarmNavChoiceCell {
    uint32_t slot[24];
    uint32_t dist[12];
} SwarmNavChoiceCell;
typedef struct SwarmSeatedChoiceSpec {
    int32_t n_exits;              /* 1 .. SWARM_CHOICE_MAX_EXITS (the table's exit count) */
    int32_t grid_res;             /* the table's grid: the venue's navigation grid (SwarmVenue::nav_res) */
    const uint32_t* index;        /* grid_res^2 index words, x fastest */
    const SwarmNavChoiceCell* entries;
    int64_t n_entries;
    const float* inv_cap_s;       /* n_exits: seconds per queued agent, 60 / (w J) (nav::setChoiceCapacities) */
    float seconds_per_unit;       /* seconds of walking per model unit (CHOICE_S_PER_UNIT) */
    float dist_quantum;           /* the distances' quantum, model units (2^-12) */
    int32_t choice_steps;         /* steps between evaluations (the reference's CHOICE_STEPS: 17 at its DT) */
} SwarmSeatedChoiceSpec;
/* Queue-aware exit choice on a seated venue (spec) or off (NULL). The table is checked (sizes, every index word's
 * entry within n_entries, every slot's exit < n_exits or empty, every anchor inside the grid) and copied to the
 * device; the choice restarts (no exit assigned, step 0) here and at every state upload. swarm_get_exit_choice reads
 * its assignments and counters. */
int swarm_set_seated_choice(SwarmHandle h, const SwarmSeatedChoiceSpec* spec);

/* One agent per seat (sectors x rows x seats, by sector, row, seat) at the seat centre jittered U(-jitter, jitter)
 * per axis, on the floor (z = floor + radius), at rest; radius and desired speed as swarm_spawn_lattice. */
int swarm_spawn_bowl(const SwarmBowlSpec* spec, float jitter, uint64_t seed, float r_lo, float r_hi, float v_mean,
                     float v_sd, float v_lo, float v_hi, float* boids, float* radius, float* v0);

/* A jittered lattice of nx x ny agents (row-major, the first n of them) at `spacing`, centred on (cx, cy), resting on
 * the floor (z = radius), at rest. Jitter U(-jitter, jitter) per axis, radius U[r_lo, r_hi], desired speed
 * N(v_mean, v_sd) clipped to [v_lo, v_hi]; seeded, identical on every platform (splitmix64 + Box-Muller in double).
 * boids: n x 8 floats (GpuBoid), radius and v0: n floats each. */
int swarm_spawn_lattice(int nx, int ny, int n, float spacing, float cx, float cy, float jitter, uint64_t seed,
                        float r_lo, float r_hi, float v_mean, float v_sd, float v_lo, float v_hi,
                        float* boids, float* radius, float* v0);

/* ---- the key sort without device allocation ----
 * No counterpart in the reference. For callers that cannot allocate device memory while they run: a plug-in step in
 * a host application's frame loop (cudaMalloc / cudaFree may synchronise the whole device, and the host owns the
 * memory budget), or a deployment that fixes its footprint at start-up. Sorts one state already in device memory --
 * d_boids, n x 8 floats, 16-byte aligned -- by cell over the given hash grid, exactly as the step's own sort, and
 * writes the sorted pairs (d_grid_id, d_boid_id: n each) and the cell table (d_cells: 2 x grid_res_x x grid_res_y) to
 * the caller's device arrays. Its working memory is a fixed array compiled into this library (about 1.8 MB per GPU
 * that loads it, held until exit): at most 65536 agents and 131072 cells; larger sizes or a misaligned state return
 * SWARM_E_INVALID. It calls no allocator. The first call on a device looks up the array's address with that device
 * current and keeps it (make that first call before any stream capture); after a cudaDeviceReset the address is
 * gone, so do not call it on that device again in the same process. Returns when its work on `stream` is done: SWARM_E_CUDA if a launch failed or the kernels met a slot
 * out of range. All calls share the array: calls that overlap on the GPU (from several host threads) race and can
 * give such an error, so order them. */
int swarm_sort_grid_noalloc(const float* d_boids, int n, int grid_res_x, int grid_res_y, float domain_min_x,
                            float domain_min_y, float domain_span_x, float domain_span_y, uint32_t* d_grid_id,
                            uint32_t* d_boid_id, uint32_t* d_cells, void* stream);

/* ---- safety metrics: write-only side outputs of each step (the reference's metrics_deposit.comp and
 * metrics_finalize.comp; CPU mirror MetricsReference, src/metrics.cpp:429-476) ----
 * Per step: every agent active in the step's input and evacuated in its output counts towards the exit at its last
 * active position (stadium: the avenue gap it crossed; grid venues: the exit box holding it, slot 5 + box index, else
 * slot 4) and records the step index; every active agent deposits one person onto the 4 floor cells around it
 * (cloud-in-cell on a metric_res^2 grid of 1 m cells, position quantised to 1/256 cell, integer weights summing to
 * 65536) with its horizontal speed; then each cell updates its peak, occupied steps, steps at or above the three
 * density thresholds (as integer masses), and 64-bit sums. All integer: the result does not depend on order. */
typedef struct SwarmMetricCounters {   /* GpuMetricCounters (include/swarm/gpu_types.hpp), 784 bytes */
    uint32_t step, active, evacuated, active_accum;
    uint32_t exits[61];
    uint32_t pad[3];
    uint32_t gangway_visits[64], gangway_last[64];
} SwarmMetricCounters;
typedef struct SwarmMetricCell {       /* GpuMetricCell, 64 bytes */
    uint32_t last_mass, last_speed_mass, peak_mass, occupied_steps;
    uint32_t steps_above[4];
    uint32_t mass_steps[2], speed_mass_steps[2], exposure_mass_steps[2], pad[2];
} SwarmMetricCell;
/* Enables the metrics after every following step: the metric grid (res x res cells of 1 metre, res a multiple of 16,
 * centred on the venue's metric_center) and each cell's threshold masses (4 per cell: LoS E, LoS F, crush, unused;
 * 0xFFFFFFFF: never; the reference's GpuMetricCellInfo::thresholdMass). Resets the accumulators. */
int swarm_metrics_enable(SwarmHandle h, int res, const uint32_t* threshold_mass);
int swarm_metrics_reset(SwarmHandle h);
/* Reads the counters, the res^2 cells and the per-agent evacuation step (0: not evacuated); any may be NULL. */
int swarm_metrics_read(SwarmHandle h, SwarmMetricCounters* counters, SwarmMetricCell* cells, uint32_t* evac_step, int n);
/* Threshold masses of a grid venue (host): each 1 m cell's walkable area is sampled on a 40 x 40 lattice (free where
 * the wall SDF is positive, inside the exit line); cells under 0.1 m^2 never reach a threshold. */
int swarm_metric_thresholds_grid(const SwarmVenue* venue, int res, uint32_t* threshold_mass);

/* ---- headless evacuation runs and the on-disk formats ---- */
/* The evacuation statistics of a run (the reference's run_experiment summary: t50 / t90 / t100). */
typedef struct SwarmEvacuation {
    int32_t steps;                /* steps run */
    int32_t initial_active;       /* agents active before the first step */
    int32_t remaining;            /* agents active after the last step */
    int32_t t50_step, t90_step, t100_step;   /* the first step after which at least 50 / 90 / 100 % of the initially
                                                active agents have left; -1: not within the steps run */
    float t50_s, t90_s, t100_s;   /* the same in seconds (step x dt); -1: not reached */
} SwarmEvacuation;
/* run_experiment's headless evacuation (DedovSergei/swarm-crowd-simulation tools/experiment/run_experiment.cpp): steps
 * until no agent is active or max_steps, counting the active agents after every step on the device (the metrics,
 * when enabled, record every step as usual). active_out (may be NULL): max_steps entries, the active count after each
 * step run. The state (and the metrics) are left after the last step run: the step at which the crowd emptied, or
 * max_steps. */
int swarm_run_evacuation(SwarmHandle h, int max_steps, int32_t* active_out, SwarmEvacuation* out);

/* Workload snapshots (tools/benchmark/bench_common.hpp:109-134 saveSnapshot / loadSnapshot): a raw GpuBoid array, n x
 * 32 bytes, nothing else. read: the file must hold exactly n agents. count: the agents a file holds (-1: not a
 * whole number of GpuBoids or unreadable). */
int swarm_snapshot_write(const char* path, const float* boids, int n);
int swarm_snapshot_read(const char* path, float* boids, int n);
int swarm_snapshot_count(const char* path);
/* The baked terrace volume (src/sdf.cpp:84-107 loadSDFVolume): res^3 float32, exactly (stadium.sdf: res 130). */
int swarm_sdf_read(const char* path, float* sdf, int res);
/* A seated venue's navigation-field cache file as the reference writes it (nav::save / nav::load,
 * src/nav_field.cpp:554-656; nav::cacheFile, include/swarm/nav_field.hpp:226-233), read into the GPU table the seated
 * venue takes (SwarmVenue::nav_cells): per cell the anchor's centre, the distance and the info bits, exactly as
 * nav::gpuCells makes them (src/nav_field.cpp:443-454). Checks the magic, the version (2), the sizes and the FNV-1a
 * checksum; expected_key: the venue's nav::cacheKey, or 0 to accept any. cells NULL: a size query (res, origin, cell
 * and 1 / cell only); else capacity >= res^2. */
int swarm_nav_cache_read(const char* path, uint64_t expected_key, SwarmNavCell* cells, int64_t capacity, int32_t* res,
                         float* origin, float* cell, float* inv_cell);
/* A seated venue's exit-choice cache file as the reference writes it (nav::saveChoice / nav::loadChoice,
 * src/exit_choice.cpp:358-427; nav::choiceCacheFile :344-348): magic "SWCHOI01", version 6, 24 candidates, the grid,
 * the key, the index and entries, each exit's clear width and name, the FNV-1a checksum of everything after the magic.
 * expected_key: the venue's nav::choiceCacheKey, or 0 to accept any. With index and entries NULL: a size query (res,
 * n_entries, exits). Else index_capacity >= res^2 and entry_capacity >= n_entries; width_m (n_exits doubles, may be
 * NULL) receives the clear widths, from which nav::setChoiceCapacities derives inv_cap_s = 60 / (w x 83.6). */
int swarm_choice_cache_read(const char* path, uint64_t expected_key, uint32_t* index, int64_t index_capacity,
                            SwarmNavChoiceCell* entries, int64_t entry_capacity, double* width_m, int32_t* res,
                            float* origin, float* cell, float* inv_cell, int32_t* n_exits, int64_t* n_entries);

/* ---- the adjoint: gradients of an evacuation loss ----
 * No counterpart in the reference, which has no differentiation. The loss of `steps` steps from the handle's state:
 *   SWARM_LOSS_NAV_DISTANCE   L = dt * sum_{t = 1..steps} sum_{i active after step t} D(p_i(t)),
 * D the bilinear sample of the venue's geodesic distance grid (the time-integrated distance to the exits). Its
 * gradient with respect to each agent's radius r_i and desired speed v0_i and to the relaxation time tau (the model
 * reads tau and relax_step = exp(-dt / tau)) comes from the hand-written adjoint of the step: branches frozen at the
 * forward's choices (contact sets, the headway argmin, clamps, wall passes), the forward state checkpointed every
 * ckpt_every steps and recomputed, with a tape, one segment at a time while the segments are reversed. */
#define SWARM_LOSS_NAV_DISTANCE 0
typedef struct SwarmLossSpec {
    int32_t kind;                 /* SWARM_LOSS_NAV_DISTANCE */
    int32_t pad;
} SwarmLossSpec;
typedef struct SwarmAdjointStats {
    float ms_checkpoint;          /* the forward pass that stores the checkpoints */
    float ms_recompute;           /* the segments' taped forward */
    float ms_reverse;             /* the reverse steps */
    float ms_total;
    int64_t launches;             /* kernels launched */
    int64_t tape_bytes;           /* device memory of the tape and checkpoints */
    /* the fused reverse's phases (block 0's clock, summed over the steps): final pass, sweeps, predict's own terms,
     * predict's pair gather; 0 on the per-phase path */
    float ms_rev_final, ms_rev_sweeps, ms_rev_predict, ms_rev_gather;
    int32_t segments;             /* checkpointed segments */
    int32_t kept_segments;        /* of them taped in the checkpoint pass (the others recomputed) */
} SwarmAdjointStats;
/* Grid venues without a floor grid (a floor grid brings in the step-up limit, whose blocked moves have no reverse),
 * one instance, no drive table, wall_passes <= 5. The handle's state is left as it was. loss_out gets L;
 * dL_dv0 and dL_dr (n each, agent order) and dL_dtau (1) the gradient; stats (may be NULL) the pass times, measured
 * with events on the handle's stream. */
int swarm_adjoint_run(SwarmHandle h, const SwarmLossSpec* loss, int steps, int ckpt_every, double* loss_out,
                      float* dL_dv0, float* dL_dr, float* dL_dtau, SwarmAdjointStats* stats);
/* Two-level checkpointing: the state is checkpointed every ckpt_every steps, and the checkpoint pass also keeps the
 * full tapes of the last segments, as many as `bytes` of device memory hold beyond the one segment always kept; only
 * the other segments are recomputed in the reverse sweep (the gradients are the same bits either way). Default 1 GiB;
 * 0: every segment but the last is recomputed. No reference counterpart. */
int swarm_adjoint_set_tape_budget(SwarmHandle h, int64_t bytes);
/* Sets the relaxation time: tau_relax = tau and relax_step = exp(-dt / tau) (rounded once from double), the
 * parameterisation the adjoint differentiates. No reference counterpart (the reference fixes tau at build time). */
int swarm_set_relaxation_time(SwarmHandle h, float tau);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif /* SWARM_CUDA_H */
