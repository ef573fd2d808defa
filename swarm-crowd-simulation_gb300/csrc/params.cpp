// The model constants of the step (SwarmParams, include/swarm_cuda.h).
//
// swarm_params_reference: the reference's values (DedovSergei/swarm-crowd-simulation include/swarm/sim_params.hpp,
// model units: 1 length = 31.25 m, 1 time = 17.490671 s). The reference emits its constants into GLSL, whose compiler
// folds constant expressions over the shortest round-trip decimal literals in double precision and rounds once
// (sim_params.hpp:19-54); its CPU port uses the same folded values. foldDecimal() below gives a float's shortest
// round-trip decimal as a double, so the folded constants here carry the same bits.
//
// swarm_params_si: the SI preset of the grid venues (dt 0.05 s, K = 8 sweeps, tau 0.5 s, per-agent radius and v0):
// the reference's constants converted from model units to metres and seconds.

#include "../../include/swarm_cuda.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace {

// The shortest decimal (1..9 significant digits) that reads back as f, as the double nearest to that decimal.
double foldDecimal(float f) {
    if (f == 0.0f) return 0.0;
    char buf[64];
    for (int digits = 1; digits <= 9; ++digits) {
        std::snprintf(buf, sizeof buf, "%.*e", digits - 1, double(f));
        if (std::strtof(buf, nullptr) == f) return std::strtod(buf, nullptr);
    }
    return double(f);
}
float fmul(float a, float b) { return float(foldDecimal(a) * foldDecimal(b)); }
float fadd(float a, float b) { return float(foldDecimal(a) + foldDecimal(b)); }
float fdiv(float a, float b) { return float(foldDecimal(a) / foldDecimal(b)); }

// FEELER_DIRS (sim_params.hpp:208-210): every 22.5 degrees from +x, counter-clockwise, as float literals
const float kFeelerDirs[16][2] = {
    {1.0f, 0.0f}, {0.92387953f, 0.38268343f}, {0.70710678f, 0.70710678f}, {0.38268343f, 0.92387953f},
    {0.0f, 1.0f}, {-0.38268343f, 0.92387953f}, {-0.70710678f, 0.70710678f}, {-0.92387953f, 0.38268343f},
    {-1.0f, 0.0f}, {-0.92387953f, -0.38268343f}, {-0.70710678f, -0.70710678f}, {-0.38268343f, -0.92387953f},
    {0.0f, -1.0f}, {0.38268343f, -0.92387953f}, {0.70710678f, -0.70710678f}, {0.92387953f, -0.38268343f}};
// STEP_UP_SLIDE_DIRS (sim_params.hpp:289): (cos, sin) of 0, 30, 60 degrees
const float kSlideDirs[3][2] = {{1.0f, 0.0f}, {0.86602540f, 0.5f}, {0.5f, 0.86602540f}};

constexpr float kWorldScale = 31.25f;      // metres per model length unit
constexpr float kTimeScale = 17.490671f;   // seconds per model time unit

void setFeelers(SwarmParams* p) {
    p->feeler_count = 16;
    for (int i = 0; i < 16; ++i) {
        p->feeler_dir[i][0] = kFeelerDirs[i][0];
        p->feeler_dir[i][1] = kFeelerDirs[i][1];
        p->feeler_off[i][0] = kFeelerDirs[i][0] * p->feeler_reach;   // float products (sim_params.hpp:231-237)
        p->feeler_off[i][1] = kFeelerDirs[i][1] * p->feeler_reach;
        p->probe_off[i][0] = kFeelerDirs[i][0] * p->plane_probe_reach;
        p->probe_off[i][1] = kFeelerDirs[i][1] * p->plane_probe_reach;
    }
    for (int k = 0; k < 3; ++k) { p->step_up_slide[k][0] = kSlideDirs[k][0]; p->step_up_slide[k][1] = kSlideDirs[k][1]; }
    p->step_up_slide_tries = 3;
}

}  // namespace

extern "C" int swarm_params_reference(SwarmParams* p) {
    if (!p) return SWARM_E_INVALID;
    std::memset(p, 0, sizeof *p);
    const float bodyRadius = 0.0064f, personalRadius = 0.008f, rPerc = 0.045f;
    const float dt = 0.01f;
    const float tauRelax = float(foldDecimal(0.5f) / foldDecimal(kTimeScale));
    const float tHeadway = float(foldDecimal(0.3f) / foldDecimal(kTimeScale));
    const float gravity = float(foldDecimal(9.81f) * foldDecimal(kTimeScale) * foldDecimal(kTimeScale) / foldDecimal(kWorldScale));
    p->dt = dt;
    p->proj_iterations = 32;
    p->perc_ring = int(rPerc / (2.0f / 40.0f)) + 1;   // sim_params.hpp:516 over the terrace's 0.05 cells
    p->uniform_body = 1;
    p->body_radius = bodyRadius;
    p->body_diam = fmul(2.0f, bodyRadius);
    p->body_diam2 = fmul(p->body_diam, p->body_diam);
    p->r_sep = fmul(2.0f, personalRadius);
    p->r_sep2 = fmul(p->r_sep, p->r_sep);
    p->sep_margin = p->r_sep - p->body_diam;
    p->k_sep = 100.0f;
    p->r_perc2 = fmul(rPerc, rPerc);
    p->v_max = 0.75f;
    p->headway_rate = fdiv(1.0f, tHeadway);
    p->relax_step = float(std::exp(-foldDecimal(dt) / foldDecimal(tauRelax)));
    p->tau_relax = tauRelax;
    p->gravity_dt = fmul(gravity, dt);
    p->proj_relax = 1.0f;
    p->proj_max_shift = fmul(0.05f, bodyRadius);
    p->safe_eps = 1e-8f;
    p->stacked_xy2 = 1e-12f;
    p->hash_to_radians = float(6.28318530718 / 4294967296.0);
    p->goal_deadzone = 1e-4f;
    p->torso_height = 0.05f;
    p->obstacle_range = 0.025f;
    p->w_obs = 10.0f;
    p->obstacle_gain = 20.0f;
    p->obstacle_min_normal = 0.01f;
    p->obstacle_grad_h = 0.0015f;
    p->obstacle_grad_scale = fdiv(0.25f, p->obstacle_grad_h);
    p->wall_root_steps = 3;
    p->wall_recast_steps = 2;
    p->wall_passes = 3;
    p->floor_search_cells = 4;
    p->sweep_bisections = 8;
    p->fence_ccd_bisections = 8;
    p->feeler_reach = fmul(1.25f, bodyRadius);
    p->plane_probe_reach = fmul(2.5f, bodyRadius);
    p->wall_recast_tol = fmul(0.02f, bodyRadius);
    p->wall_max_nz = 0.6f;
    p->centre_grad_min = 1e-3f;
    p->floor_settle_reach = fmul(1.5f, bodyRadius);
    p->max_step_up = float(foldDecimal(0.30f) / foldDecimal(kWorldScale));
    p->step_up_tol = 1e-6f;
    p->step_up_floor_reach = fmul(6.0f, bodyRadius);
    p->step_up_sample = fmul(0.125f, bodyRadius);
    p->step_up_bisections = 8;
    p->step_up_max_samples = 32;
    setFeelers(p);
    // pitch fence (sim_params.hpp:315-327), float arithmetic as the reference's constexpr
    const float inner = 0.328395f, outer = 0.335432f;
    p->fence_center[0] = 0.0f; p->fence_center[1] = 0.0f;
    p->fence_half_mid[0] = p->fence_half_mid[1] = 0.5f * (inner + outer);
    const float thkVisual = 0.5f * (outer - inner);
    p->fence_half_thk_coll = thkVisual + bodyRadius;
    // egress router (sim_params.hpp:339-351)
    p->walkway_min = outer;
    p->walkway_max = 0.422f;
    p->walkway_centre = 0.380f;
    p->avenue_half = 0.090f;
    p->aisle_max = 0.152f;
    p->aisle_centre = 0.128f;
    p->avenue_target_depth = 1.2f;
    p->pitch_recovery_depth = fadd(p->walkway_min, 0.02f);
    p->park_coord = 1000.0f;
    p->metric_cells_per_unit = 31.25f;
    p->metric_speed_scale = float(double(kWorldScale) / double(kTimeScale));
    p->r_pair_max = bodyRadius;
    // incline speed and stair spacing (sim_params.hpp:447-454), folded in double from the decimal literals
    p->v_stair_up = float(foldDecimal(0.58f) * foldDecimal(kTimeScale) / foldDecimal(kWorldScale));
    p->v_stair_down = float(foldDecimal(0.655f) * foldDecimal(kTimeScale) / foldDecimal(kWorldScale));
    p->incline_inv_ref_slope = float(1.0 / foldDecimal(0.50952545f));
    p->t_headway = tHeadway;
    return SWARM_OK;
}

extern "C" int swarm_params_si(SwarmParams* p) {
    if (!p) return SWARM_E_INVALID;
    SwarmParams ref;
    swarm_params_reference(&ref);
    std::memset(p, 0, sizeof *p);
    const double L = kWorldScale, T = kTimeScale;
    const float dt = 0.05f, tau = 0.5f, rPerc = float(0.045 * L);   // R_PERC 1.40625 m
    p->dt = dt;
    p->proj_iterations = 8;
    p->perc_ring = int(rPerc / 0.5f) + 1;   // 0.5 m hash cells: 3
    p->uniform_body = 0;
    p->body_radius = 0.2f;
    p->body_diam = 0.4f;
    p->body_diam2 = 0.4f * 0.4f;
    p->r_sep = 0.5f;
    p->r_sep2 = 0.25f;
    p->sep_margin = 0.1f;   // 2 x (personal radius 0.25 m - body radius 0.20 m)
    p->k_sep = ref.k_sep;
    p->r_perc2 = rPerc * rPerc;
    p->v_max = 2.0f;        // the clamp: the largest desired speed of the spawn distribution
    p->headway_rate = float(1.0 / 0.3);
    p->relax_step = float(std::exp(-double(dt) / double(tau)));
    p->tau_relax = tau;
    p->gravity_dt = float(9.81 * double(dt));
    p->proj_relax = 1.0f;
    p->proj_max_shift = float(0.05 * 0.2);
    p->safe_eps = float(1e-8 * L);
    p->stacked_xy2 = float(1e-12 * L * L);
    p->hash_to_radians = ref.hash_to_radians;
    p->goal_deadzone = float(1e-4 * L);
    p->torso_height = float(0.05 * L);
    p->obstacle_range = float(0.025 * L);
    p->w_obs = float(10.0 / (T * T));   // an acceleration gain: 1 / time^2
    p->obstacle_gain = 20.0f;
    p->obstacle_min_normal = 0.01f;
    p->obstacle_grad_h = float(0.0015 * L);
    p->obstacle_grad_scale = float(0.25 / double(p->obstacle_grad_h));
    p->wall_root_steps = 3;
    p->wall_recast_steps = 2;
    p->wall_passes = 3;
    p->floor_search_cells = 4;
    p->sweep_bisections = 8;
    p->fence_ccd_bisections = 8;
    p->feeler_reach = 1.25f * 0.25f;        // reaches cover the largest radius of the spawn (0.25 m)
    p->plane_probe_reach = 2.5f * 0.25f;
    p->wall_recast_tol = float(0.02 * 0.2);
    p->wall_max_nz = 0.6f;
    p->centre_grad_min = 1e-3f;
    p->floor_settle_reach = 1.5f * 0.25f;
    p->max_step_up = 0.30f;
    p->step_up_tol = float(1e-6 * L);
    p->step_up_floor_reach = 6.0f * 0.25f;
    p->step_up_sample = 0.125f * 0.25f;
    p->step_up_bisections = 8;
    p->step_up_max_samples = 32;
    setFeelers(p);
    p->park_coord = 1000.0f;
    p->metric_cells_per_unit = 1.0f;
    p->metric_speed_scale = 1.0f;
    p->r_pair_max = 0.25f;   // the spawn's largest radius; swarm_set_agent_params checks every radius against it
    p->v_stair_up = 0.58f;
    p->v_stair_down = 0.655f;
    p->incline_inv_ref_slope = ref.incline_inv_ref_slope;
    p->t_headway = 0.3f;
    return SWARM_OK;
}
