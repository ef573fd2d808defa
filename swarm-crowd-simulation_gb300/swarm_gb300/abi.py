"""ctypes mirror of the C ABI in include/swarm_cuda.h (the structs and status codes).

The structs are the data format of the library's boundary: the CUDA library, the C++ host class and the test-only
oracle all take them. Field order and types must match the header exactly (tests/test_abi.py checks the sizes).
"""
import ctypes as C

SWARM_OK = 0
SWARM_E_INVALID = -1
SWARM_E_CUDA = -2
SWARM_E_OOM = -3
SWARM_E_TIMEOUT = -4
SWARM_E_STATE = -5

SWARM_VENUE_STADIUM = 0
SWARM_VENUE_GRID = 1
SWARM_VENUE_SEATED = 2
SWARM_NAV_FIT = 0x100
SWARM_NAV_REACHABLE = 0x200

INACTIVE_CELL = 0xFFFFFFFF

# ContactBits (reference include/swarm/cpu_crowd_sim.hpp:52-61)
CONTACT_EXIT, CONTACT_FENCE_CCD, CONTACT_FENCE, CONTACT_FLOOR = 1, 2, 4, 8
CONTACT_WALL, CONTACT_AGENT, CONTACT_SWEEP, CONTACT_STEP_UP = 16, 32, 64, 128

_f = C.c_float
_i = C.c_int32


class SwarmParams(C.Structure):
    _fields_ = [
        ("dt", _f), ("proj_iterations", _i), ("perc_ring", _i), ("uniform_body", _i),
        ("body_radius", _f), ("body_diam", _f), ("body_diam2", _f), ("r_sep", _f), ("r_sep2", _f),
        ("sep_margin", _f), ("k_sep", _f), ("r_perc2", _f), ("v_max", _f), ("headway_rate", _f),
        ("relax_step", _f), ("tau_relax", _f), ("gravity_dt", _f), ("proj_relax", _f), ("proj_max_shift", _f),
        ("safe_eps", _f), ("stacked_xy2", _f), ("hash_to_radians", _f), ("goal_deadzone", _f),
        ("torso_height", _f), ("obstacle_range", _f), ("w_obs", _f), ("obstacle_gain", _f),
        ("obstacle_min_normal", _f), ("obstacle_grad_h", _f), ("obstacle_grad_scale", _f),
        ("feeler_count", _i), ("wall_root_steps", _i), ("wall_recast_steps", _i), ("wall_passes", _i),
        ("floor_search_cells", _i), ("sweep_bisections", _i), ("fence_ccd_bisections", _i), ("pad0", _i),
        ("feeler_reach", _f), ("plane_probe_reach", _f), ("wall_recast_tol", _f), ("wall_max_nz", _f),
        ("centre_grad_min", _f), ("floor_settle_reach", _f),
        ("feeler_dir", (_f * 2) * 16), ("feeler_off", (_f * 2) * 16), ("probe_off", (_f * 2) * 16),
        ("max_step_up", _f), ("step_up_tol", _f), ("step_up_floor_reach", _f), ("step_up_sample", _f),
        ("step_up_bisections", _i), ("step_up_max_samples", _i), ("step_up_slide_tries", _i), ("pad1", _i),
        ("step_up_slide", (_f * 2) * 3),
        ("fence_center", _f * 2), ("fence_half_mid", _f * 2), ("fence_half_thk_coll", _f),
        ("avenue_half", _f), ("walkway_min", _f), ("walkway_max", _f), ("walkway_centre", _f),
        ("aisle_max", _f), ("aisle_centre", _f), ("avenue_target_depth", _f), ("pitch_recovery_depth", _f),
        ("park_coord", _f),
        ("metric_cells_per_unit", _f), ("metric_speed_scale", _f), ("r_pair_max", _f),
        ("v_stair_up", _f), ("v_stair_down", _f), ("incline_inv_ref_slope", _f), ("t_headway", _f), ("pad2", _f * 1),
    ]


class SwarmSeatedLayout(C.Structure):
    """swarm::SeatedLayout (reference include/swarm/venue.hpp:99-138), model units."""
    _fields_ = [
        ("stand_front", _f), ("row0", _f), ("row_depth", _f), ("clearway", _f), ("rows", _i),
        ("conc_front", _f), ("conc_back", _f), ("outer_face", _f), ("landing_end", _f),
        ("avenue_half", _f), ("lat0", _f), ("gangway_lo", _f), ("gangway_hi", _f), ("exit_lo", _f), ("exit_hi", _f),
        ("corner_inset", _f), ("seat_inset", _f), ("face_margin", _f), ("wall_above", _f), ("wall_clear", _f),
        ("first_row", _f), ("row_rise", _f), ("seat_top", _f), ("barrier_top", _f), ("concourse_z", _f),
        ("wall_top", _f), ("rake", _f), ("max_band_steps", _i), ("gangways", _i),
        ("gw_lo", _f * 8), ("gw_hi", _f * 8), ("gw_row", _i * 8), ("gw_seated", _i * 8),
        ("doors", _i), ("door_lo", _f * 8), ("door_hi", _f * 8), ("corner_door_lo", _f),
    ]


class SwarmNavCell(C.Structure):
    _fields_ = [("anchor_x", _f), ("anchor_y", _f), ("dist", _f), ("info", C.c_uint32)]


class SwarmVenue(C.Structure):
    _fields_ = [
        ("kind", _i), ("grid_res_x", _i), ("grid_res_y", _i), ("n_exits", _i),
        ("domain_min_x", _f), ("domain_min_y", _f), ("domain_span_x", _f), ("domain_span_y", _f),
        ("exit_lo_x", _f), ("exit_lo_y", _f), ("exit_hi_x", _f), ("exit_hi_y", _f), ("exit_max_z", _f),
        ("sdf", C.POINTER(_f)), ("sdf_res", _i), ("sdf_origin", _f * 3), ("sdf_spacing", _f),
        ("wall_sdf", C.POINTER(_f)), ("wall_nx", _i), ("wall_ny", _i),
        ("wall_origin_x", _f), ("wall_origin_y", _f), ("wall_h", _f),
        ("nav_dist", C.POINTER(_f)), ("nav_nx", _i), ("nav_ny", _i),
        ("nav_origin_x", _f), ("nav_origin_y", _f), ("nav_h", _f),
        ("floor_height", C.POINTER(_f)), ("speed_factor", C.POINTER(_f)), ("exit_boxes", C.POINTER(_f)),
        ("metric_res", _i), ("metric_center_x", _f), ("metric_center_y", _f),
        ("exit_mask", C.POINTER(C.c_uint8)),
        ("seated", C.POINTER(SwarmSeatedLayout)), ("nav_cells", C.c_void_p), ("nav_res", _i),
        ("nav_grid_origin", _f), ("nav_grid_cell", _f), ("nav_grid_inv_cell", _f),
        ("incline_speed", _i), ("stair_headway", _i), ("stair_t_up", _f), ("stair_t_down", _f),
    ]


class SwarmStageTimes(C.Structure):
    _fields_ = [("hash", _f), ("sort", _f), ("cells", _f), ("predict", _f), ("project", _f),
                ("final_pass", _f), ("total", _f)]


class SwarmNavFieldStats(C.Structure):
    _fields_ = [("passes", _i), ("tiles", _i), ("tile_runs", C.c_int64), ("ms", _f), ("ms_solve", _f)]


SWARM_NAV_CPU, SWARM_NAV_GPU = 0, 1


class SwarmEvacuation(C.Structure):
    _fields_ = [("steps", _i), ("initial_active", _i), ("remaining", _i), ("t50_step", _i), ("t90_step", _i),
                ("t100_step", _i), ("t50_s", _f), ("t90_s", _f), ("t100_s", _f)]


SWARM_LOSS_NAV_DISTANCE = 0


class SwarmLossSpec(C.Structure):
    _fields_ = [("kind", _i), ("pad", _i)]


class SwarmExitChoiceSpec(C.Structure):
    _fields_ = [("n_exits", C.c_int32), ("candidates", C.c_int32), ("fields", C.POINTER(_f)),
                ("width_m", C.POINTER(_f)), ("type", C.POINTER(C.c_uint8))]


CHOICE_NONE = 0xFFFFFFFF
CHOICE_EMPTY = 0xFF
CHOICE_INDEX_FIT = 0x80000000
CHOICE_INDEX_MASK = 0x7FFFFFFF


class SwarmNavChoiceCell(C.Structure):
    _fields_ = [("slot", C.c_uint32 * 24), ("dist", C.c_uint32 * 12)]


class SwarmSeatedChoiceSpec(C.Structure):
    _fields_ = [("n_exits", C.c_int32), ("grid_res", C.c_int32), ("index", C.c_void_p), ("entries", C.c_void_p),
                ("n_entries", C.c_int64), ("inv_cap_s", C.POINTER(_f)), ("seconds_per_unit", _f),
                ("dist_quantum", _f), ("choice_steps", C.c_int32)]


class SwarmAdjointStats(C.Structure):
    _fields_ = [("ms_checkpoint", _f), ("ms_recompute", _f), ("ms_reverse", _f), ("ms_total", _f),
                ("launches", C.c_int64), ("tape_bytes", C.c_int64),
                ("ms_rev_final", _f), ("ms_rev_sweeps", _f), ("ms_rev_predict", _f), ("ms_rev_gather", _f),
                ("segments", C.c_int32), ("kept_segments", C.c_int32)]


def fptr(a):
    """A float* into a C-contiguous float32 numpy array (None for None)."""
    if a is None:
        return None
    assert a.dtype.name == "float32" and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(_f))


class SwarmMetricCounters(C.Structure):
    _fields_ = [("step", C.c_uint32), ("active", C.c_uint32), ("evacuated", C.c_uint32), ("active_accum", C.c_uint32),
                ("exits", C.c_uint32 * 61), ("pad", C.c_uint32 * 3), ("gangway_visits", C.c_uint32 * 64),
                ("gangway_last", C.c_uint32 * 64)]


METRIC_CELL_WORDS = 16   # SwarmMetricCell: 16 uint32 (last_mass, last_speed_mass, peak_mass, occupied_steps,
                         # steps_above[4], mass_steps[2], speed_mass_steps[2], exposure_mass_steps[2], pad[2])


class SwarmTuning(C.Structure):
    _fields_ = [("fused", C.c_int32), ("threads", C.c_int32), ("blocks_per_sm", C.c_int32), ("ms_per_step", C.c_float),
                ("steps_per_launch", C.c_int32)]
