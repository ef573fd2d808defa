"""Venues and spawns: the static inputs of the step.

Venue.stadium(sdf)   the reference's baked terrace (stadium.sdf, 130^3 float32, [x][y][z] z fastest; the terrace's
                     neighbour grid 40 x 40 over [-1, 1]^2, exit test EXIT_DEPTH 0.93 below EXIT_MAX_Z 0.05:
                     reference include/swarm/sim_params.hpp:57-70, 349-351)
Venue.hall(...)      a rectangular hall with door gaps on grids (SI units): the synthetic workloads below
"""
import ctypes as C
import math

import numpy as np

from . import _check, generator
from .abi import SWARM_NAV_REACHABLE, SWARM_VENUE_SEATED, SWARM_VENUE_STADIUM, SwarmSeatedLayout, SwarmVenue, fptr

SDF_RES = 130


class HallSpec(C.Structure):
    _fields_ = [("size_x", C.c_float), ("size_y", C.c_float), ("wall_thickness", C.c_float), ("exit_depth", C.c_float),
                ("margin", C.c_float), ("wall_h", C.c_float), ("nav_h", C.c_float), ("cell", C.c_float),
                ("n_doors", C.c_int32), ("door_wall", C.c_int32 * 8), ("door_center", C.c_float * 8),
                ("door_width", C.c_float * 8)]


class BowlSpec(C.Structure):
    _fields_ = [("sectors", C.c_int32), ("rows", C.c_int32), ("seats", C.c_int32), ("seat_width", C.c_float),
                ("row_pitch", C.c_float), ("rise", C.c_float), ("gangway", C.c_float), ("vomitory_width", C.c_float),
                ("vomitory_row", C.c_int32), ("perimeter_exits", C.c_int32), ("perimeter_exit_width", C.c_float),
                ("concourse", C.c_float), ("aisle", C.c_float), ("stair_speed", C.c_float), ("clearance", C.c_float),
                ("wall_h", C.c_float), ("nav_h", C.c_float),
                ("cell", C.c_float)]


def bowl_spec(sectors=32, rows=32, seats=62, seat_width=0.5, row_pitch=0.8, rise=0.4, gangway=1.2, vomitory_width=2.4,
              vomitory_row=16, perimeter_exits=8, perimeter_exit_width=4.0, concourse=4.0, aisle=1.2, stair_speed=0.6,
              clearance=0.2, wall_h=0.05, nav_h=0.1, cell=0.5):
    return BowlSpec(sectors, rows, seats, seat_width, row_pitch, rise, gangway, vomitory_width, vomitory_row,
                    perimeter_exits, perimeter_exit_width, concourse, aisle, stair_speed, clearance, wall_h, nav_h, cell)


class Venue:
    """A SwarmVenue plus the host arrays it points to (kept alive with it)."""

    def __init__(self, struct, arrays, name, meta=None):
        self.struct = struct
        self.arrays = arrays
        self.name = name
        self.meta = meta or {}

    @property
    def n_cells(self):
        return self.struct.grid_res_x * self.struct.grid_res_y

    def metric_thresholds(self, res=None):
        """Per 1 m cell threshold masses of a grid venue (walkable area sampled from its wall SDF)."""
        res = res or self.struct.metric_res
        out = np.empty((res * res, 4), np.uint32)
        _check(generator().swarm_metric_thresholds_grid(C.byref(self.struct), int(res), out.ctypes.data_as(C.c_void_p)),
               "swarm_metric_thresholds_grid")
        return res, out

    @staticmethod
    def stadium(sdf):
        sdf = np.ascontiguousarray(sdf, dtype=np.float32).reshape(-1)
        if sdf.size != SDF_RES ** 3:
            raise ValueError(f"stadium.sdf holds {sdf.size} samples, expected {SDF_RES ** 3}")
        v = SwarmVenue()
        v.kind = SWARM_VENUE_STADIUM
        v.grid_res_x = v.grid_res_y = 40
        v.domain_min_x = v.domain_min_y = -1.0
        v.domain_span_x = v.domain_span_y = 2.0
        v.exit_hi_x = 0.930
        v.exit_max_z = 0.050
        v.sdf = fptr(sdf)
        v.sdf_res = SDF_RES
        v.sdf_origin[:] = [-0.95, -0.95, -0.8092595]
        v.sdf_spacing = float(np.float32(1.9) / np.float32(127.0))   # SDF_SPACING = 1.9f / 127.0f
        v.metric_res = 64
        return Venue(v, {"sdf": sdf}, "terrace")

    @staticmethod
    def seated(layout, grid_res, domain_min, domain_span, exit_depth, exit_max_z, nav_cells=None, nav_grid=None,
               incline_speed=False, stair_times=None, name="seated"):
        """One of the reference's analytic seated venues (venues S, M, L; model units, reference constants).

        layout: its swarm::SeatedLayout as a SwarmSeatedLayout (or the struct's raw bytes); the neighbour grid
        (grid_res cells per axis over [domain_min, domain_min + domain_span]) and the exit test (max(|x|, |y|) >
        exit_depth below exit_max_z); nav_cells: its navigation field as the reference's GpuNavCell table (n x 4
        float32 words, the 4th the info bits), nav_grid = (res, origin, cell, 1 / cell); None: e_goal from the drive
        table (or the terrace's router). incline_speed: the free speed by the slope along e_goal; stair_times = (up,
        down): the stair spacing's time gaps on a full-slope incline (model time), None: the level spacing."""
        if not isinstance(layout, SwarmSeatedLayout):
            layout = SwarmSeatedLayout.from_buffer_copy(bytes(np.ascontiguousarray(layout, dtype=np.uint8)))
        v = SwarmVenue()
        v.kind = SWARM_VENUE_SEATED
        v.grid_res_x = v.grid_res_y = int(grid_res)
        v.domain_min_x = v.domain_min_y = float(domain_min)
        v.domain_span_x = v.domain_span_y = float(domain_span)
        v.exit_hi_x = float(exit_depth)
        v.exit_max_z = float(exit_max_z)
        v.metric_res = 64
        v.seated = C.pointer(layout)
        arrays = {"layout": layout}
        if nav_cells is not None:
            cells = np.ascontiguousarray(nav_cells, dtype=np.float32).reshape(-1, 4)
            res, origin, cell, inv = nav_grid
            if cells.shape[0] != int(res) * int(res):
                raise ValueError("nav_cells must hold res x res cells")
            v.nav_cells = cells.ctypes.data_as(C.c_void_p)
            v.nav_res = int(res)
            v.nav_grid_origin, v.nav_grid_cell, v.nav_grid_inv_cell = float(origin), float(cell), float(inv)
            arrays["nav_cells"] = cells
        v.incline_speed = 1 if incline_speed else 0
        if stair_times is not None:
            v.stair_headway = 1
            v.stair_t_up, v.stair_t_down = float(stair_times[0]), float(stair_times[1])
        return Venue(v, arrays, name)

    @staticmethod
    def hall(size_x, size_y, doors, wall_thickness=0.3, exit_depth=0.5, margin=1.0, wall_h=0.05, nav_h=0.1, cell=0.5,
             name="hall"):
        """doors: [(wall, centre, width)], wall 0: -x, 1: +x, 2: -y, 3: +y; centre along the wall from its midpoint."""
        spec = HallSpec()
        spec.size_x, spec.size_y, spec.wall_thickness = size_x, size_y, wall_thickness
        spec.exit_depth, spec.margin, spec.wall_h, spec.nav_h, spec.cell = exit_depth, margin, wall_h, nav_h, cell
        if len(doors) > 8:
            raise ValueError("at most 8 doors")
        spec.n_doors = len(doors)
        for i, (w, c, width) in enumerate(doors):
            spec.door_wall[i], spec.door_center[i], spec.door_width[i] = int(w), float(c), float(width)
        v = SwarmVenue()
        _check(generator().swarm_hall_layout(C.byref(spec), C.byref(v)), "swarm_hall_layout")
        wall = np.empty(v.wall_nx * v.wall_ny, np.float32)
        nav = np.empty(v.nav_nx * v.nav_ny, np.float32)
        boxes = np.empty(max(1, 4 * v.n_exits), np.float32)
        _check(generator().swarm_hall_fields(C.byref(spec), C.byref(v), fptr(wall), fptr(nav), fptr(boxes)), "swarm_hall_fields")
        v.wall_sdf = fptr(wall)
        v.nav_dist = fptr(nav)
        v.exit_boxes = fptr(boxes)
        meta = {"size": (size_x, size_y), "doors": list(doors), "spec": spec}
        return Venue(v, {"wall": wall, "nav": nav, "exit_boxes": boxes}, name, meta)


def _bowl(spec, name):
    v = SwarmVenue()
    _check(generator().swarm_bowl_layout(C.byref(spec), C.byref(v)), "swarm_bowl_layout")
    nw, nn = v.wall_nx * v.wall_ny, v.nav_nx * v.nav_ny
    wall, floor, speed = np.empty(nw, np.float32), np.empty(nw, np.float32), np.empty(nw, np.float32)
    nav, mask = np.empty(nn, np.float32), np.empty(nn, np.uint8)
    boxes = np.empty(4 * v.n_exits, np.float32)
    _check(generator().swarm_bowl_fields(C.byref(spec), C.byref(v), fptr(wall), fptr(nav), fptr(floor), fptr(speed),
                                   mask.ctypes.data_as(C.c_void_p), fptr(boxes)), "swarm_bowl_fields")
    v.wall_sdf, v.nav_dist, v.floor_height, v.speed_factor = fptr(wall), fptr(nav), fptr(floor), fptr(speed)
    v.exit_mask = mask.ctypes.data_as(C.POINTER(C.c_uint8))
    v.exit_boxes = fptr(boxes)
    arrays = {"wall": wall, "nav": nav, "floor": floor, "speed": speed, "exit_mask": mask, "exit_boxes": boxes}
    return Venue(v, arrays, name, {"spec": spec})


Venue.bowl = staticmethod(_bowl)


def nav_cells_from_anchors(anchor, info, nav_grid):
    """A seated venue's GpuNavCell table from each cell's anchor cell index and info word: the anchor's position is
    that cell's centre, origin + (i + 0.5) x cell in double rounded once (the reference's nav::Grid::centre); the
    distance word is 0 where the cell is reachable, +infinity where not (the step reads only the anchor and the info
    bits)."""
    res, origin, cell, _ = nav_grid
    res = int(res)
    anchor = np.asarray(anchor, dtype=np.int64)
    info = np.asarray(info, dtype=np.uint32)
    centre = (np.float64(np.float32(origin)) + (np.arange(res, dtype=np.float64) + 0.5) * np.float64(np.float32(cell))).astype(np.float32)
    out = np.empty((anchor.size, 4), np.float32)
    out[:, 0] = centre[anchor % res]
    out[:, 1] = centre[anchor // res]
    out[:, 2] = np.where((info & SWARM_NAV_REACHABLE) != 0, np.float32(0.0), np.float32(np.inf))
    out[:, 3] = info.view(np.float32)
    return out


def exit_fields(venue):
    """Each exit's own distance field on the venue's nav grid, for the queue-aware exit choice: (fields (n_exits,
    nav nodes), clear widths (m), types (0 avenue, 1 door)). Halls: one per door; bowls: the vomitories, then the
    perimeter exits. Solved as the venue's nearest-exit field (swarm_set_nav_solver picks the solver)."""
    v = venue.struct
    spec = venue.meta.get("spec")
    bowl = isinstance(spec, BowlSpec)
    n = spec.sectors + spec.perimeter_exits if bowl else spec.n_doors
    fields = np.empty((n, v.nav_nx * v.nav_ny), np.float32)
    widths = np.empty(n, np.float32)
    types = np.empty(n, np.uint8)
    fn = generator().swarm_bowl_exit_fields if bowl else generator().swarm_hall_exit_fields
    _check(fn(C.byref(spec), C.byref(v), fptr(fields), fptr(widths), types.ctypes.data_as(C.c_void_p)),
           "swarm_bowl_exit_fields" if bowl else "swarm_hall_exit_fields")
    return fields, widths, types


def spawn_bowl(spec, jitter=0.03, seed=0, r=(0.20, 0.25), v=(1.34, 0.26, 0.6, 2.0)):
    """One agent per seat at the seat centre, jittered: (boids (n, 8), radius (n,), v0 (n,))."""
    n = spec.sectors * spec.rows * spec.seats
    boids = np.empty((n, 8), np.float32)
    rad = np.empty(n, np.float32)
    v0 = np.empty(n, np.float32)
    _check(generator().swarm_spawn_bowl(C.byref(spec), jitter, seed, r[0], r[1], v[0], v[1], v[2], v[3], fptr(boids), fptr(rad),
                                  fptr(v0)), "swarm_spawn_bowl")
    return boids, rad, v0


def spawn_lattice(nx, ny, n=None, spacing=0.5, center=(0.0, 0.0), jitter=0.05, seed=0, r=(0.20, 0.25),
                  v=(1.34, 0.26, 0.6, 2.0)):
    """A jittered lattice spawn: (boids (n, 8), radius (n,), v0 (n,))."""
    n = nx * ny if n is None else n
    boids = np.empty((n, 8), np.float32)
    rad = np.empty(n, np.float32)
    v0 = np.empty(n, np.float32)
    _check(generator().swarm_spawn_lattice(nx, ny, n, spacing, center[0], center[1], jitter, seed, r[0], r[1], v[0], v[1], v[2],
                                     v[3], fptr(boids), fptr(rad), fptr(v0)), "swarm_spawn_lattice")
    return boids, rad, v0


# ---- the synthetic workloads (SI units, 0.5 m hash cells, dt 0.05 s, K = 8) ----
# Recorded resolutions of specs that cannot hold their lattice as written: a 64 x 64 lattice at 0.5 m spans 31.5 m, so
# the 40 m x 25 m terrace grows to 40 m x 34 m (its 4 m exit stays centred in a short wall); the 128 x 128 lattice
# spans 63.5 m, so the 80 m x 60 m hall grows to 80 m x 70 m.

def terrace_c0():
    """4 096 agents (64 x 64 lattice, 0.5 m) on a 40 m x 34 m terrace, one 4 m exit centred in the +x (short) wall."""
    venue = Venue.hall(40.0, 34.0, [(1, 0.0, 4.0)], name="terrace 40x34 m, 1 exit")
    return venue, spawn_lattice(64, 64, seed=0)


def hall_c1():
    """65 536 agents (256 x 256 lattice) in a 140 m x 140 m hall, four 4 m exits, one centred in each wall."""
    venue = Venue.hall(140.0, 140.0, [(0, 0.0, 4.0), (1, 0.0, 4.0), (2, 0.0, 4.0), (3, 0.0, 4.0)],
                       name="hall 140x140 m, 4 exits")
    return venue, spawn_lattice(256, 256, seed=0)


def bowl_c2(**kw):
    """The seated bowl: 32 sectors x 32 rows x 62 seats (63 488 agents), seat 0.5 m, row pitch 0.8 m, rise 0.4 m per
    row, 1.2 m gangways (stairs, speed factor 0.6), a 2.4 m vomitory per gangway at row 16, 8 perimeter exits of 4 m;
    agents at the seat centres jittered U(+-0.03 m), radius and desired speed as the lattice workloads (seed 0)."""
    spec = bowl_spec(**kw)
    return Venue.bowl(spec, "seated bowl %dx%dx%d" % (spec.sectors, spec.rows, spec.seats)), spawn_bowl(spec, seed=0)


def terrace_c4():
    """16 384 agents (128 x 128 lattice) in an 80 m x 70 m hall, two 4 m exits centred in the +-x walls."""
    venue = Venue.hall(80.0, 70.0, [(0, 0.0, 4.0), (1, 0.0, 4.0)], name="terrace 80x70 m, 2 exits")
    return venue, spawn_lattice(128, 128, seed=0)


def batch_instances(count=256, seed=0, n_lo=1024, n_hi=65536):
    """The instances of the batched workload: agent count log-uniform in [n_lo, n_hi], 1 or 2 exits of width
    U[1.5, 6] m, the hall side sqrt(N / 4) m + 0.5 m (4 agents / m^2 on the lattice), independent seeds."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        side_agents = int(math.ceil(math.sqrt(n)))
        side = math.sqrt(n / 4.0) + 0.5
        k = int(rng.integers(1, 3))
        walls = rng.choice(4, size=k, replace=False)
        doors = [(int(w), 0.0, float(rng.uniform(1.5, 6.0))) for w in walls]
        out.append({"n": n, "side": side, "lattice": side_agents, "doors": doors, "seed": int(rng.integers(1, 2**62))})
    return out


def build_instance(spec):
    """One instance of batch_instances(): its hall and its lattice spawn (n agents, seeded)."""
    venue = Venue.hall(spec["side"], spec["side"], spec["doors"], name=f"hall {spec['side']:.1f} m, {spec['n']} agents")
    nx = spec["lattice"]
    ny = (spec["n"] + nx - 1) // nx
    return venue, spawn_lattice(nx, ny, n=spec["n"], seed=spec["seed"])


def build_batch(count=256, seed=0, n_lo=1024, n_hi=65536, threads=None):
    """The batched workload: (venues, boids, radius, v0, counts), agents of all instances one after another. The
    instances are built on a thread pool (the native builders release the interpreter lock)."""
    import concurrent.futures as cf
    import os
    specs = batch_instances(count, seed, n_lo, n_hi)
    with cf.ThreadPoolExecutor(max_workers=threads or min(32, os.cpu_count() or 4)) as ex:
        built = list(ex.map(build_instance, specs))
    venues, bs, rs, vs, counts = [], [], [], [], []
    for spec, (v, (b, r, v0)) in zip(specs, built):
        venues.append(v)
        bs.append(b)
        rs.append(r)
        vs.append(v0)
        counts.append(spec["n"])
    return venues, np.concatenate(bs), np.concatenate(rs), np.concatenate(vs), np.array(counts, np.int32)
