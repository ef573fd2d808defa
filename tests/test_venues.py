"""The synthetic venues and spawns (host code, no GPU): the hall's fields, the lattice spawn's distributions and its
determinism, the C++ host class compiles against the C ABI."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, PKG


@pytest.fixture(scope="module")
def c0(built):
    from swarm_gb300 import venues
    return venues.terrace_c0()


def test_hall_fields(c0):
    venue, _ = c0
    v = venue.struct
    wall = venue.arrays["wall"].reshape(v.wall_ny, v.wall_nx)
    nav = venue.arrays["nav"].reshape(v.nav_ny, v.nav_nx)
    # the interior is free, the wall ring is solid, the door gap (+x wall, |y| < 2 m) is open
    def w(x, y):
        return wall[int(round((y - v.wall_origin_y) / v.wall_h)), int(round((x - v.wall_origin_x) / v.wall_h))]
    assert w(0.0, 0.0) > 10.0
    assert w(20.15, 10.0) < 0.0 and w(-20.15, 0.0) < 0.0 and w(0.0, 17.15) < 0.0
    assert w(20.15, 0.0) > 1.0           # inside the 4 m door gap
    # the geodesic distance decreases towards the door and is 0 beyond the exit line
    def d(x, y):
        return nav[int(round((y - v.nav_origin_y) / v.nav_h)), int(round((x - v.nav_origin_x) / v.nav_h))]
    assert d(21.5, 0.0) == 0.0
    assert d(-19.0, 0.0) > d(0.0, 0.0) > d(19.0, 0.0) > 0.0
    assert abs(d(0.0, 0.0) - 21.0) < 0.3    # 20 m to the wall's inner face + 0.3 wall + 0.5 exit depth, first-order FMM
    assert d(-19.0, 16.0) > d(-19.0, 0.0)   # around: farther from the door


def test_lattice_spawn_distributions_and_determinism(built):
    from swarm_gb300.venues import spawn_lattice
    b1, r1, v1 = spawn_lattice(64, 64, seed=0)
    b2, r2, v2 = spawn_lattice(64, 64, seed=0)
    b3, _, _ = spawn_lattice(64, 64, seed=1)
    assert np.array_equal(b1, b2) and np.array_equal(r1, r2) and np.array_equal(v1, v2)
    assert not np.array_equal(b1, b3)
    assert r1.min() >= 0.2 and r1.max() <= 0.25 and abs(r1.mean() - 0.225) < 0.003
    assert v1.min() >= 0.6 and v1.max() <= 2.0 and abs(v1.mean() - 1.34) < 0.02 and abs(v1.std() - 0.26) < 0.02
    lattice = np.stack(np.meshgrid(np.arange(64) - 31.5, np.arange(64) - 31.5), -1).reshape(-1, 2) * 0.5
    assert np.abs(b1[:, :2] - lattice).max() <= 0.05 + 1e-6
    assert np.array_equal(b1[:, 2], r1) and (b1[:, 3] == 1).all() and (b1[:, 4:] == 0).all()


def test_batch_instances_spec():
    import sys
    sys.path.insert(0, PKG)
    from swarm_gb300.venues import batch_instances
    inst = batch_instances(256, seed=0)
    ns = np.array([i["n"] for i in inst])
    assert len(inst) == 256 and ns.min() >= 1024 and ns.max() <= 65536
    assert 10000 < ns.mean() < 22000          # log-uniform mean 64512 / ln 64 = 15.5k
    assert all(1 <= len(i["doors"]) <= 2 and all(1.5 <= d[2] <= 6.0 for d in i["doors"]) for i in inst)


def test_cpp_host_class_compiles_and_links(built, tmp_path):
    src = tmp_path / "t.cpp"
    src.write_text('#include "swarm_gb300.hpp"\n#include <cstdio>\n'
                   'int main(){ SwarmParams p = swarm_gb300::CudaCrowdSim::referenceParams();'
                   ' std::printf("%d %g\\n", p.proj_iterations, double(p.body_radius)); return 0; }\n')
    exe = tmp_path / "t"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", PKG, "-lswarm_gb300", "-Wl,-rpath," + PKG], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["32", "0.0064"]


@pytest.fixture(scope="module")
def bowl_small(built):
    from swarm_gb300 import venues
    spec = venues.bowl_spec(sectors=8, rows=8, seats=12, vomitory_row=4, perimeter_exits=2)
    return spec, venues.Venue.bowl(spec, "small bowl"), venues.spawn_bowl(spec, seed=1)


def _node(v, arr, x, y, h, nx):
    return arr[int(round((y - v.wall_origin_y) / h)) * nx + int(round((x - v.wall_origin_x) / h))]


def test_bowl_fields_and_seats(bowl_small):
    """Seats: clear of every wall by more than the largest radius, standing on their row's tread (rise per row), on
    free nav nodes with a finite distance, outside the exits. Stairs are slower; exits exist."""
    spec, venue, (b, r, v0) = bowl_small
    v = venue.struct
    A = venue.arrays
    n = spec.sectors * spec.rows * spec.seats
    assert b.shape == (n, 8) and v.n_exits == spec.sectors + spec.perimeter_exits
    wall = np.array([_node(v, A["wall"], x, y, v.wall_h, v.wall_nx) for x, y in b[:, :2]])
    floor = np.array([_node(v, A["floor"], x, y, v.wall_h, v.wall_nx) for x, y in b[:, :2]])
    nav = np.array([_node(v, A["nav"], x, y, v.nav_h, v.nav_nx) for x, y in b[:, :2]])
    mask = np.array([_node(v, A["exit_mask"], x, y, v.nav_h, v.nav_nx) for x, y in b[:, :2]])
    assert wall.min() > 0.25
    rows = np.repeat(np.tile(np.arange(spec.rows), spec.sectors), spec.seats)
    assert np.allclose(floor, rows * spec.rise) and np.allclose(b[:, 2], floor + r, atol=1e-6)
    assert (mask == 0).all() and np.isfinite(nav).all() and nav.max() < A["nav"].max()
    assert sorted(float(x) for x in np.unique(A["speed"])) == [float(np.float32(spec.stair_speed)), 1.0]
    assert A["exit_mask"].sum() > 0


def test_bowl_nav_band_fill(bowl_small):
    """The bowl's nav field beside its walls: every wall node (wall SDF within the clearance) within 1 m of a node the
    solver reached holds the value of a nearest reached node (Euclidean, over node centres) + 3 per metre of that
    distance; wall nodes farther away keep the plain fill (the largest reached value + 10 m)."""
    ndimage = pytest.importorskip("scipy.ndimage")
    spec, venue, _ = bowl_small
    v = venue.struct
    nav = venue.arrays["nav"].reshape(v.nav_ny, v.nav_nx).astype(np.float64)
    wall = venue.arrays["wall"].reshape(v.wall_ny, v.wall_nx)[::2, ::2]   # nav node (i, j) is wall node (2i, 2j)
    top = nav.max()
    kind3 = wall <= spec.clearance
    reached = ~kind3 & (nav < top)
    dist, (iy, ix) = ndimage.distance_transform_edt(~reached, return_indices=True)
    band = kind3 & (dist * v.nav_h <= 1.0)
    assert band.sum() > 10000
    assert (nav[kind3 & (dist * v.nav_h > 1.0 + 1e-6)] == top).all()
    ys, xs = np.nonzero(band)
    rng = np.random.default_rng(0)
    for k in rng.choice(ys.size, 3000, replace=False):
        y, x = int(ys[k]), int(xs[k])
        d = dist[y, x]
        r = int(np.ceil(d))
        wy, wx = np.mgrid[max(y - r, 0):min(y + r, v.nav_ny - 1) + 1, max(x - r, 0):min(x + r, v.nav_nx - 1) + 1]
        tie = reached[wy, wx] & (np.abs(np.hypot(wy - y, wx - x) - d) < 1e-9)
        want = (nav[wy, wx][tie] + 3.0 * (d * float(v.nav_h))).astype(np.float32)
        assert tie.any() and np.float32(nav[y, x]) in want, (y, x, d)


def test_small_bowl_evacuates_on_the_oracle(bowl_small):
    """The whole crowd finds the gangways, the stairs and an exit (the oracle, 768 agents)."""
    import swarm_gb300
    from oracle import oracle as O
    spec, venue, (b, r, v0) = bowl_small
    sim = O.OracleSim(swarm_gb300.params_si(), venue.struct)
    sim.set_state(b)
    sim.set_agent_params(r, v0)
    sim.step(600)
    assert (sim.state()[:, 3] == 0).all()
