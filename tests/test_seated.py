"""The reference's analytic seated venue S on the GPU, through the C ABI, against the unmodified reference's own outputs
(tests/golden/seated_S.npz, written by tests/golden/make_seated_golden.py from the reference's CPU step built from its
own sources) and its pinned state hashes (tools/golden_state.hpp:45, :62). The sorted pairs, the cell table and the
contact bits are compared exactly; states within the step's stated tolerance (TOL) and then bit for bit.

Four models of the reference: the dense forced scenario (every seat occupied, e_goal from a drive table: the contact
model alone), the nearest exit at the level speed (e_goal from the navigation field's anchors: navCell's NOFIT ring and
surface rule, navGoal's wall rule), the incline speed with the stair spacing, and its default model -- the queue-aware
exit choice on its own candidate table (tests/golden/seated_S_choice.npz) with the incline speed and stair spacing --
against the pins "CPU counting venue S routed" (tools/golden_state.hpp:55, :69)."""
import os
import zlib

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "seated_S.npz")
TOL = 1e-5                          # model units (length, length per model time), per component
PIN_DENSE = 0xa2abaea7c0139b09      # golden_state.hpp:45  CPU counting venue S dense
PIN_NEAREST = 0xb1d6dac42f5dcd09    # golden_state.hpp:62  CPU counting venue S nearest exit, level speed


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def fnv1a(a):
    """golden::stateHash (tools/golden_state.hpp:121-126): 64-bit FNV-1a over the raw state bytes."""
    h = 0xcbf29ce484222325
    for x in np.ascontiguousarray(a).view(np.uint8).tobytes():
        h = ((h ^ x) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return h


def assert_state(got, want, what):
    assert got.shape == want.shape
    assert np.array_equal(got[:, 3], want[:, 3]), f"{what}: evacuation flags differ"
    d = np.abs(got.astype(np.float64) - want.astype(np.float64)).max()
    assert d <= TOL, f"{what}: max |diff| {d:.3g}"
    assert np.array_equal(_bits(got), _bits(want)), f"{what}: not bit-exact"


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="module")
def nav_cells(golden):
    from swarm_gb300 import venues
    delta = np.frombuffer(zlib.decompress(golden["nav_anchor_delta_z"].tobytes()), np.int32)
    info = np.frombuffer(zlib.decompress(golden["nav_info_z"].tobytes()), np.uint32)
    return venues.nav_cells_from_anchors(np.cumsum(delta.astype(np.int64)), info, golden["nav_grid"])


def drive_tables(golden):
    n = golden["dense_spawn"].shape[0]
    x = np.frombuffer(zlib.decompress(golden["dense_drive_xor_z"].tobytes()), np.uint32).reshape(-1, n, 2)
    return np.bitwise_xor.accumulate(x, axis=0).view(np.float32)


def _venue(golden, cells=None, incline=False):
    from swarm_gb300.venues import Venue
    g = golden["grid"]
    inc = golden["incline"]
    return Venue.seated(golden["layout"], int(g[0]), g[1], g[2], g[3], g[4], nav_cells=cells,
                        nav_grid=golden["nav_grid"] if cells is not None else None, incline_speed=incline,
                        stair_times=(inc[4], inc[5]) if incline else None, name="S")


def _sim(golden, state, cells=None, incline=False):
    import swarm_gb300
    sim = swarm_gb300.CrowdSim(swarm_gb300.params_reference(), _venue(golden, cells, incline), state.shape[0])
    sim.set_state(state)
    return sim


def _one_step_matches(sim, golden, prefix):
    key, ids = sim.grid()
    assert np.array_equal(key, golden[prefix + "grid1_key"]), "gridID sequence"
    assert np.array_equal(ids, golden[prefix + "grid1_id"]), "sorted boidIDs"
    assert np.array_equal(sim.cells(), golden[prefix + "cells1"]), "cell table"
    assert np.array_equal(sim.contacts(), golden[prefix + "contacts1"]), "contact branches"
    assert_state(sim.state(), golden[prefix + "state1"], "one step")


def test_reference_constants_are_the_incline_and_stair_constants(built, golden):
    """swarm_params_reference's incline and stair constants are sim_params.hpp's folded values (the reference's own)."""
    import swarm_gb300
    p = swarm_gb300.params_reference()
    inc = golden["incline"]
    assert (np.float32(p.v_stair_up), np.float32(p.v_stair_down), np.float32(p.incline_inv_ref_slope),
            np.float32(p.t_headway)) == tuple(inc[:4])
    assert np.float32(1.0) / np.float32(p.headway_rate) != 0.0


def test_fixture_decodes_to_the_reference_table(golden, nav_cells):
    """The compact navigation table decodes to a whole GpuNavCell grid whose reachable cells anchor inside it."""
    res = int(golden["nav_grid"][0])
    assert nav_cells.shape == (res * res, 4)
    info = nav_cells[:, 3].view(np.uint32)
    reach = (info & 0x200) != 0
    assert 0.5 < reach.mean() < 0.9
    assert np.isfinite(nav_cells[reach, 0]).all()
    assert drive_tables(golden).shape == (250, golden["dense_spawn"].shape[0], 2)


@pytest.mark.gpu
def test_dense_forced_one_step_vs_reference(golden):
    sim = _sim(golden, golden["dense_spawn"])
    sim.set_drive_table(drive_tables(golden)[0])
    sim.step(1)
    _one_step_matches(sim, golden, "dense_")


@pytest.mark.gpu
@pytest.mark.parametrize("fused", [True, False])
def test_dense_forced_250_steps_reproduce_the_reference_pin(golden, fused):
    """tools/golden_state.hpp:45: the dense forced scenario's state after 250 steps hashes to the reference's pin."""
    tables = drive_tables(golden)
    sim = _sim(golden, golden["dense_spawn"])
    sim.set_fused(fused)
    for t in tables:
        sim.set_drive_table(t)
        sim.step(1)
    st = sim.state()
    assert_state(st, golden["dense_state250"], "250 steps")
    assert fnv1a(st) == PIN_DENSE


@pytest.mark.gpu
def test_nearest_exit_one_step_vs_reference(golden, nav_cells):
    sim = _sim(golden, golden["nearest_spawn"], nav_cells)
    sim.step(1)
    _one_step_matches(sim, golden, "nearest_")


@pytest.mark.gpu
def test_nearest_exit_250_steps_reproduce_the_reference_pin(golden, nav_cells):
    """tools/golden_state.hpp:62: venue S's full seat spawn, nearest exit, level speed, 250 steps."""
    sim = _sim(golden, golden["nearest_spawn"], nav_cells)
    done = 0
    for k in (10, 50, 250):
        sim.step(k - done)
        done = k
        assert_state(sim.state(), golden["nearest_state%d" % k], f"{k} steps")
    assert fnv1a(sim.state()) == PIN_NEAREST


@pytest.mark.gpu
def test_incline_speed_and_stair_spacing_vs_reference(golden, nav_cells):
    """The incline free speed and the stair spacing (EMPIRICAL time gaps) on the gangway inclines: the reference's
    states after 1, 50 and 250 steps."""
    sim = _sim(golden, golden["nearest_spawn"], nav_cells, incline=True)
    sim.step(1)
    _one_step_matches(sim, golden, "incline_")
    sim.step(49)
    assert_state(sim.state(), golden["incline_state50"], "50 steps")
    sim.step(200)
    st = sim.state()
    assert_state(st, golden["incline_state250"], "250 steps")
    assert fnv1a(st) == int(golden["incline_hash250"][0])


@pytest.mark.gpu
def test_seated_execution_modes_are_bit_identical(golden, nav_cells):
    """The fused persistent step and the per-phase kernels (and their graphs) give the same bits on the seated venue."""
    a = _sim(golden, golden["nearest_spawn"], nav_cells, incline=True)
    b = _sim(golden, golden["nearest_spawn"], nav_cells, incline=True)
    b.set_fused(False)
    b.set_graph(True)
    for _ in range(3):
        a.step(7)
        b.step(7)
        assert np.array_equal(_bits(a.state()), _bits(b.state()))
    assert np.array_equal(a.cells(), b.cells())
    assert np.array_equal(a.contacts(), b.contacts())


def _harness(tmp_path):
    import ctypes as C
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    so = tmp_path / "libseated_harness.so"
    if not so.exists():
        subprocess.run([os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc"), "-gencode", "arch=compute_103a,code=sm_103a",
                        "-O2", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-Xcompiler",
                        "-fPIC,-ffp-contract=off", "-shared", "-o", str(so), os.path.join(root, "tests", "seated_harness.cu")],
                       check=True)
    H = C.CDLL(str(so))
    V = C.c_void_p
    H.hs_eval.argtypes = [V, V, C.c_int, C.c_int, V, V, V, C.c_int, C.c_float, C.c_float, C.c_float]
    return H


def _geometry_check(tmp_path, venue, golden, nav_cells, positions, npts):
    """Every geometry operation of the product (host build) against the reference's own, bit for bit, at npts random
    points of the venue's domain and at the given agent positions."""
    import ctypes as C
    from oracle import oracle as O
    if not O.ref_available():
        pytest.skip("the reference's CPU build is not here")
    os.environ.setdefault("SWARM_NAV_CACHE", str(tmp_path / "navcache"))
    import swarm_gb300
    from swarm_gb300.abi import SwarmSeatedLayout
    H = _harness(tmp_path)
    R = O.ref_lib()
    R.ref_seated_eval.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    lay = SwarmSeatedLayout.from_buffer_copy(bytes(golden["layout"]))
    P = swarm_gb300.params_reference()
    ng = golden["nav_grid"]
    half = -float(golden["grid"][1])

    def both(op, inp, width):
        inp = np.ascontiguousarray(inp, np.float32)
        n = inp.shape[0]
        a = np.zeros((n, width), np.float32)
        b = np.zeros((n, width), np.float32)
        assert R.ref_seated_eval(venue, op, n, inp.ctypes.data, a.ctypes.data) == 0
        assert H.hs_eval(C.byref(lay), C.byref(P), op, n, inp.ctypes.data, b.ctypes.data, nav_cells.ctypes.data,
                         int(ng[0]), ng[1], ng[2], ng[3]) == 0
        bad = np.nonzero((a.view(np.uint32) != b.view(np.uint32)).any(axis=1))[0]
        assert bad.size == 0, f"op {op}: {bad.size} of {n} differ, e.g. at {inp[bad[0]]}: {a[bad[0]]} vs {b[bad[0]]}"
        return a

    rng = np.random.default_rng(7)
    pos = positions[np.abs(positions[:, 0]) < 2.0 * half]
    xy = np.concatenate([rng.uniform(-half, half, (npts, 2)), pos[:, :2]]).astype(np.float32)
    fh = both(0, xy, 1)[:, 0]
    both(1, xy, 2)
    z = fh + rng.uniform(-0.01, 0.03, xy.shape[0]).astype(np.float32)
    both(2, np.c_[xy, z], 4)
    reach = rng.choice([P.feeler_reach, P.plane_probe_reach, lay.face_margin, P.step_up_sample], xy.shape[0]).astype(np.float32)
    both(3, np.c_[xy, z + lay.wall_above, reach], 3)
    both(3, np.c_[xy, fh + P.step_up_tol, reach], 3)
    f0 = fh - rng.choice([0.0, P.step_up_floor_reach], xy.shape[0]).astype(np.float32)
    both(4, np.c_[xy, xy + rng.normal(0.0, 0.004, xy.shape).astype(np.float32), f0], 3)
    e = rng.normal(0.0, 1.0, xy.shape)
    both(5, np.c_[xy, (e / np.linalg.norm(e, axis=1, keepdims=True)).astype(np.float32)], 1)
    both(6, np.c_[xy, fh + P.body_radius], 2)
    both(6, pos, 2)


def test_geometry_equals_the_reference_point_by_point(tmp_path, golden, nav_cells):
    """The seated venue's geometry and navigation lookup as compiled into the CUDA step (csrc/venue_seated.cuh, built
    for the host by tests/seated_harness.cu) against the reference's own functions (seated::floorHeight, cellKey,
    sdfGrad, wall, stepUpScan, floorSlope, nav::goal) at random points of venue S and at the fixture's agent positions:
    bit for bit. Needs the reference's CPU build (this container)."""
    pos = np.concatenate([golden[k][:, :3] for k in golden if k.startswith(("dense_state", "nearest_state", "incline_state"))])
    _geometry_check(tmp_path, b"S", golden, nav_cells, pos, 100000)


def _generated(name):
    from swarm_gb300 import venues
    g = dict(np.load(os.path.join(os.path.dirname(GOLDEN), "seated_%s.npz" % name)))
    delta = np.frombuffer(zlib.decompress(g["nav_anchor_delta_z"].tobytes()), np.int32)
    info = np.frombuffer(zlib.decompress(g["nav_info_z"].tobytes()), np.uint32)
    cells = venues.nav_cells_from_anchors(np.cumsum(delta.astype(np.int64)), info, g["nav_grid"])
    spawn = np.frombuffer(zlib.decompress(g["spawn_z"].tobytes()), np.float32).reshape(-1, 8).copy()
    return g, cells, spawn


@pytest.mark.parametrize("name", ["M", "L"])
def test_geometry_of_the_generated_venues_equals_the_reference(tmp_path, name):
    """The same comparison on the generated venues M and L: several straight gangways per wing, a door per gangway
    head, corner doors, straight gangways merging with the corner gangway."""
    g, cells, spawn = _generated(name)
    _geometry_check(tmp_path, name.encode(), g, cells, spawn[spawn[:, 3] != 0, :3], 60000)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["M", "L"])
def test_generated_venue_runs_reproduce_the_reference(name):
    """Venues M (15 832 seated, N = 16 384) and L (63 424 seated, N = 65 536) from their full seat spawns: the states
    after 1, 10, 50 and 250 steps at the nearest exit and level speed, and after 10 and 250 steps with the incline
    speed and stair spacing, hash to the reference's own states (FNV-1a of the raw state)."""
    import swarm_gb300
    g, cells, spawn = _generated(name)
    assert spawn.shape[0] == int(g["n"][0]) and int((spawn[:, 3] != 0).sum()) == int(g["n"][1])
    for prefix, incline, keep in (("nearest_", False, (1, 10, 50, 250)), ("incline_", True, (10, 250))):
        sim = swarm_gb300.CrowdSim(swarm_gb300.params_reference(), _venue(g, cells, incline), spawn.shape[0])
        sim.set_state(spawn)
        done = 0
        for k in keep:
            sim.step(k - done)
            done = k
            assert fnv1a(sim.state()) == int(g[prefix + "hash%d" % k][0]), f"{name} {prefix}{k} steps"
        sim.close()


@pytest.mark.gpu
def test_contact_lists_keep_the_bits_into_the_congested_run():
    """Venue L from its full seat spawn for 2 250 steps (past the half-empty, congested state, where sweeps move agents
    far enough to rebuild the fused step's contact lists): the fused step, which walks its contact lists in the
    sweeps, and the per-phase kernels, which walk the whole 3 x 3 rows, give the same bits every 250 steps; then the
    cell table and the contact bits."""
    import swarm_gb300
    g, cells, spawn = _generated("L")
    a = swarm_gb300.CrowdSim(swarm_gb300.params_reference(), _venue(g, cells), spawn.shape[0])
    b = swarm_gb300.CrowdSim(swarm_gb300.params_reference(), _venue(g, cells), spawn.shape[0])
    a.set_state(spawn)
    b.set_state(spawn)
    b.set_fused(False)
    for k in range(9):
        a.step(250)
        b.step(250)
        assert np.array_equal(_bits(a.state()), _bits(b.state())), f"after {250 * (k + 1)} steps"
    assert 2 * int((a.state()[:, 3] != 0).sum()) < int((spawn[:, 3] != 0).sum()), "the run reached the congested state"
    assert np.array_equal(a.cells(), b.cells())
    assert np.array_equal(a.contacts(), b.contacts())
    a.close()
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["M", "L"])
@pytest.mark.parametrize("model", ["nearest", "incline"])
def test_generated_venue_whole_evacuation_matches_the_reference(name, model):
    """Venues M and L from their full seat spawns run to the last agent out at the nearest exit, at the level speed and
    with the incline speed and stair spacing, through swarm_run_evacuation: the active count after every step is the
    reference's own CPU run (tests/golden/seated_<name>_evac.npz), so each empties at the same step."""
    import swarm_gb300
    g, cells, spawn = _generated(name)
    ref = np.load(os.path.join(os.path.dirname(GOLDEN), "seated_%s_evac.npz" % name))[model + "_active"]
    sim = swarm_gb300.CrowdSim(swarm_gb300.params_reference(), _venue(g, cells, model == "incline"), spawn.shape[0])
    sim.set_state(spawn)
    stats, active = sim.run_evacuation(ref.shape[0] + 1000)
    assert stats["remaining"] == 0 and stats["steps"] == ref.shape[0] == stats["t100_step"]
    assert np.array_equal(active, ref)
    sim.close()


# ---- the queue-aware exit choice on the reference's own table ----
CHOICE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "seated_S_choice.npz")
PIN_ROUTED = 0x434356ac8d65471d         # golden_state.hpp:55  CPU counting venue S routed
PIN_ROUTED_LEVEL = 0x22ad15f59ee18632   # golden_state.hpp:69  CPU counting venue S routed, level spacing


@pytest.fixture(scope="module")
def choice(golden):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from seated_choice import choice_index, decode_choice_entries
    g = dict(np.load(CHOICE))
    info = np.frombuffer(zlib.decompress(golden["nav_info_z"].tobytes()), np.uint32)
    meta = g["choice_meta"]
    E = int(meta[0])
    return g, choice_index(info), decode_choice_entries(g), meta[3:3 + E].astype(np.float32), float(meta[1]), float(meta[2])


def test_choice_fixture_decodes_to_a_consistent_table(choice):
    """The table decoded from the fixture: every entry referenced once by the index, in grid order; every slot an exit
    of the venue or empty, anchors inside the grid; the estimate's terms as sim_params.hpp folds them."""
    g, index, entries, inv_cap, s_per_unit, quantum = choice
    res, ne, steps = (int(x) for x in g["choice_grid"])
    assert index.shape == (res * res,) and entries.shape == (ne, 36) and steps == 17
    e = index & 0x7FFFFFFF
    assert np.array_equal(e[e != 0], np.arange(1, ne + 1))
    ex = (entries[:, :24] >> 25) & 63
    assert ((ex < inv_cap.shape[0]) | (ex == 63)).all() and ((entries[:, :24] & 0x1FFFFFF) < res * res).all()
    assert quantum == 2.0 ** -12 and s_per_unit > 0 and (inv_cap > 0).all()


def test_choice_cache_file_reads_as_the_reference_table(built, tmp_path, monkeypatch):
    """swarm_choice_cache_read on the cache file the unmodified reference writes for venue S (nav::saveChoice) gives
    the reference's own index, entries and widths (their capacities: nav::setChoiceCapacities)."""
    import ctypes as C
    import glob
    import swarm_gb300
    from oracle import oracle as O
    if not O.ref_available():
        pytest.skip("the reference build (oracle/_ref) is not on this machine")
    monkeypatch.setenv("SWARM_NAV_CACHE", str(tmp_path))
    L = O.ref_lib()
    L.ref_choice_table.restype = C.c_longlong
    L.ref_choice_table.argtypes = [C.c_char_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
    meta = np.zeros(67, np.float32)
    res = C.c_int()
    ne = L.ref_choice_table(b"S", None, 0, None, 0, meta.ctypes.data, C.byref(res))
    index = np.empty(res.value ** 2, np.uint32)
    entries = np.empty((ne, 36), np.uint32)
    L.ref_choice_table(b"S", index.ctypes.data, index.shape[0], entries.ctypes.data, ne, meta.ctypes.data, C.byref(res))
    files = glob.glob(os.path.join(str(tmp_path), "nav_S_choice_*.bin"))
    if not files:
        pytest.skip("the reference process already held venue S's table (it builds or reads one per process)")
    idx, ent, widths, grid = swarm_gb300.choice_cache_read(files[0])
    assert grid[0] == res.value and np.array_equal(idx, index) and np.array_equal(ent, entries)
    cap = (60.0 / (widths * 83.6)).astype(np.float32)
    assert np.array_equal(cap, meta[3:3 + int(meta[0])])
    bad = tmp_path / "bad.bin"
    raw = bytearray(open(files[0], "rb").read())
    raw[100] ^= 1
    bad.write_bytes(bytes(raw))
    with pytest.raises(swarm_gb300.SwarmError):
        swarm_gb300.choice_cache_read(str(bad))


def _routed(golden, nav_cells, choice, stair=True):
    from swarm_gb300.venues import Venue
    import swarm_gb300
    g, index, entries, inv_cap, s_per_unit, quantum = choice
    gr = golden["grid"]
    inc = golden["incline"]
    venue = Venue.seated(golden["layout"], int(gr[0]), gr[1], gr[2], gr[3], gr[4], nav_cells=nav_cells,
                         nav_grid=golden["nav_grid"], incline_speed=True,
                         stair_times=(inc[4], inc[5]) if stair else None, name="S")
    sim = swarm_gb300.CrowdSim(swarm_gb300.params_reference(), venue, golden["nearest_spawn"].shape[0])
    sim.set_seated_choice(index, entries, inv_cap, s_per_unit, quantum, int(g["choice_grid"][2]))
    sim.set_state(golden["nearest_spawn"])
    return sim


@pytest.mark.gpu
def test_routed_exit_choice_reproduces_the_reference(golden, nav_cells, choice):
    """The reference's default model on venue S (queue-aware exit choice, incline speed, stair spacing EMPIRICAL) from
    the seat spawn: the assignments and counters after the first choice, before and after the first evaluation (steps
    17, 18), the states after 1 and 18 steps, the hash after 50, and after 250 steps the reference's pin."""
    g = choice[0]
    sim = _routed(golden, nav_cells, choice)
    done = 0
    for s in (1, 17, 18):
        sim.step(s - done)
        done = s
        a, c = sim.exit_choice()
        ref = g["routed_counters%d" % s]
        assert np.array_equal(a, g["routed_assign%d" % s]), f"assignments after step {s}"
        # GpuChoiceCounters: queue[128], switches, forced, evaluations, eligible
        assert (c[0], c[1], c[2], c[3]) == (ref[130], ref[131], ref[128], ref[129]), f"counters after step {s}"
        if s in (1, 18):
            assert_state(sim.state(), g["routed_state%d" % s], f"{s} steps")
    sim.step(32)
    assert fnv1a(sim.state()) == int(g["routed_hash50"][0]), "50 steps"
    sim.step(200)
    assert fnv1a(sim.state()) == PIN_ROUTED == int(g["routed_hash250"][0]), "the pin after 250 steps"


@pytest.mark.gpu
def test_routed_exit_choice_with_level_spacing_reproduces_the_reference_pin(golden, nav_cells, choice):
    """The same with the level spacing on the inclines (incline speed on, stair spacing off): the reference's pin."""
    sim = _routed(golden, nav_cells, choice, stair=False)
    sim.step(250)
    assert fnv1a(sim.state()) == PIN_ROUTED_LEVEL


@pytest.mark.gpu
@pytest.mark.parametrize("model", ["routed", "routed_level", "nearest", "incline"])
def test_whole_evacuation_matches_the_reference(golden, nav_cells, choice, model):
    """Venue S's full seat spawn run to its last agent out through swarm_run_evacuation, under the reference's default
    model (queue-aware exit choice on its own table, incline speed, stair spacing), the same with the level spacing,
    at the nearest exit and level speed, and at the nearest exit with the incline speed and stair spacing: the active
    count after every step is the reference's own CPU run (tests/golden/seated_S_evac.npz), so the crowd empties at
    the same step (routed: step 1 361, the step the reference's validation output records for its CPU counting
    sort)."""
    ref = np.load(os.path.join(os.path.dirname(CHOICE), "seated_S_evac.npz"))[model + "_active"]
    if model.startswith("routed"):
        sim = _routed(golden, nav_cells, choice, stair=model == "routed")
        assert model != "routed" or ref.shape[0] == 1361
    else:
        sim = _sim(golden, golden["nearest_spawn"], nav_cells, incline=model == "incline")
    stats, active = sim.run_evacuation(ref.shape[0] + 500)
    assert stats["remaining"] == 0 and stats["steps"] == ref.shape[0] == stats["t100_step"]
    assert np.array_equal(active, ref)
    assert (sim.state()[:, 3] == 0).all()
