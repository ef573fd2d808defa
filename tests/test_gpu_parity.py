"""Parity of the CUDA step with the oracle and the reference's own outputs (the reference's tools/test_gpu.cpp
parity.grid :1894-1962 and parity.one_step :1964-2033, tightened: the sorted pairs and the cell table bit-exact, the
state within 1e-5 per component -- the step's tolerance for FP32 -- and in practice bit for bit).

Every test here calls the library through its C ABI (swarm_gb300 is a ctypes layer over include/swarm_cuda.h)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5   # metres (model units on the terrace) and metres per second, per component


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def assert_state_close(a, b, tol=TOL):
    assert a.shape == b.shape
    assert np.array_equal(a[:, 3], b[:, 3]), "evacuation flags differ"
    d = np.abs(a.astype(np.float64) - b.astype(np.float64))
    assert d.max() <= tol, f"max |diff| {d.max():.3g} at agent {np.unravel_index(d.argmax(), d.shape)}"


@pytest.fixture(scope="module")
def terrace(built, stadium_sdf):
    import swarm_gb300
    from swarm_gb300.venues import Venue
    return swarm_gb300.params_reference(), Venue.stadium(stadium_sdf)


def _sim(P, venue, state, radius=None, v0=None, capacity=None):
    import swarm_gb300
    sim = swarm_gb300.CrowdSim(P, venue, capacity or state.shape[0])
    sim.set_state(state)
    if radius is not None:
        sim.set_agent_params(radius, v0)
    return sim


# ---------------- the reference's terrace ----------------

def test_terrace_one_step_from_spawn_vs_reference_fixture(terrace, terrace_golden):
    P, venue = terrace
    g = terrace_golden
    sim = _sim(P, venue, g["spawn"])
    sim.step(1)
    key, ids = sim.grid()
    assert np.array_equal(key, g["grid1_key"]), "gridID sequence"
    assert np.array_equal(ids, g["grid1_id"]), "sorted boidIDs (stable by id)"
    assert np.array_equal(sim.cells(), g["cells1"]), "cell table"
    assert np.array_equal(sim.contacts(), g["contacts1"]), "contact branches"
    st = sim.state()
    assert_state_close(st, g["state1"])
    assert np.array_equal(_bits(st), _bits(g["state1"])), "one step is bit-exact"


def test_terrace_250_steps_reproduce_reference_hash(terrace, terrace_golden):
    P, venue = terrace
    g = terrace_golden
    sim = _sim(P, venue, g["spawn"])
    sim.step(250)
    st = sim.state()
    assert_state_close(st, g["state250"])
    assert O.state_hash(st) == int(g["hash250"][0]), "state hash after 250 steps (bit-exact trajectory)"


def test_terrace_one_step_from_congested_state(terrace, terrace_golden):
    P, venue = terrace
    g = terrace_golden
    sim = _sim(P, venue, g["state250"])
    sim.step(1)
    key, ids = sim.grid()
    assert np.array_equal(key, g["grid251_key"]) and np.array_equal(ids, g["grid251_id"])
    assert np.array_equal(sim.cells(), g["cells251"])
    assert np.array_equal(sim.contacts(), g["contacts251"])
    assert np.array_equal(_bits(sim.state()), _bits(g["state251"]))


@pytest.mark.parametrize("k", [0, 1, 2, 8])
def test_terrace_iteration_counts_vs_oracle(terrace, terrace_golden, k):
    P, venue = terrace
    st0 = terrace_golden["state250"]
    sim = _sim(P, venue, st0)
    sim.set_projection_iterations(k)
    ora = O.OracleSim(P, venue.struct)
    ora.set_state(st0)
    ora.set_projection_iterations(k)
    for _ in range(3):
        sim.step(1)
        ora.step(1)
        assert np.array_equal(_bits(sim.state()), _bits(ora.state())), k


def test_terrace_graph_replay_is_bit_identical(terrace, terrace_golden):
    P, venue = terrace
    a = _sim(P, venue, terrace_golden["spawn"])
    b = _sim(P, venue, terrace_golden["spawn"])
    b.set_graph(True)
    a.step(20)
    b.step(20)
    assert np.array_equal(_bits(a.state()), _bits(b.state()))


def test_terrace_nan_positions_and_inactive_agents(terrace, terrace_golden):
    """calc_grid.comp's sanitiser (a NaN position becomes (0, 0, 0, 1)) and evacuated agents sorted to the tail."""
    P, venue = terrace
    st = terrace_golden["state250"].copy()
    st[5, :4] = [np.nan, np.nan, np.nan, 1.0]
    st[17:40, 3] = 0.0            # evacuated (w = 0)
    st[17:40, :3] = 1000.0
    sim = _sim(P, venue, st)
    ora = O.OracleSim(P, venue.struct)
    ora.set_state(st)
    sim.step(2)
    ora.step(2)
    assert np.array_equal(sim.grid()[0], ora.grid()[0]) and np.array_equal(sim.grid()[1], ora.grid()[1])
    assert np.array_equal(_bits(sim.state()), _bits(ora.state()))


@pytest.mark.parametrize("n", [1, 33, 1000])
def test_terrace_ragged_sizes(terrace, terrace_golden, n):
    P, venue = terrace
    st = terrace_golden["spawn"][:n].copy()
    sim = _sim(P, venue, st, capacity=4096)
    ora = O.OracleSim(P, venue.struct)
    ora.set_state(st)
    sim.step(3)
    ora.step(3)
    assert np.array_equal(sim.cells(), ora.cells())
    assert np.array_equal(_bits(sim.state()), _bits(ora.state()))


def test_terrace_evacuation_time_matches_the_reference(terrace, terrace_golden):
    """The reference terrace run to full evacuation on the GPU: the active count after every step equals the
    reference's own run (tests/golden/terrace_evac_ref.npz), so the evacuation time is the reference's exactly
    (2 696 steps; the required tolerance is 1 %)."""
    import os
    P, venue = terrace
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "terrace_evac_ref.npz"))
    sim = _sim(P, venue, terrace_golden["spawn"])
    active = []
    for _ in range(int(ref["evacuation_steps"][0])):
        sim.step(1)
        active.append(int((sim.state()[:, 3] != 0).sum()))
    active = np.array(active)
    assert np.array_equal(active, ref["active"])
    t_gpu = int(np.argmax(active == 0)) + 1
    assert abs(t_gpu - int(ref["evacuation_steps"][0])) <= 0.01 * int(ref["evacuation_steps"][0])


def test_terrace_all_evacuated(terrace, terrace_golden):
    P, venue = terrace
    st = terrace_golden["spawn"][:64].copy()
    st[:, 3] = 0.0
    sim = _sim(P, venue, st)
    sim.step(2)
    assert np.array_equal(_bits(sim.state()), _bits(st))
    assert (sim.cells() == 0).all()
    key, ids = sim.grid()
    assert (key == 0xFFFFFFFF).all() and np.array_equal(ids, np.arange(64, dtype=np.uint32))


def test_terrace_drive_table(terrace, terrace_golden):
    """CpuCrowdSim::setDriveTable: forced e_goal per agent."""
    P, venue = terrace
    st = terrace_golden["state250"]
    rng = np.random.default_rng(3)
    ang = rng.uniform(0, 2 * np.pi, st.shape[0])
    drive = np.stack([np.cos(ang), np.sin(ang)], 1).astype(np.float32)
    sim = _sim(P, venue, st)
    sim.set_drive_table(drive)
    ora = O.OracleSim(P, venue.struct)
    ora.set_state(st)
    ora.set_drive_table(drive)
    sim.step(2)
    ora.step(2)
    assert np.array_equal(_bits(sim.state()), _bits(ora.state()))


def test_upload_validation(terrace, terrace_golden):
    import swarm_gb300
    P, venue = terrace
    sim = swarm_gb300.CrowdSim(P, venue, 128)
    with pytest.raises(swarm_gb300.SwarmError):
        sim.step(1)                      # no state yet
    with pytest.raises(swarm_gb300.SwarmError):
        sim.set_state(terrace_golden["spawn"][:200])   # above capacity
    with pytest.raises(swarm_gb300.SwarmError):
        sim.set_projection_iterations(-1)


# ---------------- the SI grid venues ----------------

@pytest.fixture(scope="module")
def c0(built):
    import swarm_gb300
    from swarm_gb300 import venues
    venue, spawn = venues.terrace_c0()
    return swarm_gb300.params_si(), venue, spawn


def test_grid_terrace_one_step_and_100_steps_vs_oracle(c0):
    P, venue, (boids, r, v0) = c0
    sim = _sim(P, venue, boids, r, v0)
    ora = O.OracleSim(P, venue.struct)
    ora.set_state(boids)
    ora.set_agent_params(r, v0)
    for s in range(100):
        sim.step(1)
        ora.step(1)
        if s == 0:
            assert np.array_equal(sim.grid()[0], ora.grid()[0]) and np.array_equal(sim.grid()[1], ora.grid()[1])
            assert np.array_equal(sim.cells(), ora.cells())
            assert np.array_equal(sim.contacts(), ora.contacts())
        assert_state_close(sim.state(), ora.state())
    assert np.array_equal(_bits(sim.state()), _bits(ora.state()))


def test_grid_hall_65536_one_step_vs_oracle_and_invariants(built):
    import swarm_gb300
    from swarm_gb300 import venues
    venue, (boids, r, v0) = venues.hall_c1()
    P = swarm_gb300.params_si()
    sim = _sim(P, venue, boids, r, v0)
    ora = O.OracleSim(P, venue.struct)
    ora.set_state(boids)
    ora.set_agent_params(r, v0)
    sim.step(1)
    ora.step(1)
    key, ids = sim.grid()
    assert np.array_equal(np.sort(ids), np.arange(ids.size, dtype=np.uint32)), "a permutation"
    assert (np.diff(key.astype(np.int64)) >= 0).all(), "keys sorted"
    assert np.array_equal(key, ora.grid()[0]) and np.array_equal(ids, ora.grid()[1])
    assert np.array_equal(sim.cells(), ora.cells())
    assert_state_close(sim.state(), ora.state())
    # determinism: the same input twice gives the same bits
    sim2 = _sim(P, venue, boids, r, v0)
    sim2.set_graph(True)
    sim2.step(1)
    assert np.array_equal(_bits(sim.state()), _bits(sim2.state()))


def test_grid_terrace_1000_steps_compared_every_step(c0):
    """The terrace workload's whole comparison run: 1 000 steps, the state bit for bit after every one."""
    P, venue, (boids, r, v0) = c0
    sim = _sim(P, venue, boids, r, v0)
    ora = O.OracleSim(P, venue.struct)
    ora.set_state(boids)
    ora.set_agent_params(r, v0)
    for s in range(1000):
        sim.step(1)
        ora.step(1)
        assert np.array_equal(_bits(sim.state()), _bits(ora.state())), f"step {s + 1}"
    assert (sim.state()[:, 3] == 0).sum() > 0, "the crowd has begun to leave"


def test_grid_hall_65536_2000_steps_vs_oracle(built):
    """The 140 m hall's whole run (2 000 steps, the doors congested for most of it): bit for bit every 250 steps."""
    import swarm_gb300
    from swarm_gb300 import venues
    venue, (boids, r, v0) = venues.hall_c1()
    P = swarm_gb300.params_si()
    sim = _sim(P, venue, boids, r, v0)
    ora = O.OracleSim(P, venue.struct)
    ora.set_state(boids)
    ora.set_agent_params(r, v0)
    for k in range(8):
        sim.step(250)
        ora.step(250)
        assert np.array_equal(_bits(sim.state()), _bits(ora.state())), f"after {250 * (k + 1)} steps"
    assert np.array_equal(sim.grid()[1], ora.grid()[1]) and np.array_equal(sim.cells(), ora.cells())


@pytest.mark.parametrize("fused,graph,timing", [(False, False, False), (False, False, True), (False, True, True),
                                               (False, True, False), (True, False, True)])
def test_execution_modes_are_bit_identical(terrace, terrace_golden, fused, graph, timing):
    """The persistent one-kernel step, kernel-by-kernel launches, whole-step graphs and per-stage graphs with stage
    events give the same bits."""
    P, venue = terrace
    a = _sim(P, venue, terrace_golden["spawn"])
    b = _sim(P, venue, terrace_golden["spawn"])
    b.set_fused(fused)
    b.set_graph(graph)
    b.set_timing(timing)
    for _ in range(4):
        a.step(3)
        b.step(3)
        if timing:
            t = b.stage_times()
            assert t["total"] > 0 and (fused or t["predict"] > 0)
    assert np.array_equal(_bits(a.state()), _bits(b.state()))


def test_fused_and_phase_kernels_agree_on_the_grid_hall(built):
    import swarm_gb300
    from swarm_gb300 import venues
    venue, (boids, r, v0) = venues.hall_c1()
    P = swarm_gb300.params_si()
    a = _sim(P, venue, boids, r, v0)
    b = _sim(P, venue, boids, r, v0)
    b.set_fused(False)
    b.set_graph(True)
    for _ in range(3):
        a.step(4)
        b.step(4)
        assert np.array_equal(_bits(a.state()), _bits(b.state()))
    assert np.array_equal(a.cells(), b.cells())
    assert np.array_equal(a.contacts(), b.contacts())


def test_barrier_timeout_is_reported_and_the_handle_recovers(terrace, terrace_golden):
    """A grid barrier that waits for a block that never arrives gives up after its 1 s limit: the step ends, the host
    reads SWARM_E_TIMEOUT, and the next steps run normally (no fault, no hang)."""
    import swarm_gb300
    P, venue = terrace
    st = terrace_golden["spawn"]
    sim = _sim(P, venue, st)
    assert swarm_gb300.lib().swarm_test_barrier_timeout(sim._h) == 0
    sim.step(1)
    with pytest.raises(swarm_gb300.SwarmError, match="gave up"):
        sim.synchronize()
    sim.set_state(st)
    sim.step(1)
    sim.synchronize()
    assert np.array_equal(_bits(sim.state()), _bits(terrace_golden["state1"]))


def test_evacuation_runner_matches_the_reference(terrace, terrace_golden):
    """swarm_run_evacuation on the reference terrace: the active count it keeps on the device after every step is
    the reference's own run, and its t100 is the reference's evacuation time (2 696 steps)."""
    import os
    P, venue = terrace
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "terrace_evac_ref.npz"))
    t_ref = int(ref["evacuation_steps"][0])
    sim = _sim(P, venue, terrace_golden["spawn"])
    stats, active = sim.run_evacuation(t_ref + 500)
    assert stats["steps"] == t_ref and stats["remaining"] == 0
    assert np.array_equal(active, ref["active"])
    n0 = int((terrace_golden["spawn"][:, 3] != 0).sum())
    assert stats["initial_active"] == n0
    assert stats["t100_step"] == t_ref
    assert stats["t50_step"] == int(np.argmax((n0 - ref["active"]) * 100 >= 50 * n0)) + 1
    assert stats["t90_step"] == int(np.argmax((n0 - ref["active"]) * 100 >= 90 * n0)) + 1
    assert stats["t100_s"] == pytest.approx(t_ref * P.dt, rel=1e-6)
    # the state it leaves is the state after t_ref steps: nobody active
    assert (sim.state()[:, 3] == 0).all()


def test_evacuation_runner_stops_at_max_steps(terrace, terrace_golden):
    import os
    P, venue = terrace
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "terrace_evac_ref.npz"))
    sim = _sim(P, venue, terrace_golden["spawn"])
    stats, active = sim.run_evacuation(300)
    assert stats["steps"] == 300 and active.shape == (300,)
    assert np.array_equal(active, ref["active"][:300])
    assert stats["remaining"] == int(ref["active"][299]) and stats["t100_step"] == -1


def test_chained_steps_and_fused_graphs_are_bit_identical(built):
    """Several steps in one persistent launch (a grid barrier between steps), a bounded number of steps per launch, the
    fused step replayed from a CUDA graph, and a chained call on pinned host buffers: the bits of one launch per step."""
    import torch
    import swarm_gb300
    from swarm_gb300 import venues
    venue, (boids, r, v0) = venues.terrace_c0()
    P = swarm_gb300.params_si()
    ref = _sim(P, venue, boids, r, v0)
    ref.set_tuning(True, 0, 0, 1)
    for _ in range(12):
        ref.step(1)
    want = _bits(ref.state())
    one = _sim(P, venue, boids, r, v0)
    one.step(12)
    assert one.launch_count() == 1, "twelve steps in one launch"
    assert np.array_equal(_bits(one.state()), want)
    assert np.array_equal(one.cells(), ref.cells()) and np.array_equal(one.contacts(), ref.contacts())
    chunked = _sim(P, venue, boids, r, v0)
    chunked.set_tuning(True, 0, 0, 5)
    chunked.step(12)
    assert chunked.launch_count() == 3
    assert np.array_equal(_bits(chunked.state()), want)
    graphed = _sim(P, venue, boids, r, v0)
    graphed.set_graph(True)
    for _ in range(12):
        graphed.step(1)
    assert np.array_equal(_bits(graphed.state()), want)
    host = swarm_gb300.CrowdSim(P, venue, boids.shape[0])
    host.set_agent_params(r, v0)
    buf = torch.from_numpy(boids.copy()).pin_memory()
    host.step_host(buf.data_ptr(), buf.data_ptr(), boids.shape[0], 5)
    host.step_host(buf.data_ptr(), buf.data_ptr(), boids.shape[0], 7)
    assert np.array_equal(_bits(buf.numpy()), want)
