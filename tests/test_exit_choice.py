"""The queue-aware exit choice (the reference's ExitChoice::QueueAware: physics.comp PHYSICS_PASS 0, nav::choiceStep,
src/exit_choice.cpp:580-790) on grid venues: per-exit distance fields, the candidate table, the oracle's choice pass,
and the GPU's four stage kernels against it bit for bit (assignments, counters, and the steps they steer)."""
import numpy as np
import pytest

from oracle import oracle as O

NONE = 0xFFFFFFFF
EMPTY = 0xFF


def _hall():
    from swarm_gb300 import venues
    # four doors of different widths; the crowd starts beside the +x door
    venue = venues.Venue.hall(40.0, 30.0, [(0, 0.0, 4.0), (1, 5.0, 3.0), (2, -8.0, 2.0), (3, 10.0, 6.0)],
                              name="choice hall")
    b, r, v0 = venues.spawn_lattice(40, 40, spacing=0.5, center=(10.0, 3.0), jitter=0.05, seed=5)
    return venue, b, r, v0


def _small_bowl():
    from swarm_gb300 import venues
    spec = venues.bowl_spec(sectors=8, rows=8, seats=12, vomitory_row=4, perimeter_exits=2)
    venue = venues.Venue.bowl(spec, "small bowl")
    b, r, v0 = venues.spawn_bowl(spec, seed=2)
    return venue, b, r, v0


@pytest.fixture(scope="module")
def hall(built):
    from swarm_gb300 import venues
    venue, b, r, v0 = _hall()
    return venue, b, r, v0, venues.exit_fields(venue)


@pytest.fixture(scope="module")
def bowl(built):
    from swarm_gb300 import venues
    venue, b, r, v0 = _small_bowl()
    return venue, b, r, v0, venues.exit_fields(venue)


def _oracle(P, venue, b, r, v0, fields, widths, types, K=24):
    import swarm_gb300
    ex, di = swarm_gb300.exit_choice_table(venue, fields, widths, types, K)
    ora = O.OracleSim(P, venue.struct)
    ora.set_state(b)
    ora.set_agent_params(r, v0)
    ora.set_exit_choice(fields, swarm_gb300.exit_inv_capacity(widths), ex, di)
    return ora


def test_exit_fields_agree_with_the_nearest_exit_field(hall, bowl):
    """Inside the venue the nearest exit's distance is the least of the exits' own distances (to the solver's
    rounding where one exit's opening lies on a path to another). (The bowl's fields fill the band around its walls
    from each field's own nearest reached node, which differs between fields near the exits: compared off the band.)"""
    for venue, *_, (fields, widths, types) in (hall, bowl):
        v = venue.struct
        nav = venue.arrays["nav"]
        reach = fields < fields.max(axis=1, keepdims=True)
        least = np.where(reach, fields, np.inf).min(axis=0)
        both = reach.any(axis=0) & (nav < nav.max())
        X = v.nav_origin_x + (np.arange(nav.size) % v.nav_nx) * v.nav_h
        Y = v.nav_origin_y + (np.arange(nav.size) // v.nav_nx) * v.nav_h
        if "spec" in venue.meta and hasattr(venue.meta["spec"], "n_doors"):
            both &= (np.abs(X) < 20.0) & (np.abs(Y) < 15.0)   # the hall's interior
        else:   # the bowl: nav node (i, j) is wall-grid node (2i, 2j); off the clearance band
            wall = venue.arrays["wall"].reshape(v.wall_ny, v.wall_nx)[::2, ::2].ravel()
            both &= wall > venue.meta["spec"].clearance + 0.05
        assert both.sum() > 10000
        assert np.abs(least[both] - nav[both]).max() < 0.1
        assert (fields.min(axis=1) == 0.0).all(), "every exit has sources"


def test_candidate_table_rules(bowl):
    """Ascending distances, distinct exits, the type rule (2 avenues and a door first, where reachable)."""
    import swarm_gb300
    venue, _, _, _, (fields, widths, types) = bowl
    ex, di = swarm_gb300.exit_choice_table(venue, fields, widths, types, 6)
    full = ex[:, 0] != EMPTY
    assert full.sum() > 1000
    for row_e, row_d in zip(ex[full], di[full]):
        k = int((row_e != EMPTY).sum())
        assert (row_e[:k] != EMPTY).all() and (row_e[k:] == EMPTY).all()
        assert len(set(row_e[:k].tolist())) == k
        assert (np.diff(row_d[:k]) >= 0).all()
    # cells that reach every exit hold 2 vomitories (type 0) and 1 perimeter door (type 1) among 6 candidates
    allreach = (ex != EMPTY).sum(axis=1) == 6
    t = types[np.where(ex[allreach] == EMPTY, 0, ex[allreach])]
    assert ((t == 0).sum(axis=1) >= 2).all() and ((t == 1).sum(axis=1) >= 1).all()


def test_candidate_table_rejects_invalid_specs(hall, stadium_sdf):
    """swarm_exit_choice_table's argument checks (host code, no GPU): a grid venue, 1..63 exits, 1..24 candidates,
    fields and types present, output buffers present."""
    import ctypes as C
    import swarm_gb300
    from swarm_gb300.abi import SWARM_E_INVALID, SWARM_OK
    from swarm_gb300.venues import Venue
    venue, _, _, _, (fields, widths, types) = hall
    L = swarm_gb300.lib()
    v = venue.struct
    cells = v.grid_res_x * v.grid_res_y
    ex = np.empty((cells, 24), np.uint8)
    di = np.empty((cells, 24), np.float32)
    out = (ex.ctypes.data_as(C.c_void_p), di.ctypes.data_as(C.POINTER(C.c_float)))

    def call(spec, venue_struct=v, outs=out):
        return L.swarm_exit_choice_table(C.byref(venue_struct) if venue_struct is not None else None,
                                         C.byref(spec) if spec is not None else None, *outs)

    spec, keep = swarm_gb300._choice_spec(fields, widths, types, 24)
    assert call(spec) == SWARM_OK
    for n_exits, k in ((0, 24), (64, 24), (4, 0), (4, 25)):
        bad, keep2 = swarm_gb300._choice_spec(fields, widths, types, 24)
        bad.n_exits, bad.candidates = n_exits, k
        assert call(bad) == SWARM_E_INVALID, (n_exits, k)
    no_fields, _ = swarm_gb300._choice_spec(fields, widths, types, 24)
    no_fields.fields = None
    assert call(no_fields) == SWARM_E_INVALID
    no_types, _ = swarm_gb300._choice_spec(fields, widths, types, 24)
    no_types.type = None
    assert call(no_types) == SWARM_E_INVALID
    assert call(None) == SWARM_E_INVALID
    assert call(spec, venue_struct=None) == SWARM_E_INVALID
    assert call(spec, outs=(None, out[1])) == SWARM_E_INVALID
    assert call(spec, venue_struct=Venue.stadium(stadium_sdf).struct) == SWARM_E_INVALID, "stadium: no exit fields"


def test_oracle_choice_assigns_switches_and_is_deterministic(hall):
    import swarm_gb300
    venue, b, r, v0, (fields, widths, types) = hall
    P = swarm_gb300.params_si()
    runs = []
    for _ in range(2):
        ora = _oracle(P, venue, b, r, v0, fields, widths, types)
        ora.step(1)
        a, c = ora.exit_choice()
        active = ora.state()[:, 3] != 0
        assert (a[active] != NONE).all(), "every agent holds an exit after its first step"
        ora.step(239)   # four evaluations (every 60 steps at dt 0.05 s)
        a, c = ora.exit_choice()
        runs.append((ora.state().copy(), a.copy(), c.copy()))
    (s0, a0, c0), (s1, a1, c1) = runs
    assert np.array_equal(s0.view(np.uint32), s1.view(np.uint32)) and np.array_equal(a0, a1) and np.array_equal(c0, c1)
    assert c0[0] > 0 and c0[2] > 0, f"evaluations and switches happen (counters {c0})"
    used = set(a0[s0[:, 3] != 0].tolist())
    assert len(used) >= 2, "the queue at the nearest door sends agents to others"


def _pair(P, venue, b, r, v0, fields, widths, types):
    import swarm_gb300
    sim = swarm_gb300.CrowdSim(P, venue, b.shape[0])
    sim.set_state(b)
    sim.set_agent_params(r, v0)
    sim.set_exit_choice(fields, widths, types)
    ora = _oracle(P, venue, b, r, v0, fields, widths, types)
    return sim, ora


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["hall", "bowl"])
def test_exit_choice_gpu_vs_oracle(case, hall, bowl):
    """Bit for bit, every 20 steps over 300 (five evaluations): states, assigned exits and counters."""
    import swarm_gb300
    venue, b, r, v0, (fields, widths, types) = hall if case == "hall" else bowl
    P = swarm_gb300.params_si()
    sim, ora = _pair(P, venue, b, r, v0, fields, widths, types)
    for k in range(15):
        sim.step(20)
        ora.step(20)
        assert np.array_equal(sim.state().view(np.uint32), ora.state().view(np.uint32)), f"after {20 * (k + 1)} steps"
        ga, gc = sim.exit_choice()
        oa, oc = ora.exit_choice()
        assert np.array_equal(ga, oa) and np.array_equal(gc, oc), f"choice after {20 * (k + 1)} steps"
    assert gc[2] > 0 or case == "bowl"
    sim.close()


@pytest.mark.gpu
def test_exit_choice_per_phase_path_and_restart(hall):
    """The per-phase kernels give the same bits as the fused step; a state upload restarts the choice."""
    import swarm_gb300
    venue, b, r, v0, (fields, widths, types) = hall
    P = swarm_gb300.params_si()
    out = []
    for fused in (True, False):
        sim = swarm_gb300.CrowdSim(P, venue, b.shape[0])
        sim.set_agent_params(r, v0)
        sim.set_fused(fused)
        sim.set_exit_choice(fields, widths, types)
        sim.set_state(b)
        sim.step(130)
        out.append((sim.state().copy(), sim.exit_choice()[0].copy()))
        sim.set_state(b)   # restart: nothing assigned until the next step
        assert (sim.exit_choice()[0] == NONE).all()
        sim.close()
    assert np.array_equal(out[0][0].view(np.uint32), out[1][0].view(np.uint32)) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.gpu
def test_exit_choice_through_step_host(hall):
    """swarm_step_host with the choice on (pinned buffers) gives the same bits as uploading and stepping."""
    import torch
    import swarm_gb300
    venue, b, r, v0, (fields, widths, types) = hall
    P = swarm_gb300.params_si()
    out = []
    for host in (False, True):
        sim = swarm_gb300.CrowdSim(P, venue, b.shape[0])
        sim.set_agent_params(r, v0)
        sim.set_exit_choice(fields, widths, types)
        if host:
            h_in = torch.from_numpy(b.copy()).pin_memory()
            h_out = torch.zeros_like(h_in).pin_memory()
            sim.step_host(h_in.data_ptr(), h_out.data_ptr(), b.shape[0], 70)
            out.append((h_out.numpy().copy(), sim.exit_choice()[0].copy()))
        else:
            sim.set_state(b)
            sim.step(70)
            out.append((sim.state().copy(), sim.exit_choice()[0].copy()))
        sim.close()
    assert np.array_equal(out[0][0].view(np.uint32), out[1][0].view(np.uint32)) and np.array_equal(out[0][1], out[1][1])



@pytest.mark.gpu
def test_exit_choice_evacuation_runner_rolls_back_the_choice(bowl):
    """The runner stops at the exact step the crowd empties by replaying a chunk from a saved copy; the choice's
    state is part of that copy, so its result equals the oracle stepped as many steps."""
    import swarm_gb300
    venue, b, r, v0, (fields, widths, types) = bowl
    P = swarm_gb300.params_si()
    sim, ora = _pair(P, venue, b, r, v0, fields, widths, types)
    ev, active = sim.run_evacuation(4000)
    assert ev["remaining"] == 0 and 0 < ev["steps"] < 4000
    ora.step(ev["steps"])
    assert np.array_equal(sim.state().view(np.uint32), ora.state().view(np.uint32))
    assert np.array_equal(sim.exit_choice()[0], ora.exit_choice()[0])
    sim.close()
