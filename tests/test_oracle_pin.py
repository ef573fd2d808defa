"""The oracle is pinned to the reference before it checks anything: on the reference's own terrace venue, the CPU
restatement (oracle/swarm_oracle.cpp) reproduces the unmodified reference CpuCrowdSim bit for bit -- the golden
fixtures its own code wrote (tests/golden/make_golden.py), and, where the reference tree exists, the reference run
live (oracle/_ref)."""
import os

import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module")
def terrace(built, stadium_sdf):
    import swarm_gb300
    from swarm_gb300.venues import Venue
    return swarm_gb300.params_reference(), Venue.stadium(stadium_sdf)


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_one_step_from_spawn_matches_reference_bit_for_bit(terrace, terrace_golden):
    P, venue = terrace
    g = terrace_golden
    sim = O.OracleSim(P, venue.struct)
    sim.set_state(g["spawn"])
    sim.step(1)
    key, ids = sim.grid()
    assert np.array_equal(key, g["grid1_key"]) and np.array_equal(ids, g["grid1_id"])
    assert np.array_equal(sim.cells(), g["cells1"])
    assert np.array_equal(sim.contacts(), g["contacts1"])
    assert np.array_equal(_bits(sim.state()), _bits(g["state1"]))


def test_250_steps_reproduce_the_reference_state_hash(terrace, terrace_golden):
    P, venue = terrace
    g = terrace_golden
    sim = O.OracleSim(P, venue.struct)
    sim.set_state(g["spawn"])
    sim.step(250)
    st = sim.state()
    assert np.array_equal(_bits(st), _bits(g["state250"]))
    assert O.state_hash(st) == int(g["hash250"][0]) == 0xd2da895e4067dcf7
    sim.step(1)   # one step from the congested state
    key, ids = sim.grid()
    assert np.array_equal(key, g["grid251_key"]) and np.array_equal(ids, g["grid251_id"])
    assert np.array_equal(sim.cells(), g["cells251"])
    assert np.array_equal(sim.contacts(), g["contacts251"])
    assert np.array_equal(_bits(sim.state()), _bits(g["state251"]))


def test_full_evacuation_matches_the_reference(terrace, terrace_golden):
    """The spawn run to full evacuation: the active count after every step equals the reference's (2 696 steps)."""
    P, venue = terrace
    ref = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "terrace_evac_ref.npz"))
    sim = O.OracleSim(P, venue.struct)
    sim.set_state(terrace_golden["spawn"])
    active = []
    for _ in range(int(ref["evacuation_steps"][0])):
        sim.step(1)
        active.append(int((sim.state()[:, 3] != 0).sum()))
    assert np.array_equal(np.array(active), ref["active"])


def test_thread_invariance(terrace, terrace_golden):
    """parity.thread_invariance (tools/test_gpu.cpp:2035): bit-identical for any thread count."""
    P, venue = terrace
    outs = []
    for t in (1, 3):
        sim = O.OracleSim(P, venue.struct, threads=t)
        sim.set_state(terrace_golden["state250"])
        sim.step(5)
        outs.append(sim.state())
    assert np.array_equal(_bits(outs[0]), _bits(outs[1]))


@pytest.mark.skipif(not O.ref_available(), reason="the reference tree is not in this container")
def test_live_reference_matches_oracle_at_16384_with_fewer_iterations(terrace, stadium_sdf):
    P, venue = terrace
    assert O.ref_load_sdf(os.path.join(O.ref_dir(), "stadium.sdf"))
    spawn = O.ref_spawn_terrace(16384, 7)
    for k in (32, 3, 1, 0):
        ref = O.RefSim("terrace")
        ref.set_state(spawn)
        ref.set_projection_iterations(k)
        sim = O.OracleSim(P, venue.struct)
        sim.set_state(spawn)
        sim.set_projection_iterations(k)
        for _ in range(10):
            ref.step(1)
            sim.step(1)
            assert np.array_equal(_bits(ref.state()), _bits(sim.state())), k
        assert np.array_equal(ref.contacts(), sim.contacts())
