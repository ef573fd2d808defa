"""The seated bowl (the generated 63 488-seat venue: floor heightfield, stairs with a speed factor, thin row walls,
exits given by a mask) on the GPU against the oracle, through the C ABI: bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _pair(P, venue, b, r, v0):
    import swarm_gb300
    sim = swarm_gb300.CrowdSim(P, venue, b.shape[0])
    sim.set_state(b)
    sim.set_agent_params(r, v0)
    ora = O.OracleSim(P, venue.struct)
    ora.set_state(b)
    ora.set_agent_params(r, v0)
    return sim, ora


def test_small_bowl_to_full_evacuation_vs_oracle(built):
    import swarm_gb300
    from swarm_gb300 import venues
    spec = venues.bowl_spec(sectors=8, rows=8, seats=12, vomitory_row=4, perimeter_exits=2)
    venue = venues.Venue.bowl(spec, "small bowl")
    b, r, v0 = venues.spawn_bowl(spec, seed=1)
    sim, ora = _pair(swarm_gb300.params_si(), venue, b, r, v0)
    for k in range(12):
        sim.step(50)
        ora.step(50)
        assert np.array_equal(_bits(sim.state()), _bits(ora.state())), f"after {50 * (k + 1)} steps"
        assert np.array_equal(sim.contacts(), ora.contacts())
    assert (sim.state()[:, 3] == 0).all(), "everyone evacuated"


def test_bowl_63488_vs_oracle(built):
    """The full bowl: 20 steps from the seats, bit for bit, and the sort and cell table after the first."""
    import swarm_gb300
    from swarm_gb300 import venues
    venue, (b, r, v0) = venues.bowl_c2()
    assert b.shape[0] == 63488
    sim, ora = _pair(swarm_gb300.params_si(), venue, b, r, v0)
    sim.step(1)
    ora.step(1)
    assert np.array_equal(sim.grid()[0], ora.grid()[0]) and np.array_equal(sim.grid()[1], ora.grid()[1])
    assert np.array_equal(sim.cells(), ora.cells())
    for _ in range(19):
        sim.step(1)
        ora.step(1)
    assert np.array_equal(_bits(sim.state()), _bits(ora.state()))
    assert np.array_equal(sim.contacts(), ora.contacts())


def test_bowl_63488_whole_evacuation_vs_oracle(built):
    """The seated-bowl workload's whole run from the seats to its last agent out: bit for bit against the oracle at
    checkpoints every 1 000 steps, the state at the step the crowd empties (found by the GPU run, checked on the
    oracle), then the sorted pairs, the cell table and the contact bits."""
    import swarm_gb300
    from swarm_gb300 import venues
    venue, (b, r, v0) = venues.bowl_c2()
    sim, ora = _pair(swarm_gb300.params_si(), venue, b, r, v0)
    done = 0
    while done < 16000:
        sim.step(1000)
        ora.step(1000)
        done += 1000
        st = sim.state()
        assert np.array_equal(_bits(st), _bits(ora.state())), f"after {done} steps"
        if not (st[:, 3] != 0).any():
            break
    assert not (st[:, 3] != 0).any(), f"{int((st[:, 3] != 0).sum())} agents left after {done} steps"
    assert np.array_equal(sim.grid()[0], ora.grid()[0]) and np.array_equal(sim.grid()[1], ora.grid()[1])
    assert np.array_equal(sim.cells(), ora.cells())
    assert np.array_equal(sim.contacts(), ora.contacts())
