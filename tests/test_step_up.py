"""The step-up limit on a grid venue with a floor heightfield (the reference's limitStepUp, cpu_crowd_sim.cpp:566-591,
with the floor grid in place of the baked column scan): a pedestrian climbs at most 0.30 m in one step.

The scene: a 20 m x 10 m hall, door in the +x wall; ahead of the crowd a 0.4 m platform (y > 0, the seated venues'
row riser, which must block) and a 0.2 m step (y < 0, a stair riser, which must not). 64 agents on a 1 m lattice
are driven along +x by the drive table. The oracle's rule is checked on the CPU; the GPU step is checked against
the oracle bit for bit (states and contact bits)."""
import numpy as np
import pytest

from oracle import oracle as O

PLATFORM, STEP = 0.4, 0.2
STEP_UP = 128   # the contact bit of a blocked climb


def _scene():
    from swarm_gb300 import venues
    from swarm_gb300.abi import fptr
    venue = venues.Venue.hall(20.0, 10.0, [(1, 0.0, 2.0)], name="step-up hall")
    v = venue.struct
    xs = v.wall_origin_x + np.arange(v.wall_nx, dtype=np.float64) * v.wall_h
    ys = v.wall_origin_y + np.arange(v.wall_ny, dtype=np.float64) * v.wall_h
    X, Y = np.meshgrid(xs, ys)
    ahead = (X >= 2.0) & (X <= 6.0)
    floor = np.where(ahead & (Y >= 0.25) & (Y <= 4.75), PLATFORM,
                     np.where(ahead & (Y >= -4.75) & (Y <= -0.25), STEP, 0.0)).astype(np.float32).ravel()
    venue.arrays["floor"] = floor
    v.floor_height = fptr(floor)
    b, r, v0 = venues.spawn_lattice(8, 8, spacing=1.0, center=(-2.0, 0.0), jitter=0.05, seed=3)
    drive = np.tile(np.array([[1.0, 0.0]], np.float32), (b.shape[0], 1))
    return venue, b, r, v0, drive


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_oracle_blocks_the_riser_and_climbs_the_step(built):
    """CPU: the 0.4 m platform is never climbed (the blocked moves carry the step-up bit); the 0.2 m step is."""
    import swarm_gb300
    venue, b, r, v0, drive = _scene()
    ora = O.OracleSim(swarm_gb300.params_si(), venue.struct)
    ora.set_state(b)
    ora.set_agent_params(r, v0)
    ora.set_drive_table(drive)
    blocked = np.zeros(b.shape[0], bool)
    for _ in range(20):
        ora.step(10)
        s = ora.state()
        blocked |= (ora.contacts() & STEP_UP) != 0
        on = s[:, 3] != 0
        feet = s[:, 2] - r
        # nobody stands more than 0.30 m above the ground the crowd started on
        assert (feet[on] < 0.30).all()
    s = ora.state()
    north, south = b[:, 1] > 0.0, b[:, 1] < 0.0
    assert blocked[north].sum() >= 8, "the platform's riser blocks the agents walking into it"
    assert not blocked[south].any(), "the 0.2 m step never blocks"
    climbed = south & (s[:, 3] != 0) & (np.abs(s[:, 2] - r - STEP) < 1e-4)
    passed = south & ((s[:, 3] == 0) | (s[:, 0] > 6.0))
    assert (climbed | passed).sum() >= 8, "agents climb the 0.2 m step (or have crossed it)"
    # nobody stands on the platform's footprint (agents that slid along its riser into the gap at |y| < 0.25 pass)
    act = s[:, 3] != 0
    on_platform = act & (s[:, 0] >= 1.975) & (s[:, 0] <= 6.025) & (s[:, 1] >= 0.225) & (s[:, 1] <= 4.775)
    assert not on_platform.any(), "nobody stands on the platform"


@pytest.mark.gpu
def test_step_up_gpu_vs_oracle(built):
    """GPU against the oracle, bit for bit, every 10 steps over 200 steps of the scene."""
    import swarm_gb300
    venue, b, r, v0, drive = _scene()
    P = swarm_gb300.params_si()
    sim = swarm_gb300.CrowdSim(P, venue, b.shape[0])
    sim.set_state(b)
    sim.set_agent_params(r, v0)
    sim.set_drive_table(drive)
    ora = O.OracleSim(P, venue.struct)
    ora.set_state(b)
    ora.set_agent_params(r, v0)
    ora.set_drive_table(drive)
    seen = 0
    for k in range(20):
        sim.step(10)
        ora.step(10)
        assert np.array_equal(_bits(sim.state()), _bits(ora.state())), f"after {10 * (k + 1)} steps"
        c = sim.contacts()
        assert np.array_equal(c, ora.contacts())
        seen += int(((c & STEP_UP) != 0).sum())
    assert seen > 0, "the scene exercises the limit"
