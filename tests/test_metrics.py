"""Safety metrics (metrics_deposit / metrics_finalize; the reference's MetricsReference, src/metrics.cpp:429-476):
evacuation events per exit, fixed-point cloud-in-cell density and speed mass, per-cell accumulators. Integer results:
every comparison is exact."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as O


@pytest.fixture(scope="module")
def metrics_golden():
    return dict(np.load(os.path.join(GOLDEN, "terrace_metrics_ref.npz")))


def _terrace(stadium_sdf):
    import swarm_gb300
    from swarm_gb300.venues import Venue
    return swarm_gb300.params_reference(), Venue.stadium(stadium_sdf)


def test_oracle_metrics_match_the_reference_over_250_terrace_steps(built, stadium_sdf, terrace_golden, metrics_golden):
    P, venue = _terrace(stadium_sdf)
    g = metrics_golden
    sim = O.OracleSim(P, venue.struct)
    sim.set_state(terrace_golden["spawn"])
    met = O.OracleMetrics(P, venue.struct, 64, g["threshold_mass"], 4096)
    prev = terrace_golden["spawn"]
    for _ in range(250):
        sim.step(1)
        cur = sim.state()
        met.record(prev, cur)
        prev = cur
    ctr, cells, evac = met.read()
    assert np.array_equal(ctr, g["counters"]) and ctr[2] > 0   # agents did leave, through the avenue gaps
    assert np.array_equal(cells, g["cells"])
    assert np.array_equal(evac, g["evac_step"])


def test_grid_thresholds(built):
    from swarm_gb300 import venues
    venue, _ = venues.terrace_c0()
    res, thr = venue.metric_thresholds()
    assert res % 16 == 0 and thr.shape == (res * res, 4)
    t = thr.reshape(res, res, 4)
    mid = res // 2
    # a full interior cell: 1 m^2 walkable -> ceil(1.08 * 65536), ceil(2.17 * 65536), 5 * 65536
    assert list(t[mid, mid, :3]) == [70779, 142214, 327680] and t[mid, mid, 3] == 0xFFFFFFFF
    assert (t[0, 0, :] == 0xFFFFFFFF).all()    # beyond the exit line: no floor


@pytest.mark.gpu
def test_gpu_metrics_terrace_vs_reference_fixture(built, stadium_sdf, terrace_golden, metrics_golden):
    import swarm_gb300
    P, venue = _terrace(stadium_sdf)
    g = metrics_golden
    sim = swarm_gb300.CrowdSim(P, venue, 4096)
    sim.set_state(terrace_golden["spawn"])
    sim.metrics_enable(64, g["threshold_mass"])
    sim.step(250)
    ctr, cells, evac = sim.metrics()
    assert np.array_equal(np.frombuffer(bytes(ctr), np.uint32), g["counters"])
    assert np.array_equal(cells, g["cells"])
    assert np.array_equal(evac, g["evac_step"])


@pytest.mark.gpu
@pytest.mark.parametrize("fused", [True, False])
def test_gpu_metrics_grid_terrace_vs_oracle(built, fused):
    import swarm_gb300
    from swarm_gb300 import venues
    venue, (boids, r, v0) = venues.terrace_c0()
    P = swarm_gb300.params_si()
    res, thr = venue.metric_thresholds()
    sim = swarm_gb300.CrowdSim(P, venue, boids.shape[0])
    sim.set_fused(fused)
    sim.set_state(boids)
    sim.set_agent_params(r, v0)
    sim.metrics_enable(res, thr)
    ora = O.OracleSim(P, venue.struct)
    ora.set_state(boids)
    ora.set_agent_params(r, v0)
    met = O.OracleMetrics(P, venue.struct, res, thr, boids.shape[0])
    prev = boids
    for _ in range(300):
        ora.step(1)
        cur = ora.state()
        met.record(prev, cur)
        prev = cur
    sim.step(300)
    ctr, cells, evac = sim.metrics()
    octr, ocells, oevac = met.read()
    assert np.array_equal(np.frombuffer(bytes(ctr), np.uint32), octr) and octr[2] > 0
    assert np.array_equal(cells, ocells)
    assert np.array_equal(evac, oevac)


@pytest.mark.gpu
@pytest.mark.parametrize("fused", [True, False])
def test_evacuation_runner_leaves_the_metrics_of_its_exact_run(built, stadium_sdf, terrace_golden, metrics_golden, fused):
    """swarm_run_evacuation checks the count every 256 steps and rolls the chunk in which the crowd empties back to
    that step: the state and the metrics it leaves are those of exactly t100 steps (2 696 on the reference terrace),
    bit for bit."""
    import swarm_gb300
    P, venue = _terrace(stadium_sdf)
    g = metrics_golden

    def fresh():
        sim = swarm_gb300.CrowdSim(P, venue, 4096)
        sim.set_fused(fused)
        sim.set_state(terrace_golden["spawn"])
        sim.metrics_enable(64, g["threshold_mass"])
        return sim

    a = fresh()
    stats, active = a.run_evacuation(4000)
    assert stats["steps"] == 2696 and stats["t100_step"] == 2696 and active[-1] == 0 and (active[:-1] > 0).all()
    b = fresh()
    b.step(2696)
    assert np.array_equal(a.state().view(np.uint32), b.state().view(np.uint32))
    (actr, acells, aevac), (bctr, bcells, bevac) = a.metrics(), b.metrics()
    assert bytes(actr) == bytes(bctr)
    assert np.array_equal(acells, bcells) and np.array_equal(aevac, bevac)
    # and the run goes on from there as the stepped one does
    a.step(3)
    b.step(3)
    assert np.array_equal(a.state().view(np.uint32), b.state().view(np.uint32))
    assert np.array_equal(a.metrics()[1], b.metrics()[1])
