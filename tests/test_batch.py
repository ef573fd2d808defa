"""Batched instances (swarm_batch_create): many independent evacuations of uneven size packed into one segmented
state. Each instance's part of the batch must be bit-identical to the same instance run alone -- by the oracle, and
by the CUDA step on its own handle."""
import numpy as np
import pytest

from oracle import oracle as O


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def small_batch(built):
    from swarm_gb300 import venues
    return venues.build_batch(count=6, seed=3, n_lo=256, n_hi=3000)


def test_batch_spec_and_packing(small_batch):
    vens, boids, r, v0, counts = small_batch
    assert len(vens) == 6 and boids.shape[0] == counts.sum() == r.shape[0]
    assert counts.min() >= 256 and counts.max() <= 3000


@pytest.mark.gpu
@pytest.mark.parametrize("fused", [True, False])
def test_batch_instances_equal_solo_runs(small_batch, fused):
    import swarm_gb300
    vens, boids, r, v0, counts = small_batch
    P = swarm_gb300.params_si()
    batch = swarm_gb300.BatchSim(P, vens, counts)
    batch.set_fused(fused)
    batch.set_state(boids)
    batch.set_agent_params(r, v0)
    steps = 40
    batch.step(steps)
    out = batch.state()
    starts = batch.starts
    for i, v in enumerate(vens):
        a, b = starts[i], starts[i + 1]
        solo = swarm_gb300.CrowdSim(P, v, int(b - a))
        solo.set_state(boids[a:b])
        solo.set_agent_params(r[a:b], v0[a:b])
        solo.step(steps)
        assert np.array_equal(_bits(out[a:b]), _bits(solo.state())), f"instance {i}: batch != solo CUDA"
        if i < 3:
            ora = O.OracleSim(P, v.struct)
            ora.set_state(boids[a:b])
            ora.set_agent_params(r[a:b], v0[a:b])
            ora.step(steps)
            assert np.array_equal(_bits(out[a:b]), _bits(ora.state())), f"instance {i}: batch != oracle"


@pytest.mark.gpu
def test_launch_configurations_give_the_same_bits_and_autotune_restores_state(built):
    import swarm_gb300
    from swarm_gb300 import venues
    venue, (boids, r, v0) = venues.terrace_c0()
    P = swarm_gb300.params_si()
    ref = swarm_gb300.CrowdSim(P, venue, boids.shape[0])
    ref.set_state(boids)
    ref.set_agent_params(r, v0)
    ref.step(10)
    want = ref.state()
    for cfg in [(True, 128, 1), (True, 256, 2), (True, 512, 0), (False, 0, 0)]:
        sim = swarm_gb300.CrowdSim(P, venue, boids.shape[0])
        sim.set_state(boids)
        sim.set_agent_params(r, v0)
        sim.set_tuning(*cfg)
        sim.step(10)
        assert np.array_equal(_bits(sim.state()), _bits(want)), cfg
    sim = swarm_gb300.CrowdSim(P, venue, boids.shape[0])
    sim.set_state(boids)
    sim.set_agent_params(r, v0)
    with pytest.raises(swarm_gb300.SwarmError):   # below 64 threads a block: refused (the scan tiles' size)
        sim.set_tuning(True, 32, 0)
    best = sim.autotune(steps=2)
    assert best["ms_per_step"] > 0
    assert np.array_equal(_bits(sim.state()), _bits(boids))   # the trials' state is restored
    sim.step(10)
    assert np.array_equal(_bits(sim.state()), _bits(want))


@pytest.mark.gpu
def test_full_batch_256_instances_equal_solo_runs_and_oracle(built):
    """The batched workload at full size and length (256 halls, N log-uniform in [1 024, 65 536], 3.78 M agents,
    1 000 steps): every instance bit-identical to its solo CUDA run, and 8 instances (the 4 smallest, the 4 largest) to
    the oracle."""
    import swarm_gb300
    from swarm_gb300 import venues
    vens, boids, r, v0, counts = venues.build_batch(256, 0)
    assert len(vens) == 256 and counts.min() >= 1024 and counts.max() <= 65536
    P = swarm_gb300.params_si()
    steps = 1000
    batch = swarm_gb300.BatchSim(P, vens, counts)
    batch.set_state(boids)
    batch.set_agent_params(r, v0)
    batch.set_graph(True)
    batch.step(steps)
    out = batch.state()
    starts = batch.starts
    batch.close()
    order = np.argsort(counts, kind="stable")
    check_oracle = set(order[:4].tolist()) | set(order[-4:].tolist())
    for i, v in enumerate(vens):
        a, b = starts[i], starts[i + 1]
        solo = swarm_gb300.CrowdSim(P, v, int(b - a))
        solo.set_state(boids[a:b])
        solo.set_agent_params(r[a:b], v0[a:b])
        solo.step(steps)
        assert np.array_equal(_bits(out[a:b]), _bits(solo.state())), f"instance {i} ({b - a} agents): batch != solo"
        solo.close()
        if i in check_oracle:
            ora = O.OracleSim(P, v.struct)
            ora.set_state(boids[a:b])
            ora.set_agent_params(r[a:b], v0[a:b])
            ora.step(steps)
            assert np.array_equal(_bits(out[a:b]), _bits(ora.state())), f"instance {i}: batch != oracle"
