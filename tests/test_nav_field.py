"""The navigation-field solver: first-order fast marching on the host and its GPU form (tiled relaxation to the fixed
point of the same FP64 update). The GPU field must equal the host field float for float: on random mazes with random
speed factors, on a serpentine corridor that needs many tile passes, and on the workloads' own venues (the 140 m hall
and the seated bowl), built through the venue builders with the GPU solver selected."""
import numpy as np
import pytest


def _maze(nx, ny, seed, walls=0.25, speeds=True, sources=3):
    rng = np.random.default_rng(seed)
    kind = np.where(rng.random((ny, nx)) < walls, 3, 0).astype(np.uint8)
    for _ in range(sources):
        kind[rng.integers(0, ny), rng.integers(0, nx)] = 1
    speed = rng.uniform(0.3, 1.5, (ny, nx)).astype(np.float32) if speeds else None
    return kind, speed


def _serpentine(nx, ny, corridor=6, wall=2):
    """Horizontal corridors joined at alternating ends: the one path from the source winds through every corridor."""
    kind = np.zeros((ny, nx), np.uint8)
    y, k = corridor, 0
    while y + wall < ny:
        kind[y:y + wall, :] = 3
        gap = slice(nx - corridor, nx) if k % 2 == 0 else slice(0, corridor)
        kind[y:y + wall, gap] = 0
        y += wall + corridor
        k += 1
    kind[0, 0] = 1
    return kind


# ---- the host solver (no GPU) ----

def test_plane_front_is_the_running_sum_of_steps(built):
    import swarm_gb300
    kind = np.zeros((20, 50), np.uint8)
    kind[:, 0] = 1
    out, _ = swarm_gb300.nav_field(kind, 0.1, solver="cpu")
    want = np.cumsum(np.r_[0.0, np.full(49, 0.1)]).astype(np.float32)
    assert np.array_equal(out, np.broadcast_to(want, out.shape))
    # a speed factor divides the local step: half speed, twice the travel distance per node
    out2, _ = swarm_gb300.nav_field(kind, 0.1, speed=np.full((20, 50), 0.5, np.float32), solver="cpu")
    want2 = np.cumsum(np.r_[0.0, np.full(49, 0.1 / 0.5)]).astype(np.float32)
    assert np.array_equal(out2[7], want2)


def test_walls_and_unreached_nodes_get_the_largest_distance_plus_10(built):
    import swarm_gb300
    kind = np.zeros((10, 30), np.uint8)
    kind[:, 0] = 1
    kind[:, 15] = 3          # a wall across the grid: nothing beyond it is reached
    out, _ = swarm_gb300.nav_field(kind, 0.1, solver="cpu")
    top = np.float32(np.cumsum(np.r_[0.0, np.full(14, 0.1)])[-1] + 10.0)
    assert (out[:, 15:] == top).all()
    assert out[:, :15].max() < 2.0


def test_invalid_arguments(built):
    import swarm_gb300
    kind = np.zeros((4, 4), np.uint8)
    kind[0, 0] = 1
    speed = np.ones((4, 4), np.float32)
    speed[2, 2] = 0.0        # a free node must be passable
    with pytest.raises(swarm_gb300.SwarmError):
        swarm_gb300.nav_field(kind, 0.1, speed=speed, solver="cpu")
    with pytest.raises(swarm_gb300.SwarmError):
        swarm_gb300.nav_field(np.zeros((1, 4), np.uint8), 0.1, solver="cpu")
    with pytest.raises(ValueError):
        swarm_gb300.set_nav_solver("fast")


# ---- the GPU solver against the host solver ----

@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_gpu_equals_fast_marching_on_random_mazes(built, seed):
    import swarm_gb300
    nx, ny = (333, 171) if seed % 2 else (128, 256)
    kind, speed = _maze(nx, ny, seed, speeds=seed != 3)
    cpu, _ = swarm_gb300.nav_field(kind, 0.1, speed=speed, solver="cpu")
    gpu, st = swarm_gb300.nav_field(kind, 0.1, speed=speed, solver="gpu")
    assert np.array_equal(cpu.view(np.uint32), gpu.view(np.uint32))
    assert st["passes"] > 0 and st["tile_runs"] >= st["tiles"]


@pytest.mark.gpu
def test_gpu_equals_fast_marching_on_a_serpentine(built):
    """A path that crosses the grid 40 times: the front re-enters most tiles many times."""
    import swarm_gb300
    kind = _serpentine(640, 320)
    cpu, _ = swarm_gb300.nav_field(kind, 0.05, solver="cpu")
    gpu, st = swarm_gb300.nav_field(kind, 0.05, solver="gpu")
    assert np.array_equal(cpu.view(np.uint32), gpu.view(np.uint32))
    assert st["tile_runs"] > 4 * st["tiles"]


@pytest.mark.gpu
def test_gpu_solver_builds_the_workload_venues(built):
    """The 140 m hall (2.1 M nav nodes) and the seated bowl (15.5 M nav nodes, speed-weighted: stairs at 0.6, nodes
    within 0.2 m of a wall blocked) built with the GPU solver: the same nav field as the host build."""
    import swarm_gb300
    from swarm_gb300 import venues
    for build in (venues.hall_c1, venues.bowl_c2):
        prev = swarm_gb300.set_nav_solver("cpu")
        try:
            host = build()[0].arrays["nav"]
            swarm_gb300.set_nav_solver("gpu")
            dev = build()[0].arrays["nav"]
        finally:
            swarm_gb300.set_nav_solver(prev)
        assert np.array_equal(host.view(np.uint32), dev.view(np.uint32))
