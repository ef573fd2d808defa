"""The key sort without device allocation (swarm_sort_grid_noalloc): for callers that cannot allocate device memory
while they run, e.g. a plug-in step in a host frame loop (where cudaMalloc / cudaFree may synchronise the device) or a
deployment that fixes its whole footprint at start-up. Called
through the C ABI on device arrays, it must give exactly the step's own sort (the sorted pairs and the cell table
that swarm_get_grid / swarm_get_cells return), on two calls in a row, whose shared working array keeps the first
call's contents. Integer outputs: the comparison is exact."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, state, venue, torch):
    v = venue.struct
    n = state.shape[0]
    d_state = torch.from_numpy(np.ascontiguousarray(state)).cuda()
    ncells = v.grid_res_x * v.grid_res_y
    d_grid = torch.empty(n, dtype=torch.int32, device="cuda")
    d_ids = torch.empty(n, dtype=torch.int32, device="cuda")
    d_cells = torch.empty(2 * ncells, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    f = lib.swarm_sort_grid_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    rc = f(d_state.data_ptr(), n, v.grid_res_x, v.grid_res_y, v.domain_min_x, v.domain_min_y, v.domain_span_x,
           v.domain_span_y, d_grid.data_ptr(), d_ids.data_ptr(), d_cells.data_ptr(), stream)
    assert rc == 0
    torch.cuda.synchronize()
    return (d_grid.cpu().numpy().view(np.uint32), d_ids.cpu().numpy().view(np.uint32),
            d_cells.cpu().numpy().view(np.uint32).reshape(-1, 2))


def _step_sort(P, venue, state, radius=None, v0=None):
    import swarm_gb300
    sim = swarm_gb300.CrowdSim(P, venue, state.shape[0])
    sim.set_state(state)
    if radius is not None:
        sim.set_agent_params(radius, v0)
    sim.step(1)
    return sim.grid() + (sim.cells(),)


def test_noalloc_sort_equals_the_step_sort_on_two_calls(built, stadium_sdf, terrace_golden):
    import torch
    import swarm_gb300
    from swarm_gb300 import venues
    from swarm_gb300.venues import Venue
    lib = swarm_gb300.lib()

    # first call: the 65 536-agent hall (78 400 cells)
    hall, (boids, r, v0) = venues.hall_c1()
    want = _step_sort(swarm_gb300.params_si(), hall, boids, r, v0)
    got = _noalloc(lib, boids, hall, torch)
    for w, g in zip(want, got):
        assert np.array_equal(w, g)

    # second call, on the array the first left behind: the terrace with evacuated agents and a NaN position
    terrace = Venue.stadium(stadium_sdf)
    st = terrace_golden["state250"].copy()
    st[3, :4] = [np.nan, np.nan, np.nan, 1.0]
    st[100:160, 3] = 0.0
    st[100:160, :3] = 1000.0
    want = _step_sort(swarm_gb300.params_reference(), terrace, st)
    got = _noalloc(lib, st, terrace, torch)
    for w, g in zip(want, got):
        assert np.array_equal(w, g)


def test_noalloc_rejects_sizes_beyond_its_limit(built):
    import swarm_gb300
    lib = swarm_gb300.lib()
    f = lib.swarm_sort_grid_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    dummy = C.c_void_p(16)   # never dereferenced: the size and alignment checks come first
    assert f(dummy, 65537, 10, 10, 0.0, 0.0, 1.0, 1.0, dummy, dummy, dummy, None) == -1
    assert f(dummy, 100, 400, 400, 0.0, 0.0, 1.0, 1.0, dummy, dummy, dummy, None) == -1
    # a state that is not 16-byte aligned (it is read as float4) is refused before any launch
    assert f(C.c_void_p(24), 100, 10, 10, 0.0, 0.0, 1.0, 1.0, dummy, dummy, dummy, None) == -1
