"""swarm_step_host, the call for callers that hold the state in host memory, through the C ABI.

With pinned buffers and the fused step it moves no copies: the hash phase reads the caller's input over the coherent
host link and the final pass writes the caller's output. With pageable buffers (or the per-phase kernels) it copies
each way. Every form must give the same bits as uploading the state and stepping the device state."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def scene(built):
    import swarm_gb300
    from swarm_gb300 import venues
    venue, (b, r, v0) = venues.terrace_c0()
    b = b.copy()
    b[7, 0] = np.nan       # the hash's NaN sanitiser
    b[11, 3] = 0.0         # an agent evacuated before the call
    return swarm_gb300.params_si(), venue, b, r, v0


def _device_reference(P, venue, b, r, v0, steps):
    import swarm_gb300
    sim = swarm_gb300.CrowdSim(P, venue, b.shape[0])
    sim.set_agent_params(r, v0)
    sim.set_state(b)
    sim.step(steps)
    out = sim.state().copy()
    sim.close()
    return out


@pytest.mark.parametrize("steps", [1, 3])
@pytest.mark.parametrize("fused", [True, False])
def test_step_host_pinned_and_pageable_match_the_device_path(scene, steps, fused):
    import torch
    import swarm_gb300
    P, venue, b, r, v0 = scene
    n = b.shape[0]
    ref = _device_reference(P, venue, b, r, v0, steps)
    sim = swarm_gb300.CrowdSim(P, venue, n)
    sim.set_agent_params(r, v0)
    sim.set_fused(fused)
    # pinned: the direct path (fused) or the copies (per-phase)
    h_in = torch.from_numpy(b.copy()).pin_memory()
    h_out = torch.zeros_like(h_in).pin_memory()
    sim.step_host(h_in.data_ptr(), h_out.data_ptr(), n, steps)
    assert np.array_equal(_bits(h_out.numpy()), _bits(ref))
    assert np.array_equal(_bits(sim.state()), _bits(ref)), "the device state holds the result too"
    # pageable numpy buffers: the copies
    p_in, p_out = b.copy(), np.zeros_like(b)
    sim.step_host(p_in.ctypes.data, p_out.ctypes.data, n, steps)
    assert np.array_equal(_bits(p_out), _bits(ref))
    sim.close()


def test_step_host_reports_a_barrier_timeout(scene):
    """A grid barrier that gives up ends the fused launch before the copy into the caller's pinned output: the call
    must return SWARM_E_TIMEOUT (-4), not success with a stale output, and the handle must step normally after."""
    import torch
    import swarm_gb300
    P, venue, b, r, v0 = scene
    n = b.shape[0]
    ref = _device_reference(P, venue, b, r, v0, 1)
    sim = swarm_gb300.CrowdSim(P, venue, n)
    sim.set_agent_params(r, v0)
    lib = swarm_gb300.lib()
    h_in = torch.from_numpy(b.copy()).pin_memory()
    h_out = torch.zeros_like(h_in).pin_memory()
    assert lib.swarm_test_barrier_timeout(sim._h) == 0
    assert lib.swarm_step_host(sim._h, h_in.data_ptr(), h_out.data_ptr(), n, 1) == -4
    assert lib.swarm_step_host(sim._h, h_in.data_ptr(), h_out.data_ptr(), n, 1) == 0
    assert np.array_equal(_bits(h_out.numpy()), _bits(ref))
    sim.close()


def test_step_host_in_place_and_continued_on_the_device(scene):
    """One pinned buffer as input and output, twice in a row, then two device steps: the same bits as five device
    steps from the start."""
    import torch
    import swarm_gb300
    P, venue, b, r, v0 = scene
    n = b.shape[0]
    ref = _device_reference(P, venue, b, r, v0, 5)
    sim = swarm_gb300.CrowdSim(P, venue, n)
    sim.set_agent_params(r, v0)
    buf = torch.from_numpy(b.copy()).pin_memory()
    sim.step_host(buf.data_ptr(), buf.data_ptr(), n, 2)
    sim.step_host(buf.data_ptr(), buf.data_ptr(), n, 1)
    sim.step(2)
    assert np.array_equal(_bits(sim.state()), _bits(ref))
    sim.close()


def test_step_host_pinned_buffers_off_the_32_byte_grid(scene):
    """Pinned buffers whose rows start 16 bytes off a 32-byte boundary (rows split across the host link's 32-byte
    sectors): the same bits."""
    import torch
    import swarm_gb300
    P, venue, b, r, v0 = scene
    n = b.shape[0]
    ref = _device_reference(P, venue, b, r, v0, 2)
    sim = swarm_gb300.CrowdSim(P, venue, n)
    sim.set_agent_params(r, v0)
    h_in = torch.zeros(n * 8 + 4, dtype=torch.float32).pin_memory()
    h_out = torch.zeros(n * 8 + 4, dtype=torch.float32).pin_memory()
    assert h_in.data_ptr() % 32 == 0 and h_out.data_ptr() % 32 == 0
    h_in[4:] = torch.from_numpy(b.reshape(-1))
    sim.step_host(h_in.data_ptr() + 16, h_out.data_ptr() + 16, n, 2)
    assert np.array_equal(_bits(h_out[4:].numpy().reshape(n, 8)), _bits(ref))
    sim.close()
