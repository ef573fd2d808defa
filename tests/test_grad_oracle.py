"""The gradient oracle (oracle/swarm_grad.cpp), the checker of the CUDA adjoint, checked on the CPU.

Its float instantiation must be the step: bit for bit the oracle's end state. Its dual numbers must be derivatives:
they match FP64 central finite differences wherever the perturbed runs take the primal run's branches (equal branch
signatures), at eps 1e-6 to 1e-6 relative, and at the specified eps 1e-4 on single agents to 1e-4 relative."""
import numpy as np
import pytest

from oracle import oracle as O


@pytest.fixture(scope="module")
def small(built):
    """64 agents on an 8 x 8 lattice (0.9 m) walking to a 2 m door of a 12 m x 10 m hall: pair contacts, wall contacts
    at the door posts and obstacle pushes, no evacuation within 40 steps."""
    import swarm_gb300
    from swarm_gb300.venues import Venue, spawn_lattice
    P = swarm_gb300.params_si()
    venue = Venue.hall(12.0, 10.0, [(1, 0.0, 2.0)], name="hall 12x10 m, 1 door")
    b, r, v0 = spawn_lattice(8, 8, spacing=0.9, center=(-1.0, 0.0), seed=3)
    return P, venue, b, r, v0


def _with_k(P, k):
    import ctypes
    q = type(P)()
    ctypes.memmove(ctypes.byref(q), ctypes.byref(P), ctypes.sizeof(P))
    q.proj_iterations = k
    return q


def _oracle_state(P, venue, b, r, v0, steps):
    sim = O.OracleSim(P, venue.struct)
    sim.set_state(b)
    sim.set_agent_params(r, v0)
    sim.step(steps)
    return sim.state()


def test_float_instantiation_is_the_step(built):
    import swarm_gb300
    from swarm_gb300 import venues as V
    P = swarm_gb300.params_si()
    venue, (b, r, v0) = V.terrace_c0()
    ref = _oracle_state(P, venue, b, r, v0, 25)
    _, _, sig, st = O.grad_eval(32, P, venue.struct, b, r, v0, P.tau_relax, 25, want_state=True)
    assert np.array_equal(st.view(np.uint32), ref.view(np.uint32))
    n = b.shape[0]
    rng = np.random.default_rng(5)
    dirs = (rng.standard_normal((2, n)), rng.standard_normal((2, n)), np.array([1.0, 0.0]))
    _, _, sig2, st2 = O.grad_eval(32, P, venue.struct, b, r, v0, P.tau_relax, 25, dirs=dirs, want_state=True)
    assert np.array_equal(st2.view(np.uint32), ref.view(np.uint32)), "the dual's float primal is the step"
    assert sig2 == sig


@pytest.mark.parametrize("k", [0, 1, 8])
def test_float_instantiation_sweep_counts(small, k):
    P, venue, b, r, v0 = small
    Pk = _with_k(P, k)
    ref = _oracle_state(Pk, venue, b, r, v0, 40)
    _, _, _, st = O.grad_eval(32, Pk, venue.struct, b, r, v0, Pk.tau_relax, 40, want_state=True)
    assert np.array_equal(st.view(np.uint32), ref.view(np.uint32))


def _fd64(P, venue, b, r, v0, steps, d, eps):
    dr, dv, dt = d
    Lp, _, sp, _ = O.grad_eval(64, P, venue.struct, b, r + eps * dr, v0 + eps * dv, P.tau_relax + eps * dt, steps)
    Lm, _, sm, _ = O.grad_eval(64, P, venue.struct, b, r - eps * dr, v0 - eps * dv, P.tau_relax - eps * dt, steps)
    return (Lp - Lm) / (2.0 * eps), sp, sm


def test_dual_matches_central_differences(small):
    P, venue, b, r, v0 = small
    n, steps = b.shape[0], 40
    rng = np.random.default_rng(1)
    z = np.zeros(n)
    dirs = [(z, z, 1.0), (z, rng.standard_normal(n), 0.0), (rng.standard_normal(n), z, 0.0),
            (rng.standard_normal(n), rng.standard_normal(n), 1.0)]
    dr = np.stack([d[0] for d in dirs]); dv = np.stack([d[1] for d in dirs]); dt = np.array([d[2] for d in dirs])
    _, dl, sig, _ = O.grad_eval(64, P, venue.struct, b, r, v0, P.tau_relax, steps, dirs=(dr, dv, dt))
    for k in range(len(dirs)):
        fd, sp, sm = _fd64(P, venue, b, r, v0, steps, (dr[k], dv[k], dt[k]), 1e-6)
        assert sp == sig and sm == sig, f"direction {k}: a branch flipped at eps 1e-6"
        assert abs(dl[k] - fd) <= 1e-6 * abs(fd), (k, dl[k], fd)


def test_dual_matches_fd_at_eps_1e4_single_agents(small):
    """The specified check (FP64 central differences, eps 1e-4) on single-agent parameters: wherever the +-eps runs
    keep the primal branch set, the derivative agrees to 1e-4 relative; most agents keep it over 40 steps."""
    P, venue, b, r, v0 = small
    n, steps, eps = b.shape[0], 40, 1e-4
    agents = list(range(0, n, 4))
    kept = 0
    for i in agents:
        for which in ("v0", "r"):
            e = np.zeros(n)
            e[i] = 1.0
            z = np.zeros(n)
            d = (e, z, 0.0) if which == "r" else (z, e, 0.0)
            _, dl, sig, _ = O.grad_eval(64, P, venue.struct, b, r, v0, P.tau_relax, steps,
                                        dirs=(d[0][None], d[1][None], np.array([d[2]])))
            fd, sp, sm = _fd64(P, venue, b, r, v0, steps, d, eps)
            if sp == sig and sm == sig:
                kept += 1
                assert abs(dl[0] - fd) <= 1e-4 * abs(fd) + 1e-9, (i, which, dl[0], fd)
    assert kept >= len(agents), f"only {kept} of {2 * len(agents)} single-agent perturbations kept their branches"
