"""The CUDA adjoint (swarm_adjoint_run) against the gradient oracle (oracle/swarm_grad.cpp).

The adjoint differentiates the FP32 step with its branches frozen at the forward's choices. Its checker is the
oracle's Dual<float> run: the same FP32 trajectory (bit for bit the step), the same branches, tangents in double. A
directional derivative <grad, u> from the adjoint must match the dual's along u to GRAD_RTOL relative to the
direction's scale (the FP32 accumulation of the reverse pass is the only difference). The loss must match the
oracle's to 1e-9 relative (both sum D in double, in different orders). Gradients do not depend on the checkpoint
interval and repeat bit for bit. Against FP64 central differences (eps 1e-4): every single-agent parameter whose
perturbed runs keep the branch set of the FP32 run agrees to 1e-3 relative; on the 16 384-agent C4 hall, every
front agent whose perturbed runs keep their branches, save one whose FP32 and FP64 trajectories are shown to part.

Every call goes through the C ABI (swarm_gb300 is a ctypes layer over include/swarm_cuda.h)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-3


@pytest.fixture(scope="module")
def small(built):
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


def _gpu(P, venue, b, r, v0, steps, ckpt, stats=False, fused=True):
    import swarm_gb300
    sim = swarm_gb300.CrowdSim(P, venue, b.shape[0])
    sim.set_fused(fused)
    sim.set_state(b)
    sim.set_agent_params(r, v0)
    out = sim.adjoint(steps, ckpt, stats=stats)
    return sim, out


def _directions(n, rng, singles):
    z = np.zeros(n)
    dirs = [(z, z, 1.0), (z, rng.standard_normal(n), 0.0), (rng.standard_normal(n), z, 0.0),
            (rng.standard_normal(n), rng.standard_normal(n), 1.0)]
    for i in singles:
        e = np.zeros(n)
        e[i] = 1.0
        dirs.append((e, z, 0.0) if i % 2 else (z, e, 0.0))
    return dirs[:8]


def _check_against_dual(P, venue, b, r, v0, steps, ckpt, singles=(3, 10, 27, 44), seed=0, fused=True):
    n = b.shape[0]
    _, (L, gv, gr, gt) = _gpu(P, venue, b, r, v0, steps, ckpt, fused=fused)
    dirs = _directions(n, np.random.default_rng(seed), singles)
    dr = np.stack([d[0] for d in dirs]); dv = np.stack([d[1] for d in dirs]); dt = np.array([d[2] for d in dirs])
    L32, dl, _, _ = O.grad_eval(32, P, venue.struct, b, r, v0, P.tau_relax, steps, dirs=(dr, dv, dt))
    assert abs(L - L32) <= 1e-9 * abs(L32), (L, L32)
    got = dr @ gr.astype(np.float64) + dv @ gv.astype(np.float64) + dt * float(gt)
    # the scale of a direction: its derivative, or the gradient's size along it (a component near 0)
    scale = np.maximum(np.abs(dl), np.abs(dr) @ np.abs(gr) + np.abs(dv) @ np.abs(gv) + np.abs(dt) * abs(gt))
    err = np.abs(got - dl) / np.maximum(scale, 1e-12)
    assert err.max() <= GRAD_RTOL, f"directional derivatives {got} vs dual {dl}: rel err {err}"
    return gv, gr, gt


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "per-phase"])
@pytest.mark.parametrize("k", [8, 1, 0])
def test_adjoint_small_hall_matches_dual(small, k, fused):
    P, venue, b, r, v0 = small
    _check_against_dual(_with_k(P, k), venue, b, r, v0, steps=40, ckpt=7, fused=fused)


def test_adjoint_checkpoint_interval_and_repeatability(small):
    P, venue, b, r, v0 = small
    sim, (L1, gv1, gr1, gt1) = _gpu(P, venue, b, r, v0, 40, 40)
    before = sim.state()
    L2, gv2, gr2, gt2 = sim.adjoint(40, 1)
    L3, gv3, gr3, gt3 = sim.adjoint(40, 13)
    L4, gv4, gr4, gt4 = sim.adjoint(40, 13)
    assert np.array_equal(sim.state(), before), "the handle's state is left as it was"
    for gv, gr, gt, L in ((gv2, gr2, gt2, L2), (gv3, gr3, gt3, L3), (gv4, gr4, gt4, L4)):
        assert L == L1 and gt == gt1
        assert np.array_equal(gv, gv1) and np.array_equal(gr, gr1)


def test_adjoint_kept_tapes_give_the_same_gradient(small):
    """Two-level checkpointing: the checkpoint pass keeps the tapes of the last segments that the tape budget holds;
    every budget gives the same bits as recomputing every segment but the last."""
    P, venue, b, r, v0 = small
    sim, _ = _gpu(P, venue, b, r, v0, 40, 7)
    K = P.proj_iterations
    ncells = venue.struct.grid_res_x * venue.struct.grid_res_y
    step_bytes = (6 + max(K, 1) + K) * sim.n * 16 + sim.n * 17 + (ncells + 1 + 3) // 4 * 4 * 4
    runs = []
    for budget in (0, 2 * 7 * step_bytes, 1 << 30):
        sim.set_adjoint_tape_budget(budget)
        runs.append(sim.adjoint(40, 7, stats=True))
    assert [st["kept_segments"] for *_, st in runs] == [1, 3, 6] and runs[0][4]["segments"] == 6
    L0, gv0, gr0, gt0, _ = runs[0]
    for L, gv, gr, gt, _ in runs[1:]:
        assert L == L0 and gt == gt0
        assert np.array_equal(gv, gv0) and np.array_equal(gr, gr0)


def test_adjoint_terrace_4096(built):
    import swarm_gb300
    from swarm_gb300 import venues as V
    P = swarm_gb300.params_si()
    venue, (b, r, v0) = V.terrace_c0()
    gv, gr, gt = _check_against_dual(P, venue, b, r, v0, steps=60, ckpt=20, singles=(100, 2047, 3000, 4095))
    # the per-phase reverse sums each gather in one order, the fused one over 4 lanes: the same gradient to rounding
    _, (L2, gv2, gr2, gt2) = _gpu(P, venue, b, r, v0, 60, 20, fused=False)
    for a, c in ((gv, gv2), (gr, gr2)):
        assert np.abs(a - c).max() <= 1e-4 * np.abs(c).max()
    assert abs(gt - gt2) <= 1e-4 * abs(gt2)


def test_adjoint_vs_fp64_central_differences(small):
    """FP64 central differences, eps 1e-4, on single agents of the 64-agent hall: compared where the +-eps FP64 runs
    and the FP32 run all take one branch set (the FP32 and FP64 trajectories then differ by rounding only)."""
    P, venue, b, r, v0 = small
    n, steps, eps = b.shape[0], 40, 1e-4
    _, (L, gv, gr, gt) = _gpu(P, venue, b, r, v0, steps, 20)
    _, _, sig32, _ = O.grad_eval(32, P, venue.struct, b, r, v0, P.tau_relax, steps)
    _, _, sig64, _ = O.grad_eval(64, P, venue.struct, b, r, v0, P.tau_relax, steps)
    assert sig32 == sig64, "the FP32 and FP64 runs take one branch set over these steps"
    compared = 0
    for i in range(n):
        for which in ("v0", "r"):
            e = np.zeros(n)
            e[i] = eps
            rp, rm = (r + e, r - e) if which == "r" else (r, r)
            vp, vm = (v0 + e, v0 - e) if which == "v0" else (v0, v0)
            Lp, _, sp, _ = O.grad_eval(64, P, venue.struct, b, rp, vp, P.tau_relax, steps)
            Lm, _, sm, _ = O.grad_eval(64, P, venue.struct, b, rm, vm, P.tau_relax, steps)
            if not (sp == sig64 and sm == sig64):
                continue
            fd = (Lp - Lm) / (2 * eps)
            g = float(gr[i] if which == "r" else gv[i])
            compared += 1
            assert abs(g - fd) <= GRAD_RTOL * max(abs(fd), 1e-3), (i, which, g, fd)
    # the tau derivative
    Lp, _, sp, _ = O.grad_eval(64, P, venue.struct, b, r, v0, P.tau_relax + eps, steps)
    Lm, _, sm, _ = O.grad_eval(64, P, venue.struct, b, r, v0, P.tau_relax - eps, steps)
    if sp == sig64 and sm == sig64:
        fd = (Lp - Lm) / (2 * eps)
        assert abs(gt - fd) <= GRAD_RTOL * abs(fd), (gt, fd)
    assert compared >= 64, f"only {compared} single-agent parameters kept their branches"


def test_autograd_function(small):
    torch = pytest.importorskip("torch")
    import swarm_gb300
    from swarm_gb300.autograd import evacuation_loss
    P, venue, b, r, v0 = small
    sim = swarm_gb300.CrowdSim(P, venue, b.shape[0])
    vt = torch.tensor(v0, dtype=torch.float64, requires_grad=True)
    rt = torch.tensor(r, dtype=torch.float64, requires_grad=True)
    tt = torch.tensor(float(P.tau_relax), dtype=torch.float64, requires_grad=True)
    loss = evacuation_loss(sim, b, vt, rt, tt, steps=30, ckpt_every=10)
    loss.backward()
    _, (L, gv, gr, gt) = _gpu(P, venue, b, r, v0, 30, 10)
    assert float(loss.detach()) == L
    assert np.array_equal(vt.grad.numpy(), gv.astype(np.float64))
    assert np.array_equal(rt.grad.numpy(), gr.astype(np.float64))
    assert float(tt.grad) == float(np.float32(gt))


@pytest.fixture(scope="module")
def hall_c4(built):
    import swarm_gb300
    from swarm_gb300 import venues as V
    venue, (b, r, v0) = V.terrace_c4()
    return swarm_gb300.params_si(), venue, b, r, v0


def test_adjoint_c4_400_steps_matches_dual(hall_c4):
    """The specified workload in full (16 384 agents, 400 steps, checkpoints every 20): the adjoint is the exact
    derivative of the FP32 step with the forward's branches, to GRAD_RTOL, even where the congested crowd amplifies
    tangents by orders of magnitude."""
    P, venue, b, r, v0 = hall_c4
    n, steps = b.shape[0], 400
    _, (L, gv, gr, gt) = _gpu(P, venue, b, r, v0, steps, 20)
    rng = np.random.default_rng(7)
    z = np.zeros(n)
    e = np.zeros(n)
    e[int(np.argmax(np.abs(gv)))] = 1.0
    dr = np.stack([z, rng.standard_normal(n), z, z])
    dv = np.stack([z, z, rng.standard_normal(n), e])
    dt = np.array([1.0, 0.0, 0.0, 0.0])
    L32, dl, _, _ = O.grad_eval(32, P, venue.struct, b, r, v0, P.tau_relax, steps, dirs=(dr, dv, dt))
    assert abs(L - L32) <= 1e-9 * abs(L32)
    got = dr @ gr.astype(np.float64) + dv @ gv.astype(np.float64) + dt * float(gt)
    err = np.abs(got - dl) / np.abs(dl)
    assert err.max() <= GRAD_RTOL, f"{got} vs {dl}: {err}"


def _c4_front_fd(P, venue, b, r, v0, steps, eps=1e-4):
    """FP64 central differences on the desired speed of the 16 agents at the crowd's front (the lattice columns
    nearest the exits, walking freely; inside the lattice the headway clamp makes dL/dv0 exactly 0), with the FP64
    dual along the same 16 directions. Returns (agents, kept: the +-eps FP64 runs took the FP64 run's branches, fd,
    the FP64 dual)."""
    n = b.shape[0]
    _, _, sig64, _ = O.grad_eval(64, P, venue.struct, b, r, v0, P.tau_relax, steps)
    front = np.argsort(-np.abs(b[:, 0]) + 0.2 * np.abs(b[:, 1]))[:16]
    d64 = np.zeros(16)
    for c in range(0, 16, 8):
        dv = np.zeros((8, n))
        dv[np.arange(8), front[c:c + 8]] = 1.0
        _, dl, _, _ = O.grad_eval(64, P, venue.struct, b, r, v0, P.tau_relax, steps, dirs=(np.zeros((8, n)), dv, np.zeros(8)))
        d64[c:c + 8] = dl
    kept, fd = np.zeros(16, bool), np.zeros(16)
    for k, i in enumerate(front):
        d = np.zeros(n)
        d[i] = eps
        Lp, _, sp, _ = O.grad_eval(64, P, venue.struct, b, r, v0 + d, P.tau_relax, steps)
        Lm, _, sm, _ = O.grad_eval(64, P, venue.struct, b, r, v0 - d, P.tau_relax, steps)
        kept[k] = sp == sig64 and sm == sig64
        fd[k] = (Lp - Lm) / (2 * eps)
    return front, kept, fd, d64


def test_adjoint_c4_vs_fp64_central_differences_20_steps(hall_c4):
    """The C4 hall (16 384 agents), 20 steps: every front agent whose +-eps FP64 runs keep their branches agrees with
    FP64 central differences (eps 1e-4) to GRAD_RTOL (measured: 2.7e-5 at most)."""
    P, venue, b, r, v0 = hall_c4
    steps = 20
    _, (L, gv, gr, gt) = _gpu(P, venue, b, r, v0, steps, 20)
    front, kept, fd, _ = _c4_front_fd(P, venue, b, r, v0, steps)
    assert kept.sum() >= 12, f"only {kept.sum()} of 16 kept their branches"
    err = np.abs(gv[front].astype(np.float64) - fd) / np.abs(fd)
    assert err[kept].max() <= GRAD_RTOL, list(zip(front[kept], err[kept]))


def test_adjoint_c4_vs_fp64_central_differences(hall_c4):
    """The C4 hall, 40 steps: every front agent whose +-eps FP64 runs keep their branches agrees with FP64 central
    differences (eps 1e-4) to GRAD_RTOL, except where the FP32 trajectory has parted from the FP64 one. Such an agent
    is excluded only with the proof of both halves: the FP64 dual matches FD to 1e-5 (FD is the FP64 program's
    derivative) and the adjoint matches the FP32 dual to GRAD_RTOL (it is the FP32 program's derivative), while the
    two duals differ by more than GRAD_RTOL (over 16 384 agents the FP32 and FP64 runs part at a few near-tie
    decisions). Measured: one of the 14 kept agents (1.3e-3), the rest within 8.4e-5."""
    P, venue, b, r, v0 = hall_c4
    n, steps = b.shape[0], 40
    _, (L, gv, gr, gt) = _gpu(P, venue, b, r, v0, steps, 20)
    front, kept, fd, d64 = _c4_front_fd(P, venue, b, r, v0, steps)
    assert kept.sum() >= 12, f"only {kept.sum()} of 16 kept their branches"
    g = gv[front].astype(np.float64)
    err = np.abs(g - fd) / np.abs(fd)
    over = kept & (err > GRAD_RTOL)
    if over.any():
        idx = np.flatnonzero(over)
        dv = np.zeros((len(idx), n))
        dv[np.arange(len(idx)), front[idx]] = 1.0
        _, d32, _, _ = O.grad_eval(32, P, venue.struct, b, r, v0, P.tau_relax, steps,
                                   dirs=(np.zeros_like(dv), dv, np.zeros(len(idx))))
        for j, k in enumerate(idx):
            why = (front[k], g[k], fd[k], d64[k], d32[j])
            assert abs(d64[k] - fd[k]) <= 1e-5 * abs(fd[k]), why
            assert abs(g[k] - d32[j]) <= GRAD_RTOL * abs(d32[j]), why
            assert abs(d32[j] - d64[k]) > GRAD_RTOL * abs(d64[k]), why
    assert over.sum() <= 2, list(zip(front[over], err[over]))
