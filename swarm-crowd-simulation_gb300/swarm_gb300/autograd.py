"""torch.autograd binding of the adjoint (swarm_adjoint_run): gradient checks and parameter calibration.

    loss = evacuation_loss(sim, state, v0, radius, tau, steps=400, ckpt_every=20)
    loss.backward()          # v0.grad, radius.grad, tau.grad

The forward sets the parameters on the simulation, uploads the start state and runs the adjoint (forward and
reverse together: the gradient is computed with the loss and kept for backward). Float64 parameter tensors are
rounded to float32 for the step. CPU or CUDA tensors; the gradients come back on the parameters' device.
"""
import numpy as np
import torch


class EvacuationLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, v0, radius, tau, sim, state, steps, ckpt_every):
        v = v0.detach().to("cpu", torch.float32).numpy()
        r = radius.detach().to("cpu", torch.float32).numpy()
        sim.set_state(state)
        sim.set_agent_params(r, v)
        sim.set_relaxation_time(float(tau.detach().cpu()))
        L, gv, gr, gt = sim.adjoint(int(steps), int(ckpt_every))
        ctx.save_for_backward(torch.from_numpy(gv).to(v0.device, v0.dtype), torch.from_numpy(gr).to(radius.device, radius.dtype),
                              torch.tensor(gt, dtype=tau.dtype, device=tau.device))
        return torch.tensor(L, dtype=torch.float64, device=v0.device)

    @staticmethod
    def backward(ctx, gL):
        gv, gr, gt = ctx.saved_tensors
        g = gL.to(gv.dtype)
        return g * gv, g * gr, (gL.to(gt.dtype) * gt).reshape(gt.shape), None, None, None, None


def evacuation_loss(sim, state, v0, radius, tau, steps, ckpt_every=20):
    """L = dt * sum_t sum_i D(p_i(t)) over `steps` steps from `state` (an (n, 8) float32 array), differentiable in
    v0 (n,), radius (n,) and tau (a 0-d tensor)."""
    state = np.ascontiguousarray(state, dtype=np.float32)
    return EvacuationLoss.apply(v0, radius, tau, sim, state, steps, ckpt_every)
