"""torch.autograd.Function over the CUDA adjoint (tea_gb300_adjoint_*).

The library does all of the work: the forward model is TeaLeaf's CG
timestep run by the C ABI, and the gradient comes from its adjoint kernels.
This module only moves tensors across the boundary so that torch's gradient
checks (and any torch optimiser) can drive it.
"""
import torch

from . import lib


class TimeSteppedLoss(torch.autograd.Function):
    """loss = 0.5*||u_T(exp(log_density)) - u_obs||^2 for `cfg.steps`
    TeaLeaf timesteps from energy0.  Differentiable in log_density only."""

    @staticmethod
    def forward(ctx, log_density, energy0, u_obs, adj, cfg):
        density = torch.exp(log_density).contiguous()
        energy0 = energy0.contiguous()
        u_obs = u_obs.contiguous()
        torch.cuda.synchronize()
        loss, _ = adj.forward(density, energy0, u_obs, cfg=cfg)
        ctx.adj, ctx.cfg = adj, cfg
        ctx.save_for_backward(density, energy0, u_obs)
        return torch.tensor(loss, dtype=torch.float64, device=log_density.device)

    @staticmethod
    def backward(ctx, grad_loss):
        density, energy0, u_obs = ctx.saved_tensors
        adj, cfg = ctx.adj, ctx.cfg
        # another forward call may have replaced the kept pass: run it again
        adj.forward(density, energy0, u_obs, cfg=cfg)
        grad = torch.empty_like(density)
        adj.backward(grad)
        return grad * grad_loss, None, None, None, None


def time_stepped_loss(log_density, energy0, u_obs, adj, cfg):
    return TimeSteppedLoss.apply(log_density, energy0, u_obs, adj, cfg)
