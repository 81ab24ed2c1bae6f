"""torch.autograd binding of the checkpointed adjoint (nnpp_forward_ckpt / nnpp_backward).

MassLossCurve maps theta = (D_liquid[0..3], k_diss) -- a float64 tensor of 5 -- to the
cumulative Mg mass-loss curve sampled every `sample_every` steps.  Each call resets the
simulation to its initial state, installs theta (D_solid[k] scales with D_liquid[k]) and
runs the forward with checkpoints on the GPU; backward() runs the adjoint of the explicit
step backwards through the recomputed segments.  This is the calibration interface: the
reference has no gradients and is tuned by hand-edited .datac* files (utils.h:2343-2484).
"""
import numpy as np
import torch

from . import MIXED, NSPECIES


def _install(sim, base, theta):
    p = base.copy()
    for k in range(NSPECIES):
        f = float(theta[k]) / base.D_liquid[k]
        p.D_liquid[k] = float(theta[k])
        p.D_solid[k] = base.D_solid[k] * f
    p.k_diss = float(theta[NSPECIES])
    sim.set_params(p)


class MassLossCurve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, sim, base_params, n_steps, precision=MIXED, ckpt_every=50,
                sample_every=20):
        th = theta.detach().to("cpu", torch.float64).numpy()
        _install(sim, base_params, th)
        sim.reset()
        curve = sim.forward_ckpt(n_steps, precision, ckpt_every, sample_every)
        ctx.sim = sim
        return torch.from_numpy(curve).to(theta.device, theta.dtype)

    @staticmethod
    def backward(ctx, grad_curve):
        g = grad_curve.detach().to("cpu", torch.float64).numpy()
        gD, gk = ctx.sim.backward(np.ascontiguousarray(g))
        grad = torch.from_numpy(np.concatenate([gD, [gk]])).to(grad_curve.device, grad_curve.dtype)
        return grad, None, None, None, None, None, None


def mass_loss_curve(theta, sim, base_params, n_steps, precision=MIXED, ckpt_every=50,
                    sample_every=20):
    """Differentiable cumulative Mg mass-loss curve of `sim` for theta (5,)."""
    return MassLossCurve.apply(theta, sim, base_params, n_steps, precision, ckpt_every,
                               sample_every)
