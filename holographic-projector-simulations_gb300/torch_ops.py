"""PyTorch integration: the Huygens sum as an autograd Function.

Forward is ``Plan.execute`` (the split-precision or FP64 kernel); backward is
the hand-written adjoint kernel (``holo_plan_adjoint``: the conjugate-transposed
sum with roles swapped and the sign negated), so phase-only holograms can be
optimised by gradient descent through y -> z without storing the N x M phasor
matrix.  The reference has no gradients; this is the differentiable extension
of its y -> z pass (cuda/main.cu:186).
"""
from __future__ import annotations

import math

import torch

from .api import Plan


class HuygensFunction(torch.autograd.Function):
    """(amp, phase) of N sources -> (M, 2) float64 field (re, im) at the targets."""

    @staticmethod
    def forward(ctx, amp, phase, plan: Plan, sign: int, lam: float):
        a = amp.detach().to(torch.float64).contiguous()
        p = phase.detach().to(torch.float64).contiguous()
        y = torch.view_as_real(plan.execute(a, p, sign, lam)).contiguous()
        ctx.save_for_backward(a, p)
        ctx.plan, ctx.sign, ctx.lam = plan, sign, lam
        ctx.dtypes = (amp.dtype, phase.dtype)
        return y

    @staticmethod
    def backward(ctx, grad_y):
        a, p = ctx.saved_tensors
        g = grad_y.to(torch.float64).contiguous()
        ga, gp = ctx.plan.adjoint(a, p, g, ctx.sign, ctx.lam)
        grad_amp = ga.to(ctx.dtypes[0]) if ctx.needs_input_grad[0] else None
        grad_phase = gp.to(ctx.dtypes[1]) if ctx.needs_input_grad[1] else None
        return grad_amp, grad_phase, None, None, None


def huygens(amp: torch.Tensor, phase: torch.Tensor, plan: Plan, sign: int,
            lam: float) -> torch.Tensor:
    """Differentiable y[m] = sum_n amp_n exp(i(phase_n + sign k r_nm)) / r_nm, as (M, 2)."""
    return HuygensFunction.apply(amp, phase, plan, sign, lam)


def dense_reference(amp: torch.Tensor, phase: torch.Tensor, u: torch.Tensor, v: torch.Tensor,
                    sign: int, lam: float) -> torch.Tensor:
    """The same sum as dense FP64 torch ops (small sizes only; for checking gradients)."""
    k = (2.0 * math.pi) / lam
    r = torch.cdist(v.to(torch.float64), u.to(torch.float64))  # (M, N)
    th = phase.to(torch.float64)[None, :] + sign * k * r
    w = amp.to(torch.float64)[None, :] / r
    return torch.stack([(w * torch.cos(th)).sum(1), (w * torch.sin(th)).sum(1)], dim=1)


def intensity_loss(z: torch.Tensor, target: torch.Tensor) -> torch.Tensor:
    """MSE between |z|^2 normalised to unit mean and the target intensity."""
    inten = z[:, 0] ** 2 + z[:, 1] ** 2
    inten = inten / inten.mean()
    return torch.mean((inten - target) ** 2)


def optimise_phase_hologram(projector_pos: torch.Tensor, target_pos: torch.Tensor,
                            target: torch.Tensor, lam: float, steps: int = 100, lr: float = 0.05,
                            seed: int = 0, precision: str = "split32", callback=None):
    """Phase-only hologram by Adam through the y -> z pass (Forwards).

    Parameters are FP32 projector phases initialised uniform in [0, 2 pi) with
    unit amplitudes; the loss is ``intensity_loss``.  Returns (phases, losses)."""
    dev = projector_pos.device
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = projector_pos.shape[0]
    phase = (torch.rand(n, generator=g, dtype=torch.float32) * (2 * math.pi)).to(dev)
    phase.requires_grad_(True)
    amp = torch.ones(n, dtype=torch.float64, device=dev)
    plan = Plan(projector_pos.reshape(-1), target_pos.reshape(-1), precision)
    opt = torch.optim.Adam([phase], lr=lr)
    losses = []
    try:
        for step in range(steps):
            opt.zero_grad(set_to_none=True)
            z = huygens(amp, phase, plan, +1, lam)
            loss = intensity_loss(z, target)
            loss.backward()
            opt.step()
            losses.append(float(loss.detach()))
            if callback is not None:
                callback(step, losses[-1])
    finally:
        plan.close()
    return phase.detach(), losses
