"""torch.autograd bridge for the PBF adjoint (pbf_adjoint_* through
``PBFAdjoint``).

``rollout(adjoint, x0, v0, rest_density, xsph, steps)`` returns the final
(x, v) of ``steps`` differentiable steps; gradients flow to x0, v0 (CUDA
tensors of shape (n, 4), w ignored) and to the scalar tensors rest_density
and xsph.  One rollout per adjoint handle may be awaiting its backward at a
time: the handle keeps that forward's checkpoints.
"""

from __future__ import annotations

import torch


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, rest_density, xsph, adjoint, steps):
        adjoint.set_physics(float(rest_density), float(xsph))
        x, v = adjoint.forward(x0.detach().contiguous(), v0.detach().contiguous(), int(steps))
        ctx.adjoint = adjoint
        ctx.meta = (rest_density.dtype, rest_density.device, xsph.dtype, xsph.device)
        return x, v

    @staticmethod
    def backward(ctx, gx, gv):
        gx0, gv0, grho, gc = ctx.adjoint.backward(gx.contiguous(), gv.contiguous())
        rt, rd, ct, cd = ctx.meta
        return (gx0, gv0, torch.tensor(grho, dtype=rt, device=rd),
                torch.tensor(gc, dtype=ct, device=cd), None, None)


def rollout(adjoint, x0, v0, rest_density, xsph, steps: int):
    if not torch.is_tensor(rest_density):
        rest_density = torch.tensor(float(rest_density), dtype=torch.float64)
    if not torch.is_tensor(xsph):
        xsph = torch.tensor(float(xsph), dtype=torch.float64)
    return _Rollout.apply(x0, v0, rest_density, xsph, adjoint, steps)
