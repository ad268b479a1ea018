"""torch.autograd wrappers of the engine's distance gradients.

Replaces the reference's row-by-row FP64 Jacobian assembly in
``Python/klampt/math/autodiff/pytorch.py:72-115`` (ADModule.backward) for the
distance functions of ``geometry_ad.py:405-814`` (GeomGeomDistance,
MinDistance): the forward pass returns the value, the gradient comes from the
engine's adjoint kernel in the same launch and is applied in backward.
Torch is only the autograd plumbing here; all computation is libkgpu.so.
"""

from __future__ import annotations

import torch

from .engine import World


class SoftMinDistance(torch.autograd.Function):
    """L[t] = -tau log sum exp(-d/tau) over the (waypoint, link, object) pairs
    of trajectory t (pairs more than 12 tau above the minimum left out),
    q: [T, W, L] float32 CUDA tensor.  Returns float64 [T]."""

    @staticmethod
    def forward(ctx, q: torch.Tensor, world: World, tau: float = 0.01, robot: int = 0):
        L, g = world.softmin(q.detach(), tau, robot=robot, want_grad=q.requires_grad)
        ctx.save_for_backward(g if g is not None else torch.empty(0, device=q.device))
        return L

    @staticmethod
    def backward(ctx, gL: torch.Tensor):
        (g,) = ctx.saved_tensors
        if g.numel() == 0:
            return None, None, None, None
        return (gL.to(g.dtype)[:, None, None] * g), None, None, None


class MinDistance(torch.autograd.Function):
    """Minimum signed link-object distance per configuration, clamped at
    `cutoff` (gradient zero when clamped), q: [B, L].  Returns float64 [B]."""

    @staticmethod
    def forward(ctx, q: torch.Tensor, world: World, cutoff: float = 1.0, robot: int = 0):
        d, pair, cp, g = world.distance(q.detach(), cutoff, robot=robot, want_grad=True)
        ctx.save_for_backward(g)
        return d

    @staticmethod
    def backward(ctx, gd: torch.Tensor):
        (g,) = ctx.saved_tensors
        return (gd.to(g.dtype)[:, None] * g), None, None, None


class SelfMinDistance(torch.autograd.Function):
    """Minimum distance between the robot's own links over its enabled self
    pairs per configuration, clamped at `cutoff` (gradient zero when clamped
    or in contact), q: [B, L].  Returns float64 [B]."""

    @staticmethod
    def forward(ctx, q: torch.Tensor, world: World, cutoff: float = 1.0, robot: int = 0):
        d, pair, cp, g = world.self_distance(q.detach(), cutoff, robot=robot, want_grad=True)
        ctx.save_for_backward(g)
        return d

    @staticmethod
    def backward(ctx, gd: torch.Tensor):
        (g,) = ctx.saved_tensors
        return (gd.to(g.dtype)[:, None] * g), None, None, None
