"""Densification statistics (the first consumer of the backward's outputs).

``DensificationStats`` keeps the per-point state that Pointrix's
``DensificationController`` accumulates between densification steps
(``pointrix/controller/gs.py:249-257``: ``grad_accum [N,1]``,
``acc_steps [N,1]``, ``max_radii [N]``) and updates it with one library
kernel per step, as ``preprocess`` does (``gs.py:318-333``, with the
screen-space gradient of ``accumulate_viewspace_grad``, ``gs.py:260-284``):
for the points with ``radius > 0``, ``max_radii`` takes the larger radius,
``grad_accum`` adds the norm of the (optionally ``W/2, H/2``-scaled)
screen-space gradient summed over the batch's views, ``acc_steps`` adds one.
No boolean-mask indexing, so no host synchronisation.
"""
from __future__ import annotations

import torch

from ._lib import call
from .ops import _c, _ptr, _stream, _timed

__all__ = ["DensificationStats", "accumulate"]


def accumulate(grad_accum, acc_steps, max_radii, uv_grad, radii, normalize=None):
    """In-place update of the three statistics.  ``uv_grad`` is [N,2] (or a
    list of per-view [N,2] gradients, summed), ``radii`` [N] int32 (or a list,
    max-reduced); ``normalize`` = (W, H) scales the gradient by (W/2, H/2)."""
    if isinstance(uv_grad, (list, tuple)):
        g = uv_grad[0].detach().reshape(-1, 2).clone()
        for t in uv_grad[1:]:
            g += t.detach().reshape(-1, 2)
        uv_grad = g
    if isinstance(radii, (list, tuple)):
        radii = torch.stack([r.reshape(-1) for r in radii]).max(dim=0).values
    n = grad_accum.shape[0]
    uv_grad = _c(uv_grad.detach().reshape(-1, 2))
    radii = _c(radii.reshape(-1).to(torch.int32))
    if uv_grad.shape[0] != n or radii.numel() != n or acc_steps.numel() != n or max_radii.numel() != n:
        raise ValueError("densification statistics: N disagrees between the tensors")
    for name, t in (("grad_accum", grad_accum), ("acc_steps", acc_steps), ("max_radii", max_radii)):
        if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
            raise ValueError(f"{name} must be a contiguous CUDA float32 tensor")
    sx, sy = (normalize[0] / 2.0, normalize[1] / 2.0) if normalize else (1.0, 1.0)
    dev = grad_accum.device
    with _timed("densify_accumulate", dev, 1 if n else 0):
        call("pgb_densify_accumulate", _ptr(uv_grad), n, _ptr(radii), float(sx), float(sy),
             _ptr(grad_accum), _ptr(acc_steps), _ptr(max_radii), _stream(dev))


class DensificationStats:
    """The controller's accumulated state for ``n`` points on ``device``."""

    def __init__(self, n: int, device="cuda", normalize_grad: bool = False):
        self.normalize_grad = normalize_grad
        self.reset(n, device)

    def reset(self, n: int, device=None):
        device = device or self.grad_accum.device
        self.grad_accum = torch.zeros(n, 1, device=device)
        self.acc_steps = torch.zeros(n, 1, device=device)
        self.max_radii = torch.zeros(n, device=device)

    def preprocess(self, radii, uv_points, width=None, height=None):
        """One step's update from the render outputs: ``radii`` ([N] or a
        list per view) and ``uv_points`` (the ``ndc`` leaves, or a list of
        them; their ``.grad`` is read)."""
        pts = uv_points if isinstance(uv_points, (list, tuple)) else [uv_points]
        grads = [p.grad if p.grad is not None else torch.zeros_like(p) for p in pts]
        norm = (width, height) if self.normalize_grad else None
        accumulate(self.grad_accum, self.acc_steps, self.max_radii, grads, radii, norm)

    def average_grad(self):
        """grad_accum / acc_steps with unvisited points at zero (the
        densification criterion's input)."""
        g = self.grad_accum / self.acc_steps
        return torch.where(g.isnan(), torch.zeros_like(g), g)
