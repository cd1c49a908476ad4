"""Whole-step CUDA graphs: capture a training (or render) step once, replay it.

A training step over the msplat operators is a few hundred kernel launches
(the operators, the torch glue between them, the loss, autograd and the
optimizer).  Replaying them as one CUDA graph removes the per-launch host
cost and the gaps between launches.  What the step needs for that:

* no host synchronisation inside: the renderer sorts with
  ``MsplatRender.Config.sort_capacity`` (K stays on the device) and the
  optimizer is ``pointrix_gb300.optim.Adam(..., capturable=True)``;
* inputs that change between steps live in tensors that stay in place: copy
  new values into them (``dst.copy_(src)``) before each replay;
* the step sets the gradients to None first (``optimizer.zero_grad(
  set_to_none=True)``), so the captured backward writes them rather than
  accumulating;
* no output of an earlier eager step that still holds an autograd graph
  (a tensor with a ``grad_fn``) is alive at capture: such a graph keeps the
  leaves' gradient accumulators bound to the stream of that eager step, and
  the captured backward would then make that stream wait on the capture
  (keep ``.detach()``-ed results instead).

Device-side faults of a replay (an expired bounded wait, K above the sort
capacity) are reported by :func:`pointrix_gb300.ops.check_device_status`.
"""
from __future__ import annotations

import gc

import torch

from . import ops

__all__ = ["GraphedStep"]


class GraphedStep:
    """``GraphedStep(fn)`` runs ``fn()`` ``warmup`` times on a side stream,
    captures one more call into a CUDA graph, and returns that call's
    outputs from every ``__call__`` (the same tensors, refreshed by the
    replay)."""

    def __init__(self, fn, warmup: int = 2, device=None):
        self.device = torch.device("cuda", torch.cuda.current_device()) if device is None \
            else torch.device(device)
        # finish the host-side bookkeeping of earlier eager calls (pinned
        # read-back buffers, deferred status checks) before capturing: its
        # cleanup must not land in the middle of a capture
        torch.cuda.synchronize(self.device)
        ops._drain_pending(block=True)
        gc.collect()
        side = torch.cuda.Stream(self.device)
        main = torch.cuda.current_stream(self.device)
        side.wait_stream(main)
        with torch.cuda.stream(side):
            for _ in range(warmup):
                fn()
        main.wait_stream(side)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.outputs = fn()

    def __call__(self):
        self.graph.replay()
        return self.outputs
