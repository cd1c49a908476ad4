"""Adam for the Gaussian parameters, one kernel launch per step.

Replaces the torch Adam update of Pointrix's training step
(``pointrix/optimizer/optimizer.py:128-140``) with ``pgb_adam_step``: every
parameter group is one entry of a segment table and the whole update is a
single HBM stream (28 bytes per element).  Same update rule as
``torch.optim.Adam`` (no weight decay, no amsgrad); the step count and bias
corrections are kept on the host (per parameter, as torch does), so a step
never synchronises.  With ``capturable=True`` the step counts live on the
device instead and the bias corrections are formed there, so a step can be
captured in a CUDA graph and replayed.
"""
from __future__ import annotations

import torch

from . import _lib
from .ops import _timed


class Adam(torch.optim.Optimizer):
    def __init__(self, params, lr=1e-3, betas=(0.9, 0.999), eps=1e-8, capturable=False):
        if not 0.0 <= eps:
            raise ValueError(f"invalid eps {eps}")
        super().__init__(params, dict(lr=lr, betas=betas, eps=eps))
        self.capturable = bool(capturable)
        # capturable mode: one device step count per parameter (a fixed slot
        # each, in _count_all), gathered into _steps_dev in the order of the
        # segments of the current step; re-gathered whenever the set of
        # parameters with a gradient changes
        self._slots: dict = {}
        self._count_all = None
        self._steps_dev = None
        self._steps_key = None

    @torch.no_grad()
    def step(self, closure=None):
        loss = closure() if closure is not None else None
        segs = []
        cfg = None
        for group in self.param_groups:
            b1, b2 = group["betas"]
            key = (b1, b2, group["eps"])
            if cfg is None:
                cfg = key
            elif cfg != key:
                raise ValueError("pointrix_gb300.optim.Adam: all groups must share betas and eps")
            for p in group["params"]:
                if p.grad is None:
                    continue
                if not (p.is_cuda and p.dtype == torch.float32 and p.is_contiguous()
                        and p.grad.is_contiguous()):
                    raise ValueError("Adam: parameters and gradients must be contiguous CUDA float32")
                st = self.state[p]
                if not st:
                    st["step"] = 0
                    st["exp_avg"] = torch.zeros_like(p)
                    st["exp_avg_sq"] = torch.zeros_like(p)
                st["step"] += 1
                t = st["step"]
                segs.append((p, p.grad, st["exp_avg"], st["exp_avg_sq"], float(group["lr"]),
                             1.0 - b1 ** t, 1.0 - b2 ** t))
        if not segs:
            return loss

        b1, b2, eps = cfg
        lib = _lib.lib()
        dev = segs[0][0].device
        stream = torch.cuda.current_stream(dev).cuda_stream
        if self.capturable:
            self._gather_counts([p for p, *_ in segs], dev)
        for i in range(0, len(segs), 32):
            chunk = segs[i:i + 32]
            table = (_lib.AdamSegment * len(chunk))(*[
                _lib.AdamSegment(p.data_ptr(), g.data_ptr(), m.data_ptr(), v.data_ptr(), p.numel(),
                                 lr, bc1, bc2)
                for p, g, m, v, lr, bc1, bc2 in chunk])
            if self.capturable:
                with _timed("adam_step", dev, 2):
                    _lib.check(lib.pgb_adam_step_device(table, len(chunk), b1, b2, eps,
                                                        self._steps_dev[i:].data_ptr(),
                                                        self._bc_dev[2 * i:].data_ptr(), stream),
                               "pgb_adam_step_device")
            else:
                with _timed("adam_step", dev, 1):
                    _lib.check(lib.pgb_adam_step(table, len(chunk), b1, b2, eps, stream),
                               "pgb_adam_step")
        return loss

    def _gather_counts(self, params, dev):
        """Device step counts of ``params`` (this step's segments, in order)
        in ``_steps_dev``.  A parameter seen for the first time starts from
        its host count before this step; counts of parameters left out of a
        step stay in their slots untouched."""
        key = tuple(id(p) for p in params)
        if key == self._steps_key:
            return
        new = [p for p in params if id(p) not in self._slots]
        if new:
            for p in new:
                self._slots[id(p)] = len(self._slots)
            init = torch.tensor([self.state[p]["step"] - 1 for p in new], dtype=torch.int32,
                                device=dev)
            self._count_all = init if self._count_all is None else torch.cat(
                [self._write_back(), init])
        else:
            self._count_all = self._write_back()
        self._slots_dev = torch.tensor([self._slots[id(p)] for p in params], dtype=torch.int64,
                                       device=dev)
        self._steps_dev = self._count_all.index_select(0, self._slots_dev)
        self._bc_dev = torch.empty(2 * len(params), dtype=torch.float32, device=dev)
        self._steps_key = key

    def _write_back(self):
        """_count_all with the counts the previous segments advanced."""
        if self._steps_dev is not None:
            self._count_all.index_copy_(0, self._slots_dev, self._steps_dev)
        return self._count_all
