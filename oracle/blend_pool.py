"""The oracle's tile-by-tile blend and loss gradient on a pool of host
processes.

TEST INFRASTRUCTURE ONLY (the CPU legs of ``bench.py`` time the float64
training step with it).  Threads do not speed the per-tile torch work up
(its many small operators contend), so the tiles go to worker processes
started with ``spawn`` (safe after the parent has used a GPU): the inputs
live in shared memory, written in place by the parent before each call,
every worker sums its tiles' gradients into its own shared buffer, and the
parent adds the buffers.  The arithmetic is ``msplat_cpu.blend_tile`` and
the result equals ``msplat_cpu.blend_loss_grad`` up to the order of the
float64 sums.
"""
from __future__ import annotations

import torch
import torch.multiprocessing as mp

from . import msplat_cpu as O

_W = {}   # per-worker state (set by _init)


def _init(shared, counter, W, H, bg, w1, w2, scale):
    torch.set_num_threads(1)
    with counter.get_lock():
        idx = counter.value
        counter.value += 1
    _W.update(shared=shared, idx=idx, W=W, H=H, bg=bg, w1=w1, w2=w2, scale=scale)


def _task(tiles):
    s_ = _W["shared"]
    U, Cn, Op, F, ids, rng, target = (s_[k] for k in ("U", "Cn", "Op", "F", "ids", "rng", "target"))
    grads = s_["grads"][_W["idx"]]
    n2, n3 = 2, 5
    C = F.shape[1]
    W, H, bg = _W["W"], _W["H"], _W["bg"]
    total = 0.0
    for t in tiles:
        s, e = int(rng[t, 0]), int(rng[t, 1])
        pxi, pyi, pix = O._tile_pixels(t, W, H)
        if e <= s:
            img = torch.full((C, pix.numel()), float(bg), dtype=torch.float64)
            d = img - target[:, pix]
            total += float((_W["w1"] * d.abs().sum() + _W["w2"] * (d * d).sum()) * _W["scale"])
            continue
        g = ids[s:e].long()
        leaves = [x[g].clone().requires_grad_(True) for x in (U, Cn, Op, F)]
        col, Tf, _ = O.blend_tile(*leaves, torch.arange(g.numel()), pxi, pyi)
        img = (col + Tf[:, None] * bg).t()
        d = img - target[:, pix]
        loss = (_W["w1"] * d.abs().sum() + _W["w2"] * (d * d).sum()) * _W["scale"]
        gl = torch.autograd.grad(loss, leaves)
        total += float(loss.detach())
        grads[:, :n2].index_add_(0, g, gl[0])
        grads[:, n2:n3].index_add_(0, g, gl[1])
        grads[:, n3:n3 + 1].index_add_(0, g, gl[2])
        grads[:, n3 + 1:].index_add_(0, g, gl[3])
    return total


class BlendPool:
    """``workers`` spawned processes for a view of W x H with ``n``
    Gaussians, C feature channels and at most ``capacity`` list entries; the
    loss is ``scale * sum(w1 |img - target| + w2 (img - target)^2)``."""

    def __init__(self, n, C, capacity, W, H, target, workers, bg=0.0, w1=1.0, w2=0.2, scale=1.0,
                 tiles_per_task=32):
        gx, gy = O.tile_grid(W, H)
        self.T = gx * gy
        self.capacity = int(capacity)
        self.tiles_per_task = tiles_per_task
        f64 = dict(dtype=torch.float64)
        self.shared = {
            "U": torch.zeros(n, 2, **f64), "Cn": torch.zeros(n, 3, **f64),
            "Op": torch.zeros(n, 1, **f64), "F": torch.zeros(n, C, **f64),
            "ids": torch.zeros(self.capacity, dtype=torch.int32),
            "rng": torch.zeros(self.T, 2, dtype=torch.int64),
            "target": target.detach().reshape(C, -1).to(torch.float64).clone(),
            "grads": [torch.zeros(n, 6 + C, **f64) for _ in range(workers)],
        }
        for k, v in self.shared.items():
            for t in (v if isinstance(v, list) else [v]):
                t.share_memory_()
        ctx = mp.get_context("spawn")
        counter = ctx.Value("i", 0)
        self.pool = ctx.Pool(workers, initializer=_init,
                             initargs=(self.shared, counter, W, H, bg, w1, w2, scale))
        # start every worker now, so that later calls time only the work
        self.pool.map(_task, [[] for _ in range(workers * 4)])

    def run(self, uv, conic, opacity, feature, ids, tile_range):
        """Loss and (d_uv, d_conic, d_opacity, d_feature) of one blend."""
        s = self.shared
        K = ids.numel()
        if K > self.capacity:
            raise ValueError(f"BlendPool: {K} list entries exceed the capacity {self.capacity}")
        s["U"].copy_(uv.detach())
        s["Cn"].copy_(conic.detach())
        s["Op"].copy_(opacity.detach().reshape(-1, 1))
        s["F"].copy_(feature.detach())
        s["ids"][:K].copy_(ids)
        s["rng"].copy_(tile_range.long())
        for g in s["grads"]:
            g.zero_()
        chunks = [list(range(t, min(t + self.tiles_per_task, self.T)))
                  for t in range(0, self.T, self.tiles_per_task)]
        loss = sum(self.pool.imap_unordered(_task, chunks))
        tot = s["grads"][0].clone()
        for g in s["grads"][1:]:
            tot += g
        return loss, tot[:, 0:2], tot[:, 2:5], tot[:, 5:6].reshape(opacity.shape), tot[:, 6:]

    def close(self):
        self.pool.terminate()
        self.pool.join()
