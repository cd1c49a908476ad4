"""The parity bars, in one place.

* Images and depths: within ``IMG_ATOL`` = 1e-5 abs of the float64
  rendition on every pixel whose float64 skip/stop decisions do not sit on a
  threshold (``oracle.msplat_cpu.threshold_pixels``); a flagged pixel may
  take the other side of its decision, which moves it by at most one
  splat's share (alpha <= 1/255 for the skip test, the last contributor's
  weight for the stop test), and flagged pixels must stay rare.
* Gradients: relative L2 error below ``GRAD_RTOL`` = 1e-4 for every tensor,
  and every entry of a Gaussian that no flagged pixel considers within
  ``GRAD_RTOL`` of the tensor's largest entry.
"""
from __future__ import annotations

import torch

IMG_ATOL = 1e-5
GRAD_RTOL = 1e-4
FLAGGED_MAX_FRACTION = 1e-3


def _cpu64(t):
    return t.detach().cpu().double()


def assert_image_close(img, ref, flagged=None, atol=IMG_ATOL, what="image"):
    """``img``, ``ref`` [C,H,W] (or [H,W]); ``flagged`` [H,W] bool or None."""
    a, b = _cpu64(img), _cpu64(ref)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    err = (a - b).abs()
    if err.dim() == 3:
        err = err.amax(dim=0)
    if flagged is None:
        flagged = torch.zeros_like(err, dtype=torch.bool)
    flagged = flagged.cpu().reshape(err.shape)
    assert float(flagged.float().mean()) <= FLAGGED_MAX_FRACTION or int(flagged.sum()) <= 4, \
        (what, "too many threshold pixels", int(flagged.sum()))
    worst = float(err[~flagged].max()) if bool((~flagged).any()) else 0.0
    assert worst < atol, (what, "max abs error off the thresholds", worst)
    return worst


def assert_grad_close(g, ref, gauss_flagged=None, rtol=GRAD_RTOL, what="grad"):
    """Relative L2 over the tensor, and the worst entry (scaled by the largest
    reference entry) over the rows of Gaussians not flagged."""
    a, b = _cpu64(g), _cpu64(ref)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    assert bool(torch.isfinite(a).all()), (what, "non-finite gradient")
    den = b.norm().clamp(min=1e-30)
    rel = float((a - b).norm() / den)
    assert rel < rtol, (what, "relative L2", rel)
    scale = b.abs().max().clamp(min=1e-30)
    err = (a - b).abs() / scale
    if gauss_flagged is not None and a.dim() >= 1 and a.shape[0] == gauss_flagged.numel():
        err = err[~gauss_flagged.cpu()]
    worst = float(err.max()) if err.numel() else 0.0
    assert worst < rtol, (what, "worst entry off the thresholds", worst)
    return rel, worst
