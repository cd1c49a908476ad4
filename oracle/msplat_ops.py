"""The oracle's operators under msplat's call signatures.

TEST INFRASTRUCTURE ONLY (like the rest of ``oracle/``).  Bound as
``msplat`` when the reference's own ``MsplatRender.render_iter``
(``pointrix/model/renderer/msplat.py:94-158``) is executed on the CPU, so
that the reference's glue -- direction, SH warm-up mask, ``+0.5``/clamp,
feature packing, the ``ndc`` gradient sink, the per-view loop of
``render_batch`` -- runs unmodified around the CPU restatement of the six
operators.  The positional signatures are the call sites'
(``msplat.py:104,109-113,118,121-130,133-135,148-151``).
"""
from __future__ import annotations

from . import msplat_cpu as O


def compute_sh(sh_coeffs, view_dirs):
    return O.compute_sh(sh_coeffs, view_dirs)


def project_point(xyz, intr, extr, W, H, nearest=O.NEAREST_DEFAULT):
    return O.project_point(xyz, intr, extr, W, H, nearest=nearest)


def compute_cov3d(scales, uquats, visible):
    return O.compute_cov3d(scales, uquats, visible)


def ewa_project(xyz, cov3d, intr, extr, uv, W, H, visible):
    return O.ewa_project(xyz, cov3d, intr, extr, uv, W, H, visible)


def sort_gaussian(uv, depth, W, H, radius, tiles_touched):
    return O.sort_gaussian(uv, depth, W, H, radius, tiles_touched)


def alpha_blending(uv, conic, opacity, feature, gaussian_ids_sorted, tile_range, bg, W, H, ndc):
    """``ndc`` [N,2] (a zero leaf) receives d loss / d uv, as msplat's
    ``alpha_blending`` fills ``ndc.grad`` (``msplat.py:141-150``): the blend
    reads ``uv + ndc``, whose gradient both ``uv`` and ``ndc`` receive."""
    if ndc is not None:
        uv = uv + ndc.to(uv.dtype)
    return O.alpha_blending(uv, conic, opacity, feature, gaussian_ids_sorted, tile_range, bg, W, H)

