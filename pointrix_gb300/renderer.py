"""Host-side mirror of Pointrix's msplat renderer plug-in.

``MsplatRender`` keeps the interface of the reference class
(``pointrix/model/renderer/msplat.py:12-247``): the ``Config`` fields
``update_sh_iter``, ``max_sh_degree`` and ``render_depth``; ``render_iter``
with the same keyword arguments and returned keys (``rendered_features_split``,
``uv_points`` -- the ``ndc`` leaf whose ``.grad`` the densification controller
reads -- ``visibility`` and ``radii``); ``render_batch`` with the same
stacking of views; ``update_sh_degree``, ``state_dict`` and
``load_state_dict``.  It chains the six operators of :mod:`pointrix_gb300.ops`
exactly as the reference chains msplat's (``msplat.py:94-151``).

``RenderFeatures`` mirrors ``pointrix/model/renderer/utils/renderer_utils.py``:
named per-Gaussian features are concatenated along the last dimension for
blending and the [C,H,W] result is split back by channel counts, in keyword
order.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict

import torch

from . import fused, ops


class RenderFeatures:
    """Named per-Gaussian features packed for one ``alpha_blending`` call."""

    def __init__(self, **kwargs) -> None:
        for k, v in kwargs.items():
            setattr(self, k, v)

    def _items(self):
        return [(k, v) for k, v in self.__dict__.items() if isinstance(v, torch.Tensor)]

    def to(self, device) -> None:
        for k, v in self._items():
            setattr(self, k, v.to(device))

    def combine(self) -> torch.Tensor:
        """[N, sum of channels], in keyword order."""
        return torch.cat([v for _, v in self._items()], dim=-1)

    def split(self, feature: torch.Tensor) -> Dict[str, torch.Tensor]:
        """Slices of the [C,H,W] image per feature name."""
        out, start = {}, 0
        for k, v in self._items():
            end = start + v.shape[-1]
            out[k] = feature[start:end, ...]
            start = end
        return out


class MsplatRender:
    """Differentiable splatting renderer over the GB300 msplat operators."""

    @dataclass
    class Config:
        update_sh_iter: int = 1000
        max_sh_degree: int = 3
        render_depth: bool = False
        # recompute the sorted tile lists and per-pixel state in the backward
        # instead of keeping them from the forward (memory for 4K views)
        recompute_backward: bool = False
        # bands of tile rows for the recompute mode (0: enough that a band
        # holds about ops.BAND_ENTRIES entries)
        recompute_bands: int = 0
        # view direction + SH mask + compute_sh + 0.5 + clamp in one kernel
        # (when shs is dense [N,K,3] storage)
        fused_view_colour: bool = True
        # project_point + compute_cov3d + ewa_project in one kernel each way
        fused_preprocess: bool = True
        # > 0: sort with K kept on the device and lists of this capacity (no
        # host synchronisation; the step can be captured in a CUDA graph)
        sort_capacity: int = 0

    def __init__(self, cfg: "MsplatRender.Config | dict | None" = None, white_bg: bool = False,
                 device="cuda", nearest: float = ops.NEAREST_DEFAULT):
        if isinstance(cfg, dict):
            cfg = MsplatRender.Config(**cfg)
        self.cfg = cfg or MsplatRender.Config()
        self.setup(white_bg, device)
        self.nearest = nearest

    def setup(self, white_bg, device, **kwargs):
        self.sh_degree = 0
        self.device = device
        self.bg_color = 1.0 if white_bg else 0.0

    # -- one view --------------------------------------------------------
    def render_iter(self, height, width, extrinsic_matrix, intrinsic_params, camera_center,
                    position, opacity, scaling, rotation, shs, **kwargs) -> dict:
        """Renders one view.  ``shs`` is [N,K,3]; ``extrinsic_matrix`` the
        world->camera [4,4] (or [3,4]); ``intrinsic_params`` [4] or [1,4].
        Extra keyword tensors listed in ``kwargs['extra_features']`` (a dict
        name -> [N,c]) are blended as additional channels after rgb/depth."""
        n = position.shape[0]
        active = (self.sh_degree + 1) ** 2
        if self.cfg.fused_view_colour and fused.sh_rgb_supported(shs):
            rgb = fused.sh_rgb(shs, position, camera_center, active)
        else:
            direction = position - camera_center.reshape(1, 3).expand(n, 3)
            direction = direction / direction.norm(dim=1, keepdim=True)
            sh_coeff = shs.permute(0, 2, 1)
            if active >= sh_coeff.shape[-1]:
                # the warm-up mask is all ones: multiplying by it is the identity
                rgb = ops.compute_sh(sh_coeff, direction)
            else:
                sh_mask = torch.zeros_like(sh_coeff)
                sh_mask[..., :active] = 1.0
                rgb = ops.compute_sh(sh_coeff * sh_mask, direction)
            rgb = (rgb + 0.5).clamp(min=0.0)

        extr = extrinsic_matrix[:3, :]
        if self.cfg.fused_preprocess:
            uv, depth, conic, radius, tiles_touched = fused.preprocess(
                position, scaling, rotation, intrinsic_params, extr, width, height,
                nearest=self.nearest)
        else:
            uv, depth = ops.project_point(position, intrinsic_params, extr, width, height,
                                          nearest=self.nearest)
            visible = depth != 0
            cov3d = ops.compute_cov3d(scaling, rotation, visible)
            conic, radius, tiles_touched = ops.ewa_project(position, cov3d, intrinsic_params, extr,
                                                           uv, width, height, visible)
        feats = {"rgb": rgb}
        if self.cfg.render_depth:
            feats["depth"] = depth
        feats.update(kwargs.get("extra_features") or {})
        render_features = RenderFeatures(**feats)
        if self.cfg.recompute_backward:
            packed = render_features.combine()
        else:  # blended as one [N,C] feature without concatenating the pieces
            packed = [v.reshape(n, -1) for _, v in render_features._items()]

        ndc = torch.zeros_like(uv, requires_grad=True)
        try:
            ndc.retain_grad()
        except Exception as e:  # a leaf created under no_grad cannot retain
            raise ValueError("ndc does not have grad") from e
        image = ops.rasterize(uv, conic, opacity, packed, depth, radius, tiles_touched,
                              self.bg_color, width, height, ndc,
                              recompute=self.cfg.recompute_backward,
                              bands=self.cfg.recompute_bands or None,
                              capacity=self.cfg.sort_capacity or None)
        return {
            "rendered_features": image,
            "rendered_features_split": render_features.split(image),
            "uv_points": ndc,
            "visibility": radius > 0,
            "radii": radius,
        }

    # -- a batch of views, one after another (the reference's plain loop) --
    def render_batch(self, render_dict: dict) -> dict:
        batched = ("extrinsic_matrix", "camera_center")
        per_name: Dict[str, list] = {}
        uv_points, vis, radii = [], [], []
        for i in range(render_dict["extrinsic_matrix"].shape[0]):
            args = {k: (v[i, ...] if k in batched else v) for k, v in render_dict.items()}
            res = self.render_iter(**args)
            for name, img in res["rendered_features_split"].items():
                per_name.setdefault(name, []).append(img)
            uv_points.append(res["uv_points"])
            vis.append(res["visibility"].unsqueeze(0))
            radii.append(res["radii"].unsqueeze(0))
        out = {name: torch.stack(v, dim=0) for name, v in per_name.items()}
        out.update({
            "uv_points": uv_points,
            "visibility": torch.cat(vis).any(dim=0),
            "radii": torch.cat(radii, 0).max(dim=0).values,
        })
        return out

    def update_sh_degree(self, step):
        if step % self.cfg.update_sh_iter == 0 and self.sh_degree < self.cfg.max_sh_degree:
            self.sh_degree += 1

    def load_state_dict(self, state_dict):
        self.sh_degree = state_dict["sh_degree"]

    def state_dict(self):
        return {"sh_degree": self.sh_degree}
