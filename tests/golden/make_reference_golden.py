"""Generates ``tests/golden/reference/glue.pt`` by executing Pointrix's own
Python code (the reference) on the CPU.

The msplat operators are absent from the reference, but the code around them
is not: this script runs, unmodified, the reference's

* ``RenderFeatures.combine/split`` (``pointrix/model/renderer/utils/renderer_utils.py:30-71``),
* ``unitquat_to_rotmat`` and ``quat_to_rotmat`` (``pointrix/utils/pose.py:40-118``),
* ``ssim`` (``pointrix/model/loss.py:71-125``),
* ``DensificationController.preprocess`` with ``accumulate_viewspace_grad``
  (``pointrix/controller/gs.py:260-284, 318-333``),
* ``MsplatRender.render_iter`` and ``render_batch``
  (``pointrix/model/renderer/msplat.py:51-213``) and, when installed,
  ``MsplatNormalRender.render_iter`` (``examples/supervise/renderer.py:25-102``),

the renderers with ``import msplat`` bound to the oracle's CPU operators: the
projection, covariance, EWA and sort in float32 (so that every integer
decision is the one the GPU takes, bit for bit) and the colour and the blend
evaluated in float64 on those float32 intermediates (the precision
reference).  It records the outputs, the gradients of a smooth loss, and the
pixels and Gaussians whose float64 decisions sit on a threshold
(``oracle.msplat_cpu.threshold_pixels``).  The GPU tests hold the GB300
renderer to these numbers, so the renderer's glue is pinned to the
reference's code and its operators to the oracle.

    python tests/golden/make_reference_golden.py [--src DIR]

``DIR`` is the reference tree (the directory holding ``pointrix/``), e.g. the
read-only checkout at /root/reference or the offline install
``baseline/_ref``; without it ``tests/refload.py`` finds the install.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import sys
from types import SimpleNamespace

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import refload  # noqa: E402
from oracle import msplat_cpu as O  # noqa: E402
from pointrix_gb300 import workloads as WL  # noqa: E402

OUT = os.path.join(HERE, "reference", "glue.pt")
FILES = ("model/renderer/msplat.py", "model/renderer/utils/renderer_utils.py", "utils/pose.py",
         "model/loss.py", "controller/gs.py")


# ------------------------------------------------- oracle bound as msplat ---
def _f64(t):
    return t.to(torch.float64)


class MixedOracle(SimpleNamespace):
    """msplat's six operators from the oracle: the geometric operators in the
    dtype of their inputs (float32 here), colour and blend in float64 on
    those inputs.  ``ndc`` receives d loss / d uv as msplat's does."""

    __name__ = "oracle_mixed"

    def __init__(self):
        super().__init__()
        self.compute_sh = lambda sh, d: O.compute_sh(_f64(sh), _f64(d))
        self.project_point = lambda xyz, intr, extr, W, H, nearest=O.NEAREST_DEFAULT: \
            O.project_point(xyz, intr, extr, W, H, nearest=nearest)
        self.compute_cov3d = O.compute_cov3d
        self.ewa_project = O.ewa_project
        self.sort_gaussian = O.sort_gaussian

    @staticmethod
    def alpha_blending(uv, conic, opacity, feature, ids, rng, bg, W, H, ndc):
        u = _f64(uv) + _f64(ndc)
        return O.alpha_blending(u, _f64(conic), _f64(opacity), _f64(feature), ids, rng, bg, W, H)


def glue_scene(seed=31, n=500, W=56, H=40):
    """A small SH-3 scene that fills a 56x40 view with overlapping splats
    (partial edge tiles in both directions)."""
    g = torch.Generator().manual_seed(seed)
    pos = torch.randn(n, 3, generator=g) * 0.7
    scale = torch.exp(torch.randn(n, 3, generator=g) * 0.4 - 2.6)
    q = torch.randn(n, 4, generator=g)
    rot = q / q.norm(dim=1, keepdim=True)
    opac = torch.sigmoid(torch.randn(n, 1, generator=g) * 1.5)
    shs = torch.randn(n, 16, 3, generator=g) * 0.05
    shs[:, 0, :] = torch.randn(n, 3, generator=g) * 0.3
    normals = torch.nn.functional.normalize(torch.randn(n, 3, generator=g), dim=-1)
    cams = [WL.make_camera(g, W, H, 48.0, 3.5) for _ in range(2)]
    targets = [torch.rand(4, H, W, generator=g) for _ in range(2)]
    return dict(position=pos, scaling=scale, rotation=rot, opacity=opac, shs=shs, normals=normals,
                W=W, H=H, intr=cams[0].intr, extr=torch.stack([c.extr for c in cams]),
                center=torch.stack([c.center for c in cams]), targets=targets)


def _leaves(sc):
    return {k: sc[k].clone().requires_grad_(True)
            for k in ("position", "opacity", "scaling", "rotation", "shs")}


def _flags(sc, view):
    """Threshold flags of one view from the float32 intermediates."""
    extr = sc["extr"][view][:3]
    uv, depth = O.project_point(sc["position"], sc["intr"], extr, sc["W"], sc["H"], nearest=0.2)
    vis = depth != 0
    cov = O.compute_cov3d(sc["scaling"], sc["rotation"], vis)
    conic, radius, tiles = O.ewa_project(sc["position"], cov, sc["intr"], extr, uv, sc["W"], sc["H"], vis)
    ids, rng = O.sort_gaussian(uv, depth, sc["W"], sc["H"], radius, tiles)
    pix, pix_grad, gauss = O.threshold_pixels(uv, conic, sc["opacity"], ids, rng, sc["W"], sc["H"])
    return dict(pix=pix, pix_grad=pix_grad, gauss=gauss)


def render_iter_case(mod, sc, view=0, sh_degree=2):
    r = refload.make_render(mod, render_depth=True)
    r.sh_degree = sh_degree
    lv = _leaves(sc)
    extr = sc["extr"][view].clone().requires_grad_(True)
    intr = sc["intr"].clone().requires_grad_(True)
    with refload.cuda_calls_stay_on_cpu():
        out = r.render_iter(sc["H"], sc["W"], extr, intr, sc["center"][view], lv["position"],
                            lv["opacity"], lv["scaling"], lv["rotation"], lv["shs"])
    img = torch.cat([out["rendered_features_split"]["rgb"], out["rendered_features_split"]["depth"]])
    loss = ((img - sc["targets"][view].double()) ** 2).mean()
    loss.backward()
    grads = {k: v.grad.clone() for k, v in lv.items()}
    grads["extr"], grads["intr"] = extr.grad.clone(), intr.grad.clone()
    grads["uv_points"] = out["uv_points"].grad.clone()
    return dict(rgb=out["rendered_features_split"]["rgb"].detach(),
                depth=out["rendered_features_split"]["depth"].detach(),
                radii=out["radii"], visibility=out["visibility"], loss=loss.detach(), grads=grads,
                flags=_flags(sc, view), sh_degree=sh_degree)


def render_batch_case(mod, sc):
    r = refload.make_render(mod, render_depth=True)
    r.sh_degree = 3
    lv = _leaves(sc)
    rd = dict(height=sc["H"], width=sc["W"], extrinsic_matrix=sc["extr"], intrinsic_params=sc["intr"],
              camera_center=sc["center"], **lv)
    with refload.cuda_calls_stay_on_cpu():
        out = r.render_batch(rd)
    img = torch.cat([out["rgb"], out["depth"]], 1)                   # [2,4,H,W]
    loss = ((img - torch.stack(sc["targets"]).double()) ** 2).mean()
    loss.backward()
    grads = {k: v.grad.clone() for k, v in lv.items()}
    grads["uv_points"] = [p.grad.clone() for p in out["uv_points"]]
    return dict(rgb=out["rgb"].detach(), depth=out["depth"].detach(), radii=out["radii"],
                visibility=out["visibility"], loss=loss.detach(), grads=grads,
                flags=[_flags(sc, v) for v in range(2)])


def normal_case(nmod, sc, view=0):
    # white background: every pixel's rendered normal is non-zero, so the
    # example's per-pixel normalisation stays finite
    r = refload.make_render(nmod, cls="MsplatNormalRender", white_bg=True)
    lv = _leaves(sc)
    normals = sc["normals"].clone().requires_grad_(True)
    out = r.render_iter(sc["H"], sc["W"], sc["extr"][view], sc["intr"], sc["center"][view],
                        lv["position"], lv["opacity"], lv["scaling"], lv["rotation"], lv["shs"],
                        normals=normals)
    rgb, nrm = out["rendered_features_split"]["rgb"], out["rendered_features_split"]["normal"]
    t = sc["targets"][view].double()
    loss = ((rgb - t[:3]) ** 2).mean() + ((nrm - t[1:]) ** 2).mean()
    loss.backward()
    grads = {k: v.grad.clone() for k, v in lv.items()}
    grads["normals"] = normals.grad.clone()
    grads["uv_points"] = out["uv_points"].grad.clone()
    return dict(rgb=rgb.detach(), normal=nrm.detach(), radii=out["radii"], loss=loss.detach(),
                grads=grads)


# ------------------------------------------------------------ the rest ---
def features_case(ru):
    g = torch.Generator().manual_seed(41)
    rgb, depth, normal = (torch.rand(64, c, generator=g) for c in (3, 1, 3))
    img = torch.rand(7, 5, 6, generator=g)
    rf = ru.RenderFeatures(rgb=rgb, depth=depth, normal=normal)
    return dict(rgb=rgb, depth=depth, normal=normal, image=img, combined=rf.combine(),
                split=rf.split(img))


def pose_case(po):
    g = torch.Generator().manual_seed(43)
    q = torch.randn(64, 4, generator=g, dtype=torch.float64)
    u = q / q.norm(dim=1, keepdim=True)
    return dict(q=q, unit=u, unitquat_to_rotmat=po.unitquat_to_rotmat(u),
                quat_to_rotmat=po.quat_to_rotmat(q))


def ssim_case(lo):
    g = torch.Generator().manual_seed(47)
    y = torch.rand(3, 33, 40, generator=g, dtype=torch.float64)
    x = (y + 0.1 * torch.randn(3, 33, 40, generator=g, dtype=torch.float64)).clamp(0, 1)
    xl = x.clone().requires_grad_(True)
    val = lo.ssim(xl, y)
    val.backward()
    return dict(x=x, y=y, value=val.detach(), grad=xl.grad)


def controller_case(gs):
    g = torch.Generator().manual_seed(53)
    n, W, H = 3000, 640, 480
    ctrl = object.__new__(gs.DensificationController)
    ctrl.cfg = SimpleNamespace(normalize_grad=True)
    ctrl.width, ctrl.height = W, H
    ctrl.grad_accum = torch.zeros(n, 1)
    ctrl.acc_steps = torch.zeros(n, 1)
    ctrl.max_radii = torch.zeros(n)
    steps = []
    for _ in range(3):
        uvs, rads = [], []
        for _v in range(2):
            p = torch.zeros(n, 2, requires_grad=True)
            p.grad = torch.randn(n, 2, generator=g) * 1e-3
            uvs.append(p)
            rads.append(torch.randint(-2, 30, (n,), generator=g).clamp(min=0).to(torch.int32))
        # render_batch's aggregation of the per-view outputs (msplat.py:209-213)
        vis = torch.cat([(r > 0).unsqueeze(0) for r in rads]).any(dim=0)
        radii = torch.cat([r.unsqueeze(0) for r in rads], 0).max(dim=0).values
        ctrl.preprocess(visibility=vis, radii=radii, uv_points=uvs)
        steps.append(dict(uv_grads=[p.grad.clone() for p in uvs], radii=rads,
                          grad_accum=ctrl.grad_accum.clone(), acc_steps=ctrl.acc_steps.clone(),
                          max_radii=ctrl.max_radii.clone()))
    return dict(n=n, W=W, H=H, steps=steps)


def digests(root):
    out = {}
    for f in FILES:
        p = os.path.join(str(root), f)
        with open(p, "rb") as fh:
            out[f] = hashlib.sha256(fh.read()).hexdigest()
    return out


def make_all():
    root = refload.pointrix_dir()
    if root is None:
        raise SystemExit("reference source not found (give --src or install baseline/_ref)")
    mixed = MixedOracle()
    mod = refload.msplat_renderer(mixed)
    sc = glue_scene()
    res = dict(digests=digests(root), scene=sc,
               features=features_case(refload.renderer_utils()),
               pose=pose_case(refload.pose()), ssim=ssim_case(refload.loss()),
               controller=controller_case(refload.gs_controller()),
               render_iter=render_iter_case(mod, sc), render_batch=render_batch_case(mod, sc))
    nmod = refload.normal_renderer(mixed)
    if nmod is not None:
        res["normal"] = normal_case(nmod, sc)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=None, help="reference tree holding pointrix/")
    a = ap.parse_args()
    if a.src:
        os.environ["PGB_POINTRIX_SRC"] = a.src
    torch.set_num_threads(1)
    res = make_all()
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    torch.save(res, OUT)
    print("wrote", OUT, "normal case:", "normal" in res)


if __name__ == "__main__":
    main()
