"""Generates tests/golden/*.pt from the CPU oracle.

The reference operator backend (msplat) is absent from the reference tree and
the reference has no tests or fixtures, so these vectors come from the
oracle itself: they freeze its behaviour (float32 rendition for the
bit-exact outputs, float64 for the image and gradients) so that any change to
it, and the GPU path on the GPU, is checked against the same numbers.

    python tests/golden/make_golden.py
"""
import os
import sys

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import msplat_cpu as O  # noqa: E402
from pointrix_gb300 import workloads as WL  # noqa: E402

CASES = {
    # name: (seed, n, W, H, focal, radius, sh)
    "tiny_sh0_64x48": (11, 400, 64, 48, 60.0, 3.0, 1),
    "tiny_sh3_70x41": (12, 600, 70, 41, 55.0, 3.2, 16),
}


def make_case(seed, n, W, H, f, rad, K):
    g = torch.Generator().manual_seed(seed)
    pos = (torch.rand(n, 3, generator=g) * 2 - 1) * 0.8
    log_s = torch.randn(n, 3, generator=g) * 0.4 - 3.0
    q = torch.randn(n, 4, generator=g)
    op_logit = torch.randn(n, 1, generator=g)
    shs = torch.randn(n, K, 3, generator=g) * 0.3
    cam = WL.make_camera(g, W, H, f, rad)
    target = torch.rand(4, H, W, generator=g)
    # activated parameters are stored as the operators receive them, so the
    # GPU test feeds bit-identical float32 inputs
    scale = torch.exp(log_s)
    quat = q / q.norm(dim=1, keepdim=True)
    opac = torch.sigmoid(op_logit)
    inputs = dict(position=pos, scale=scale, rotation=quat, opacity=opac, shs=shs,
                  intr=cam.intr, extr=cam.extr[:3].contiguous(), center=cam.center, W=W, H=H,
                  target=target)
    # float32 rendition: bit-exact outputs
    uv, depth = O.project_point(pos, cam.intr, inputs["extr"], W, H, nearest=0.2)
    vis = depth != 0
    cov = O.compute_cov3d(scale, quat, vis)
    conic, radius, tiles = O.ewa_project(pos, cov, cam.intr, inputs["extr"], uv, W, H, vis)
    ids, rng = O.sort_gaussian(uv, depth, W, H, radius, tiles)
    out32 = dict(uv=uv, depth=depth, cov3d=cov, conic=conic, radius=radius, tiles=tiles, ids=ids,
                 tile_range=rng)
    # float64 rendition with the float32 tile lists: image and gradients
    leaves = [t.double().requires_grad_(True) for t in (pos, scale, quat, opac, shs)]
    intr64 = cam.intr.double().requires_grad_(True)
    extr64 = inputs["extr"].double().requires_grad_(True)
    p, s, qq, o, sh = leaves
    d = p - cam.center.double()[None]
    d = d / d.norm(dim=1, keepdim=True)
    rgb = (O.compute_sh(sh.permute(0, 2, 1), d) + 0.5).clamp(min=0)
    uv64, depth64 = O.project_point(p, intr64, extr64, W, H, nearest=0.2)
    cov64 = O.compute_cov3d(s, qq, vis)
    conic64 = O.ewa_project(p, cov64, intr64, extr64, uv, W, H, vis)[0]
    img = O.alpha_blending(uv64, conic64, o, torch.cat([rgb, depth64], 1), ids, rng, 0.0, W, H)
    loss = ((img - target.double()) ** 2).mean()   # smooth loss: no sign flips at rounding level
    loss.backward()
    out64 = dict(image=img.detach(), loss=loss.detach(),
                 grads={k: t.grad for k, t in zip(("position", "scale", "rotation", "opacity", "shs"),
                                                  leaves)} | {"intr": intr64.grad, "extr": extr64.grad})
    return dict(inputs=inputs, out32=out32, out64=out64)


def main():
    for name, cfg in CASES.items():
        torch.save(make_case(*cfg), os.path.join(HERE, name + ".pt"))
        print("wrote", name)


if __name__ == "__main__":
    main()
