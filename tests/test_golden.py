"""Golden vectors (tests/golden/*.pt, made by tests/golden/make_golden.py).

CPU: the oracle still reproduces them exactly.  GPU: the CUDA path reproduces
the bit-exact outputs exactly and the float64 image/gradients within the
stated tolerances (images 1e-5 abs; gradients 1e-4 of the largest entry)."""
import os

import pytest
import torch

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(f[:-3] for f in os.listdir(HERE) if f.endswith(".pt"))


def load(name):
    return torch.load(os.path.join(HERE, name + ".pt"), weights_only=False)


@pytest.mark.parametrize("name", CASES)
def test_oracle_reproduces_golden(name):
    from tests.golden.make_golden import CASES as GEN, make_case

    g = load(name)
    fresh = make_case(*GEN[name])
    for k, v in g["out32"].items():
        assert torch.equal(fresh["out32"][k], v), k
    assert torch.allclose(fresh["out64"]["image"], g["out64"]["image"], atol=1e-12)
    for k, v in g["out64"]["grads"].items():
        assert torch.allclose(fresh["out64"]["grads"][k], v, atol=1e-12), k


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_golden(name):
    from pointrix_gb300 import ops

    g = load(name)
    i = g["inputs"]
    dev = "cuda"
    W, H = i["W"], i["H"]
    leaves = [t.to(dev).requires_grad_(True) for t in
              (i["position"], i["scale"], i["rotation"], i["opacity"], i["shs"])]
    intr = i["intr"].to(dev).requires_grad_(True)
    extr = i["extr"].to(dev).requires_grad_(True)
    p, s, q, o, sh = leaves
    d = p - i["center"].to(dev)[None]
    d = d / d.norm(dim=1, keepdim=True)
    rgb = (ops.compute_sh(sh.permute(0, 2, 1), d) + 0.5).clamp(min=0)
    uv, depth = ops.project_point(p, intr, extr, W, H, nearest=0.2)
    vis = depth != 0
    cov = ops.compute_cov3d(s, q, vis)
    conic, radius, tiles = ops.ewa_project(p, cov, intr, extr, uv, W, H, vis)
    ids, rng = ops.sort_gaussian(uv, depth, W, H, radius, tiles)
    got = dict(uv=uv, depth=depth, cov3d=cov, conic=conic, radius=radius, tiles=tiles, ids=ids, tile_range=rng)
    for k, v in g["out32"].items():
        assert torch.equal(got[k].detach().cpu(), v), k
    img = ops.alpha_blending(uv, conic, o, torch.cat([rgb, depth], 1), ids, rng, 0.0, W, H)
    assert (img.detach().cpu().double() - g["out64"]["image"]).abs().max() < 1e-5
    loss = ((img - i["target"].to(dev)) ** 2).mean()
    loss.backward()
    mine = dict(zip(("position", "scale", "rotation", "opacity", "shs"), (t.grad for t in leaves)))
    mine.update(intr=intr.grad, extr=extr.grad)
    for k, ref in g["out64"]["grads"].items():
        err = float((mine[k].cpu().double() - ref).abs().max() / ref.abs().max().clamp(min=1e-30))
        assert err < 1e-4, (k, err)
