"""CPU tests of the oracle itself: known answers from the mathematics, exact
gradients (torch.autograd.gradcheck in float64), float32/float64 agreement and
the sort's structural properties.  No GPU."""
import math

import pytest
import torch

from oracle import msplat_cpu as O
from pointrix_gb300 import workloads as WL

torch.set_default_dtype(torch.float32)


def test_sh_constants_closed_form():
    assert O.SH_C0 == pytest.approx(0.28209479177387814, abs=1e-16)  # point_utils.py:35
    # orthonormality of the real SH basis on the sphere (Monte Carlo, fp64)
    g = torch.Generator().manual_seed(0)
    d = torch.randn(400000, 3, generator=g, dtype=torch.float64)
    d = d / d.norm(dim=1, keepdim=True)
    Y = O.sh_basis(d, 16)
    gram = (Y.T @ Y) * (4 * math.pi / d.shape[0])
    assert torch.allclose(gram, torch.eye(16, dtype=torch.float64), atol=2e-2)


def test_cov3d_identity_rotation_is_diag_s2():
    s = torch.tensor([[0.1, 0.2, 0.3]], dtype=torch.float64)
    q = torch.tensor([[1.0, 0, 0, 0]], dtype=torch.float64)
    cov = O.compute_cov3d(s, q, torch.tensor([[True]]))
    assert torch.allclose(cov, torch.tensor([[0.01, 0, 0, 0.04, 0, 0.09]], dtype=torch.float64))


def test_project_point_known_answer_and_culling():
    intr = torch.tensor([[100.0, 120.0, 50.0, 40.0]], dtype=torch.float64)
    extr = torch.cat([torch.eye(3), torch.zeros(3, 1)], 1).double()
    xyz = torch.tensor([[0.0, 0.0, 2.0], [0.2, -0.1, 1.0], [0.0, 0.0, 0.1], [5.0, 0.0, 1.0]],
                       dtype=torch.float64)
    uv, depth = O.project_point(xyz, intr, extr, 100, 80)
    assert torch.allclose(uv[0], torch.tensor([50.0, 40.0], dtype=torch.float64))
    assert torch.allclose(uv[1], torch.tensor([70.0, 28.0], dtype=torch.float64))
    assert depth[0, 0] == 2.0 and depth[1, 0] == 1.0
    assert depth[2, 0] == 0 and depth[3, 0] == 0        # behind near plane / outside extent
    assert (uv[2] == 0).all() and (uv[3] == 0).all()


def test_ewa_isotropic_radius_and_conic():
    # an isotropic Gaussian of std s at depth z on the optical axis projects to
    # a circle of std f s / z; conic = 1/(var + 0.3)
    f, s, z = 200.0, 0.05, 2.0
    intr = torch.tensor([f, f, 64.0, 64.0], dtype=torch.float64)
    extr = torch.cat([torch.eye(3), torch.zeros(3, 1)], 1).double()
    xyz = torch.tensor([[0.0, 0.0, z]], dtype=torch.float64)
    cov = torch.tensor([[s*s, 0, 0, s*s, 0, s*s]], dtype=torch.float64)
    uv, _ = O.project_point(xyz, intr, extr, 128, 128)
    conic, radius, tiles = O.ewa_project(xyz, cov, intr, extr, uv, 128, 128, torch.tensor([True]))
    var = (f * s / z) ** 2 + 0.3
    assert conic[0, 0].item() == pytest.approx(1 / var) and conic[0, 2].item() == pytest.approx(1 / var)
    assert conic[0, 1].item() == pytest.approx(0.0, abs=1e-15)
    r = math.ceil(3 * math.sqrt(var))
    assert radius[0].item() == r
    x0, x1 = int((64 - r) / 16), int((64 + r + 15) / 16)
    assert tiles[0].item() == (x1 - x0) ** 2


def _tiny_scene(n=24, W=40, H=32, seed=3, dtype=torch.float64):
    g = torch.Generator().manual_seed(seed)
    pos = (torch.rand(n, 3, generator=g) * 2 - 1).to(dtype) * 0.6
    scales = torch.exp(torch.randn(n, 3, generator=g) * 0.3 - 2.3).to(dtype)
    q = torch.randn(n, 4, generator=g).to(dtype)
    q = q / q.norm(dim=1, keepdim=True)
    op = torch.sigmoid(torch.randn(n, 1, generator=g)).to(dtype)
    cam = WL.make_camera(g, W, H, 40.0, 3.0)
    return pos, scales, q, op, cam


def test_gradcheck_project_cov_ewa():
    pos, scales, q, op, cam = _tiny_scene()
    intr = cam.intr.double().requires_grad_(True)
    extr = cam.extr[:3].double().requires_grad_(True)
    pos = pos.requires_grad_(True)
    scales = scales.requires_grad_(True)
    q = q.requires_grad_(True)

    def f_proj(p, i, e):
        uv, d = O.project_point(p, i, e, cam.W, cam.H)
        return uv, d

    assert torch.autograd.gradcheck(f_proj, (pos, intr, extr), eps=1e-6, atol=1e-5)
    vis = O.project_point(pos, intr, extr, cam.W, cam.H)[1] != 0
    assert torch.autograd.gradcheck(lambda s, r: O.compute_cov3d(s, r, vis), (scales, q), eps=1e-6, atol=1e-5)
    uv = O.project_point(pos, intr, extr, cam.W, cam.H)[0].detach()

    def f_ewa(p, s, r, i, e):
        cov = O.compute_cov3d(s, r, vis)
        return O.ewa_project(p, cov, i, e, uv, cam.W, cam.H, vis)[0]

    assert torch.autograd.gradcheck(f_ewa, (pos, scales, q, intr, extr), eps=1e-6, atol=1e-5)


def test_gradcheck_compute_sh():
    g = torch.Generator().manual_seed(5)
    sh = torch.randn(6, 3, 16, generator=g, dtype=torch.float64, requires_grad=True)
    d = torch.randn(6, 3, generator=g, dtype=torch.float64)
    d = (d / d.norm(dim=1, keepdim=True)).requires_grad_(True)
    assert torch.autograd.gradcheck(O.compute_sh, (sh, d), eps=1e-6, atol=1e-6)


def test_gradcheck_alpha_blending_small():
    pos, scales, q, op, cam = _tiny_scene(n=20, W=24, H=20)
    intr, extr = cam.intr.double(), cam.extr[:3].double()
    uv, depth = O.project_point(pos, intr, extr, cam.W, cam.H)
    vis = depth != 0
    cov = O.compute_cov3d(scales, q, vis)
    conic, radius, tiles = O.ewa_project(pos, cov, intr, extr, uv, cam.W, cam.H, vis)
    ids, rng = O.sort_gaussian(uv.float(), depth.float(), cam.W, cam.H, radius, tiles)
    assert ids.numel() > 0
    g = torch.Generator().manual_seed(9)
    feat = torch.rand(20, 4, generator=g, dtype=torch.float64)
    args = [t.detach().clone().requires_grad_(True) for t in (uv, conic, op, feat)]

    def f(u, c, o, ft):
        return O.alpha_blending(u, c, o, ft, ids, rng, 0.3, cam.W, cam.H)

    assert torch.autograd.gradcheck(f, args, eps=1e-7, atol=1e-5, rtol=1e-4)


def test_float32_and_float64_oracles_agree():
    scene, cam = WL.scene_small(0, n=4096)
    pos, sc, q, op, shs = scene.activated()
    res = {}
    for dt in (torch.float32, torch.float64):
        img, uv, radius, aux = O.render_view(pos.to(dt), sc.to(dt), q.to(dt), op.to(dt), shs.to(dt), None,
                                             cam.center.to(dt), cam.intr.to(dt), cam.extr[:3].to(dt),
                                             cam.W, cam.H)
        res[dt] = (img, radius)
    # integer decisions may differ only where fp32 rounding crosses a ceil boundary
    r32, r64 = res[torch.float32][1], res[torch.float64][1]
    assert (r32 != r64).float().mean() < 1e-3
    assert (res[torch.float32][0].double() - res[torch.float64][0]).abs().max() < 5e-3


def test_sort_structure_and_stability():
    scene, cam = WL.scene_small(1, n=2048)
    pos, sc, q, op, shs = scene.activated()
    E = cam.extr[:3]
    uv, depth = O.project_point(pos, cam.intr, E, cam.W, cam.H)
    vis = depth != 0
    cov = O.compute_cov3d(sc, q, vis)
    conic, radius, tiles = O.ewa_project(pos, cov, cam.intr, E, uv, cam.W, cam.H, vis)
    ids, rng = O.sort_gaussian(uv, depth, cam.W, cam.H, radius, tiles)
    assert ids.numel() == int(tiles.sum())
    d = depth.reshape(-1)
    for t in range(rng.shape[0]):
        s, e = rng[t].tolist()
        if e > s:
            seg = ids[s:e].long()
            dd = d[seg]
            assert bool((dd[1:] >= dd[:-1]).all())
    # every Gaussian appears exactly tiles_touched times
    cnt = torch.bincount(ids.long(), minlength=pos.shape[0])
    assert torch.equal(cnt.to(torch.int32), tiles)


def test_sort_rejects_inconsistent_tiles():
    uv = torch.tensor([[8.0, 8.0]])
    depth = torch.tensor([[1.0]])
    with pytest.raises(ValueError):
        O.sort_gaussian(uv, depth, 32, 32, torch.tensor([2], dtype=torch.int32),
                        torch.tensor([5], dtype=torch.int32))


def test_empty_inputs():
    ids, rng = O.sort_gaussian(torch.zeros(0, 2), torch.zeros(0, 1), 20, 20,
                               torch.zeros(0, dtype=torch.int32), torch.zeros(0, dtype=torch.int32))
    assert ids.numel() == 0 and rng.shape == (4, 2) and int(rng.abs().sum()) == 0
    img = O.alpha_blending(torch.zeros(0, 2), torch.zeros(0, 3), torch.zeros(0, 1), torch.zeros(0, 3),
                           ids, rng, 0.5, 20, 20)
    assert torch.all(img == 0.5)


def test_tilewise_loss_gradient_equals_autograd_over_the_image():
    """``blend_loss_grad`` (tile by tile, bounded memory, threads) gives the
    loss, image and gradients of ``alpha_blending`` + autograd."""
    scene, cam = WL.scene_small(6, n=1500)
    a = [t.double() for t in scene.activated()]
    img32, uv32, rad32, aux = O.render_view(*[t.float() for t in a], None, cam.center, cam.intr,
                                            cam.extr[:3], cam.W, cam.H)
    g = torch.Generator().manual_seed(3)
    N = a[0].shape[0]
    uv = uv32.double()
    conic, op = aux["conic"].double(), a[3]
    feat = torch.rand(N, 5, generator=g, dtype=torch.float64)
    target = torch.rand(5, cam.H, cam.W, generator=g, dtype=torch.float64)
    leaves = [x.clone().requires_grad_(True) for x in (uv, conic, op, feat)]
    img = O.alpha_blending(*leaves, aux["ids"], aux["tile_range"], 0.3, cam.W, cam.H)
    d = img - target
    loss = d.abs().sum() + 0.2 * (d * d).sum()
    loss.backward()
    tflat = target.reshape(5, -1)

    def pixel_loss(im, pix):
        dd = im - tflat[:, pix]
        return dd.abs().sum() + 0.2 * (dd * dd).sum()

    for workers in (1, 3):
        L, im2, *gr = O.blend_loss_grad(uv, conic, op, feat, aux["ids"], aux["tile_range"], 0.3,
                                        cam.W, cam.H, pixel_loss, workers=workers)
        assert abs(L - float(loss)) < 1e-9 * float(loss)
        assert torch.allclose(im2, img.detach(), atol=1e-13)
        for x, y in zip(gr, leaves):
            assert torch.allclose(x, y.grad, atol=1e-11, rtol=1e-9)


def test_blend_pool_equals_tilewise_gradient():
    """The spawned-process pool (bench's CPU legs) gives the loss and the
    gradients of ``blend_loss_grad``."""
    from oracle.blend_pool import BlendPool
    scene, cam = WL.scene_small(7, n=1200)
    a = [t.float() for t in scene.activated()]
    _, uv32, _, aux = O.render_view(*a, None, cam.center, cam.intr, cam.extr[:3], cam.W, cam.H)
    g = torch.Generator().manual_seed(4)
    uv, conic, op = uv32.double(), aux["conic"].double(), a[3].double()
    feat = torch.rand(uv.shape[0], 4, generator=g, dtype=torch.float64)
    target = torch.rand(4, cam.H, cam.W, generator=g, dtype=torch.float64)
    tflat = target.reshape(4, -1)
    scale = 1.0 / tflat.numel()

    def pixel_loss(im, pix):
        dd = im - tflat[:, pix]
        return (dd.abs().sum() + 0.2 * (dd * dd).sum()) * scale

    L, _, *ref = O.blend_loss_grad(uv, conic, op, feat, aux["ids"], aux["tile_range"], 0.0,
                                   cam.W, cam.H, pixel_loss)
    pool = BlendPool(uv.shape[0], 4, aux["ids"].numel() + 10, cam.W, cam.H, target, workers=2,
                     scale=scale)
    try:
        for _ in range(2):      # the shared buffers are reused
            L2, *got = pool.run(uv, conic, op, feat, aux["ids"], aux["tile_range"])
            assert abs(L2 - L) < 1e-12
            for x, y in zip(got, ref):
                assert torch.allclose(x, y, atol=1e-15, rtol=1e-10)
    finally:
        pool.close()
