"""Full-size checks at the training workload: 1,000,000 SH-3 Gaussians, one
1600x1060 view, K ~ 16.6M (Gaussian, tile) entries.

The oracle's sort does not run at this size in a test's time, so the sort is
checked through properties that do not depend on size and together fix its
output exactly: every visible Gaussian appears tiles_touched times, each
entry's tile lies in its Gaussian's rectangle, the tile ranges partition
[0, K) in tile order, and within a tile (depth, id) strictly increases --
i.e. each Gaussian covers exactly the tiles of its rectangle, in the stable
(tile, depth, id) order of the reference's 64-bit key sort.  The
per-Gaussian integer and float outputs of the projection are compared with
the float32 oracle over all 1M Gaussians, bit for bit.  The blend forward
(RGB + depth) and the seven-channel backward of the training loss are
compared with the float64 oracle on sampled tiles (bars of
``tests/bars.py``: 1e-5 abs on every channel off the threshold pixels,
gradients 1e-4)."""
import pytest
import torch

from oracle import msplat_cpu as O
from pointrix_gb300 import ops
from pointrix_gb300 import workloads as WL
from tests.bars import assert_grad_close, assert_image_close

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module")
def view():
    scene, cam = WL.scene_train_view(1, n=1_000_000)
    pos, sc, q, op, shs = (t.to(DEV) for t in scene.activated())
    intr, extr = cam.intr.to(DEV), cam.extr[:3].to(DEV).contiguous()
    W, H = cam.W, cam.H
    uv, depth = ops.project_point(pos, intr, extr, W, H, nearest=0.2)
    vis = depth != 0
    cov = ops.compute_cov3d(sc, q, vis)
    conic, radius, tiles = ops.ewa_project(pos, cov, intr, extr, uv, W, H, vis)
    ids, rng = ops.sort_gaussian(uv, depth, W, H, radius, tiles)
    d = pos - cam.center.to(DEV)[None]
    d = d / d.norm(dim=1, keepdim=True)
    rgb = (ops.compute_sh(shs.permute(0, 2, 1), d) + 0.5).clamp(min=0)
    normal = WL.normals_from_scene(sc, q)
    return dict(W=W, H=H, uv=uv, depth=depth, conic=conic, radius=radius, tiles=tiles, op=op,
                ids=ids, rng=rng, feat=torch.cat([rgb, depth], 1).contiguous(), cov=cov,
                feat7=torch.cat([rgb, depth, normal], 1).contiguous(),
                inputs=(pos, sc, q, intr, extr))


def test_full_size_sort_is_the_stable_tile_depth_id_order(view):
    v = view
    W, H = v["W"], v["H"]
    gx, gy = O.tile_grid(W, H)
    n = v["uv"].shape[0]
    ids, rng = v["ids"].long(), v["rng"].long()
    K = ids.numel()
    radius = v["radius"].reshape(-1)
    visible = radius > 0
    touched = v["tiles"].reshape(-1).long()
    assert K == int(touched[visible].sum()) and K > 10_000_000
    # every visible Gaussian tiles_touched times, the others never
    assert torch.equal(torch.bincount(ids, minlength=n), torch.where(visible, touched, 0))
    # the ranges partition [0, K) in tile order; empty tiles are [0, 0)
    assert rng.shape[0] == gx * gy
    full = rng[:, 1] > rng[:, 0]
    assert bool((rng[~full] == 0).all())
    r = rng[full]
    assert int(r[0, 0]) == 0 and int(r[-1, 1]) == K and bool((r[1:, 0] == r[:-1, 1]).all())
    tile_of = torch.repeat_interleave(torch.nonzero(full).flatten(), r[:, 1] - r[:, 0])
    # each entry's tile inside its Gaussian's rectangle (float32 steps, as the sort)
    uv = v["uv"][ids]
    xmin, xmax, ymin, ymax = O.tile_rect(uv[:, 0], uv[:, 1], radius[ids].float(), W, H)
    tx, ty = tile_of % gx, tile_of // gx
    assert bool(((tx >= xmin) & (tx < xmax) & (ty >= ymin) & (ty < ymax)).all())
    # within a tile, (depth, id) strictly increasing
    same = tile_of[1:] == tile_of[:-1]
    dep = v["depth"].reshape(-1)[ids]
    d0, d1, i0, i1 = dep[:-1], dep[1:], ids[:-1], ids[1:]
    assert bool((((d0 < d1) | ((d0 == d1) & (i0 < i1))) | ~same).all())
    ops.check_device_status()


def _sampled_tiles(W, H, count=24, seed=11):
    gx, gy = O.tile_grid(W, H)
    g = torch.Generator().manual_seed(seed)
    return sorted(torch.randperm(gx * gy, generator=g)[:count].tolist())


def _tile_mask(tiles, W, H):
    gx, _ = O.tile_grid(W, H)
    m = torch.zeros(H, W, dtype=torch.bool)
    for t in tiles:
        x0, y0 = (t % gx) * 16, (t // gx) * 16
        m[y0:y0 + 16, x0:x0 + 16] = True
    return m


def _cpu64(t):
    return t.detach().cpu().double()


def test_full_size_projection_bitexact_over_all_gaussians(view):
    """uv, depth, cov3d, conic, radius and tiles touched of all 1M Gaussians
    equal the float32 oracle's bit for bit."""
    v = view
    pos, sc, q, intr, extr = (t.cpu() for t in v["inputs"])
    W, H = v["W"], v["H"]
    uv, depth = O.project_point(pos, intr, extr, W, H, nearest=0.2)
    assert torch.equal(v["uv"].cpu(), uv) and torch.equal(v["depth"].cpu(), depth)
    cov = O.compute_cov3d(sc, q, depth != 0)
    assert torch.equal(v["cov"].cpu(), cov)
    conic, radius, tiles = O.ewa_project(pos, cov, intr, extr, uv, W, H, depth != 0)
    assert torch.equal(v["radius"].cpu(), radius)
    assert torch.equal(v["tiles"].cpu(), tiles)
    assert torch.equal(v["conic"].cpu(), conic)
    assert int((radius > 0).sum()) > 500_000


def test_full_size_blend_matches_oracle_on_sampled_tiles(view):
    v = view
    W, H = v["W"], v["H"]
    img, fT, nc = ops.alpha_blending_with_state(v["uv"], v["conic"], v["op"], v["feat"], v["ids"],
                                                v["rng"], 0.0, W, H)
    tiles = _sampled_tiles(W, H)
    args = (v["uv"].cpu(), v["conic"].cpu(), v["op"].cpu(), v["ids"].cpu(), v["rng"].cpu(), W, H)
    ref, fT_o, nc_o = O.alpha_blending(_cpu64(v["uv"]), _cpu64(v["conic"]), _cpu64(v["op"]),
                                       _cpu64(v["feat"]), v["ids"].cpu(), v["rng"].cpu(), 0.0, W, H,
                                       tiles=tiles, return_state=True)
    flagged = O.threshold_pixels(*args, tiles=tiles)[0]
    outside = ~_tile_mask(tiles, W, H)
    # pixels outside the sampled tiles are not compared (the oracle left them at bg)
    ref_img = torch.where(outside[None], img.detach().cpu().double(), ref)
    assert_image_close(img, ref_img, flagged, what="image (RGB + depth)")
    assert bool((nc.cpu() == nc_o)[~flagged & ~outside].all())
    assert_image_close(fT, torch.where(outside, fT.cpu().double(), fT_o), flagged, what="final T")
    ops.check_device_status()


def test_full_size_seven_channel_backward_on_sampled_tiles(view):
    """The training step's blend backward (RGB + depth + normal, gradient of
    L1 + 0.2 L2 against a fixed random target), restricted to sampled tiles
    by zeroing the image gradient elsewhere, against the float64 oracle's
    autograd on the same tiles: uv, conic, opacity and feature gradients."""
    v = view
    W, H = v["W"], v["H"]
    leaves = [t.detach().clone().requires_grad_(True) for t in (v["uv"], v["conic"], v["op"], v["feat7"])]
    ndc = torch.zeros_like(v["uv"], requires_grad=True)
    img = ops.alpha_blending(*leaves, v["ids"], v["rng"], 0.0, W, H, ndc)
    g = torch.Generator().manual_seed(5)
    target = torch.rand(img.shape, generator=g).to(DEV)
    with torch.no_grad():
        d = img - target
        dout = (torch.sign(d) + 0.4 * d) / d.numel()       # d (L1 + 0.2 L2) / d img
    tiles = _sampled_tiles(W, H, seed=17)
    inside = _tile_mask(tiles, W, H).to(DEV)
    dout = torch.where(inside[None], dout, torch.zeros_like(dout))
    img.backward(dout)
    ref_leaves = [_cpu64(t).requires_grad_(True) for t in leaves]
    ref = O.alpha_blending(*ref_leaves, v["ids"].cpu(), v["rng"].cpu(), 0.0, W, H, tiles=tiles)
    ref.backward(dout.cpu().double())
    gflag = O.threshold_pixels(v["uv"].cpu(), v["conic"].cpu(), v["op"].cpu(), v["ids"].cpu(),
                               v["rng"].cpu(), W, H, tiles=tiles)[2]
    for name, a, b in zip(("uv", "conic", "opacity", "feature"), leaves, ref_leaves):
        assert_grad_close(a.grad, b.grad, gflag, what=name)
    assert torch.equal(ndc.grad, leaves[0].grad)
    ops.check_device_status()
