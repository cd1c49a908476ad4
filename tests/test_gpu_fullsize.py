"""Full-size checks at the training workload: 1,000,000 SH-3 Gaussians, one
1600x1060 view, K ~ 16.6M (Gaussian, tile) entries.

The oracle's sort does not run at this size in a test's time, so the sort is
checked through properties that do not depend on size and together fix its
output exactly: every visible Gaussian appears tiles_touched times, each
entry's tile lies in its Gaussian's rectangle, the tile ranges partition
[0, K) in tile order, and within a tile (depth, id) strictly increases --
i.e. each Gaussian covers exactly the tiles of its rectangle, in the stable
(tile, depth, id) order of the reference's 64-bit key sort.  The blend is
compared with the float64 oracle on sampled tiles (tolerances as in
test_gpu_ops: 1e-5 abs, depth 1e-5 relative to the scene depth)."""
import pytest
import torch

from oracle import msplat_cpu as O
from pointrix_gb300 import ops
from pointrix_gb300 import workloads as WL

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
    return dict(W=W, H=H, uv=uv, depth=depth, conic=conic, radius=radius, tiles=tiles, op=op,
                ids=ids, rng=rng, feat=torch.cat([rgb, depth], 1).contiguous())


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


def test_full_size_blend_matches_oracle_on_sampled_tiles(view):
    v = view
    W, H = v["W"], v["H"]
    gx, gy = O.tile_grid(W, H)
    img, fT, nc = ops.alpha_blending_with_state(v["uv"], v["conic"], v["op"], v["feat"], v["ids"],
                                                v["rng"], 0.0, W, H)
    g = torch.Generator().manual_seed(11)
    tiles = sorted(torch.randperm(gx * gy, generator=g)[:24].tolist())
    cpu64 = lambda t: t.detach().cpu().double()  # noqa: E731
    ref, fT_o, nc_o = O.alpha_blending(cpu64(v["uv"]), cpu64(v["conic"]), cpu64(v["op"]),
                                       cpu64(v["feat"]), v["ids"].cpu(), v["rng"].cpu(), 0.0, W, H,
                                       tiles=tiles, return_state=True)
    img = img.detach().cpu().double()
    depth_scale = float(v["depth"].max())
    for t in tiles:
        x0, y0 = (t % gx) * 16, (t // gx) * 16
        sl = (slice(y0, min(y0 + 16, H)), slice(x0, min(x0 + 16, W)))
        a, b = img[(slice(None),) + sl], ref[(slice(None),) + sl]
        assert (a[:3] - b[:3]).abs().max() < 1e-5, t
        assert (a[3] - b[3]).abs().max() < 1e-5 * depth_scale, t
        assert (fT.cpu().double()[sl] - fT_o[sl]).abs().max() < 1e-5, t
        assert (nc.cpu()[sl] != nc_o[sl]).float().mean() < 0.02, t
    ops.check_device_status()
