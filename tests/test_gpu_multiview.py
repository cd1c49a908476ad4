"""Batched multi-view rendering against rendering each view alone: images
bit-identical (the bar is 1e-5 abs; within a tile the order is the same),
gradients within 1e-4 relative L2 (float atomics may add in another
order)."""
import pytest
import torch

from pointrix_gb300 import multiview, ops
from pointrix_gb300 import workloads as WL

pytestmark = pytest.mark.gpu


def _cams():
    g = torch.Generator().manual_seed(31)
    sizes = [(256, 256), (200, 120), (333, 217), (64, 48)]
    return [WL.make_camera(g, W, H, 0.9 * W, 3.5 + 0.3 * i).to("cuda") for i, (W, H) in enumerate(sizes)]


def _leaves():
    scene, _ = WL.scene_small(7, n=12000)
    return [t.cuda().requires_grad_(True) for t in scene.activated()]


def _per_view(leaves, cams):
    pos, sc, q, op, shs = leaves
    imgs = []
    for cam in cams:
        d = pos - cam.center.reshape(1, 3)
        d = d / d.norm(dim=1, keepdim=True)
        rgb = (ops.compute_sh(shs.permute(0, 2, 1), d) + 0.5).clamp(min=0)
        extr = cam.extr[:3, :]
        uv, depth = ops.project_point(pos, cam.intr, extr, cam.W, cam.H)
        vis = depth != 0
        cov = ops.compute_cov3d(sc, q, vis)
        conic, radius, tiles = ops.ewa_project(pos, cov, cam.intr, extr, uv, cam.W, cam.H, vis)
        ids, rng = ops.sort_gaussian(uv, depth, cam.W, cam.H, radius, tiles)
        imgs.append(ops.alpha_blending(uv, conic, op, torch.cat([rgb, depth], 1), ids, rng, 0.1,
                                       cam.W, cam.H))
    return imgs


@pytest.mark.parametrize("tile_height", [16, 32])
def test_batched_views_match_per_view(tile_height):
    """Also with 16 x 32 tiles: the per-box filter keeps exactly the splats
    of the 16 x 16 lists, so the images are still bit-identical."""
    cams = _cams()
    ref_leaves, bat_leaves = _leaves(), _leaves()
    ref = _per_view(ref_leaves, cams)
    bat, _, _ = multiview.render_views(*bat_leaves, cams, bg=0.1, tile_height=tile_height)
    g = torch.Generator().manual_seed(3)
    ups = [torch.randn(r.shape, generator=g).cuda() for r in ref]
    for a, b in zip(ref, bat):
        assert a.shape == b.shape
        assert torch.equal(a, b)
    torch.autograd.backward(ref, ups)
    torch.autograd.backward(bat, ups)
    for a, b in zip(ref_leaves, bat_leaves):
        assert float((a.grad - b.grad).norm() / a.grad.norm()) < 1e-4
    ops.check_device_status()


def test_view_count_limits():
    cams = _cams()
    leaves = _leaves()
    with pytest.raises(ValueError):
        multiview.blend_views(torch.zeros(10, 2, device="cuda"), torch.zeros(10, 3, device="cuda"),
                              torch.zeros(10, device="cuda"), torch.zeros(10, 3, device="cuda"),
                              torch.zeros(0, dtype=torch.int32, device="cuda"),
                              torch.zeros(1, 2, dtype=torch.int32, device="cuda"), 0.0,
                              [(16, 16)] * 65, 10)


def test_batched_views_capacity_mode_in_a_graph():
    """The batch with K kept on the device, captured once and replayed:
    the same images as the host-K batch."""
    from pointrix_gb300.graph import GraphedStep
    cams = _cams()
    leaves = [t.detach() for t in _leaves()]
    ref, _, _ = multiview.render_views(*leaves, cams, bg=0.1)
    K = sum(int(r.numel()) for r in ref)           # an ample capacity: entries <= pixels * N
    cap = 64 * K

    def fn():
        imgs, _, _ = multiview.render_views(*leaves, cams, bg=0.1, capacity=cap)
        return imgs

    graphed = GraphedStep(fn, warmup=1)
    for _ in range(2):
        out = graphed()
        torch.cuda.synchronize()
        for a, b in zip(ref, out):
            assert torch.equal(a, b)
    ops.check_device_status()


@pytest.mark.parametrize("capacity_extra", [None, 4096])
def test_batched_sort_lists_match_per_view_sorts(capacity_extra):
    """The batch sorts view-local tile ids over a view-major emission: for
    every view v and tile t, tile_range[base_v + t] must select exactly the
    list that sorting view v alone gives for t (element ids offset by v N)."""
    cams = _cams()
    pos, sc, q, op, shs = _leaves()
    n = pos.shape[0]
    uvs, depths, radii, tiles, per = [], [], [], [], []
    with torch.no_grad():
        for cam in cams:
            extr = cam.extr[:3, :]
            uv, depth = ops.project_point(pos, cam.intr, extr, cam.W, cam.H)
            vis = depth != 0
            cov = ops.compute_cov3d(sc, q, vis)
            _, radius, nt = ops.ewa_project(pos, cov, cam.intr, extr, uv, cam.W, cam.H, vis)
            uvs.append(uv); depths.append(depth); radii.append(radius); tiles.append(nt)
            per.append(ops.sort_gaussian(uv, depth, cam.W, cam.H, radius, nt))
    K = sum(int(i.numel()) for i, _ in per)
    cap = None if capacity_extra is None else K + capacity_extra
    sizes = [(c.W, c.H) for c in cams]
    ids, rng = multiview.sort_views(torch.cat(uvs), torch.cat(depths), torch.cat(radii),
                                    torch.cat(tiles), sizes, n, capacity=cap)
    ids, rng = ids.cpu().long(), rng.cpu().long()
    assert int((rng[:, 1] - rng[:, 0]).sum()) == K
    base = 0
    for v, (ids_v, rng_v) in enumerate(per):
        T_v = rng_v.shape[0]
        got = torch.cat([ids[rng[base + t, 0]:rng[base + t, 1]] for t in range(T_v)]) - v * n
        assert torch.equal(got, ids_v.cpu().long()), v
        empty = (rng_v[:, 1] == rng_v[:, 0]).cpu()
        assert bool((rng[base:base + T_v][empty] == 0).all())
        base += T_v
    ops.check_device_status()


def test_finish_views_after_one_image_begin_is_reported():
    """Phase two of a batch needs the batch's phase one (view-major depth
    order): after the one-image phase one it reports PGB_ERR_INVALID in the
    info word (its outputs are then undefined, as after any reported fault)."""
    from pointrix_gb300 import _lib
    cams = _cams()[:2]
    pos, sc, q, op, shs = _leaves()
    n = pos.shape[0]
    uvs, depths, radii, tiles = [], [], [], []
    with torch.no_grad():
        for cam in cams:
            extr = cam.extr[:3, :]
            uv, depth = ops.project_point(pos, cam.intr, extr, cam.W, cam.H)
            vis = depth != 0
            cov = ops.compute_cov3d(sc, q, vis)
            _, radius, nt = ops.ewa_project(pos, cov, cam.intr, extr, uv, cam.W, cam.H, vis)
            uvs.append(uv); depths.append(depth); radii.append(radius); tiles.append(nt)
    uv, depth, radius, nt = (torch.cat(x) for x in (uvs, depths, radii, tiles))
    sizes = [(c.W, c.H) for c in cams]
    h = ops.sort_gaussian_begin(uv, depth, sizes[0][0], sizes[0][1], radius, nt)  # one image
    K = h.count()
    T = sum(multiview._tiles(W, H) for W, H in sizes)
    T_local = max(multiview._tiles(W, H) for W, H in sizes)
    _, bk = ops._sort_scratch(h.n, K, 16 * T_local, 16)
    scratch_k = torch.empty(max(bk, 1), dtype=torch.uint8, device="cuda")
    ids = torch.empty(max(K, 1), dtype=torch.int32, device="cuda")
    rng = torch.empty(T, 2, dtype=torch.int32, device="cuda")
    _lib.call("pgb_sort_gaussian_finish_views", h.uv.data_ptr(), h.radius.data_ptr(),
              h.tiles.data_ptr(), n, multiview._sizes_array(sizes), len(sizes), K,
              h.scratch_n.data_ptr(), h.bn, scratch_k.data_ptr(), bk, h.info.data_ptr(),
              ids.data_ptr(), rng.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(h.info[1]) == 1  # PGB_ERR_INVALID (the outputs are then undefined)


def test_tall_tiles_need_fewer_entries_and_every_variant_agrees():
    """16 x 32 tile lists: fewer entries than 16 x 16 for the same batch, and
    every compiled forward / backward variant gives the same images (bit for
    bit) and gradients (1e-5, float sums in another order)."""
    from pointrix_gb300 import autotune
    cams = _cams()
    leaves = _leaves()
    with torch.no_grad():
        ref, _, _ = multiview.render_views(*leaves, cams, bg=0.1)
    pos, sc, q, op, shs = leaves
    sizes = [(c.W, c.H) for c in cams]
    with torch.no_grad():
        uvr = [multiview.fused.preprocess(pos, sc, q, c.intr, c.extr[:3], c.W, c.H) for c in cams]
    uv = torch.cat([u[0] for u in uvr])
    radius = torch.cat([u[3] for u in uvr])
    t16 = torch.cat([u[4] for u in uvr])
    t32 = multiview.tile_counts_views(uv, radius, sizes, pos.shape[0], 32)
    assert int(t32.sum()) < int(t16.sum())
    g = torch.Generator().manual_seed(9)
    ups = [torch.randn(r.shape, generator=g).cuda() for r in ref]
    grads = []
    try:
        for bf in multiview._blend_batches_h(0, 32):
            for bb in multiview._blend_batches_h(1, 32):
                autotune.set_pins(f"fwd={bf},bwd={bb}")
                lv = [t.detach().clone().requires_grad_(True) for t in leaves]
                out, _, _ = multiview.render_views(*lv, cams, bg=0.1, tile_height=32)
                for a, b in zip(out, ref):
                    assert torch.equal(a, b), (bf, bb)
                torch.autograd.backward(out, ups)
                grads.append([t.grad for t in lv])
    finally:
        autotune.set_pins("")
    for gr in grads[1:]:
        for a, b in zip(gr, grads[0]):
            assert float((a - b).norm() / b.norm()) < 1e-5
    ops.check_device_status()


def test_every_variant_agrees_on_16x16_views():
    """Batched views with 16 x 16 tiles take every blend form (the flat,
    one-warp-per-half and one-warp-per-tile backwards included): images bit
    for bit, gradients within 1e-5 (float sums in another order)."""
    from pointrix_gb300 import autotune
    cams = _cams()
    leaves = _leaves()
    with torch.no_grad():
        ref, _, _ = multiview.render_views(*leaves, cams, bg=0.1, tile_height=16)
    g = torch.Generator().manual_seed(10)
    ups = [torch.randn(r.shape, generator=g).cuda() for r in ref]
    grads = []
    try:
        for bf in multiview._blend_batches_h(0, 16):
            for bb in multiview._blend_batches_h(1, 16):
                autotune.set_pins(f"fwd={bf},bwd={bb}")
                lv = [t.detach().clone().requires_grad_(True) for t in leaves]
                out, _, _ = multiview.render_views(*lv, cams, bg=0.1, tile_height=16)
                for a, b in zip(out, ref):
                    assert torch.equal(a, b), (bf, bb)
                torch.autograd.backward(out, ups)
                grads.append(((bf, bb), [t.grad for t in lv]))
    finally:
        autotune.set_pins("")
    for codes, gr in grads[1:]:
        for a, b in zip(gr, grads[0][1]):
            assert float((a - b).norm() / b.norm()) < 1e-5, codes
    ops.check_device_status()
