"""GPU parity of every operator against the CPU oracle, through the C ABI.

Bars (stated per test):
* integer outputs (radius, tiles_touched, sorted ids, tile ranges) and the
  float outputs of the FMA-free projection kernels (uv, depth, cov3d, conic):
  bit-exact against the float32 oracle;
* images (every channel, depth included) and SH colours: within 1e-5 abs
  of the float64 oracle on the same inputs, on every pixel whose float64
  skip/stop decisions do not sit on a threshold (``tests/bars.py``; such
  pixels are counted and must stay rare), and the last-contributor counts
  equal there;
* gradients: within 1e-4 of the float64 oracle's autograd gradient,
  relative to the largest gradient entry of that tensor (the chain
  gradients: 1e-4 relative L2, and 1e-4 of the largest entry for every
  Gaussian no threshold pixel considers).
"""
import pytest
import torch

from oracle import msplat_cpu as O
from pointrix_gb300 import ops
from pointrix_gb300 import workloads as WL
from tests.bars import assert_grad_close, assert_image_close

pytestmark = pytest.mark.gpu
DEV = "cuda"
IMG_ATOL = 1e-5
GRAD_RTOL = 1e-4


def scaled_err(a, b):
    if b is None:                      # the reference has no dependence: expect zeros
        return float(a.detach().abs().max())
    a, b = a.detach().double().cpu(), b.detach().double().cpu()
    den = b.abs().max().clamp(min=1e-30)
    return float((a - b).abs().max() / den)


def cpu(t, dt=None):
    t = t.detach().cpu()
    return t if dt is None else t.to(dt)


class Prepared:
    """GPU preprocessing of one scene + camera, with the inputs kept."""

    def __init__(self, scene, cam, channels=("rgb", "depth"), sh_degree=None):
        pos, sc, q, op, shs = (t.to(DEV) for t in scene.activated())
        self.pos, self.sc, self.q, self.op, self.shs = pos, sc, q, op, shs
        self.cam = cam
        self.W, self.H = cam.W, cam.H
        self.intr = cam.intr.to(DEV)
        self.extr = cam.extr[:3].to(DEV).contiguous()
        self.center = cam.center.to(DEV)
        d = pos - self.center[None]
        self.dirs = d / d.norm(dim=1, keepdim=True)
        self.shc = shs.permute(0, 2, 1)
        self.rgb_raw = ops.compute_sh(self.shc, self.dirs)
        self.uv, self.depth = ops.project_point(pos, self.intr, self.extr, self.W, self.H, nearest=0.2)
        self.vis = self.depth != 0
        self.cov = ops.compute_cov3d(sc, q, self.vis)
        self.conic, self.radius, self.tiles = ops.ewa_project(pos, self.cov, self.intr, self.extr, self.uv,
                                                              self.W, self.H, self.vis)
        self.ids, self.rng = ops.sort_gaussian(self.uv, self.depth, self.W, self.H, self.radius, self.tiles)
        feats = [(self.rgb_raw + 0.5).clamp(min=0)]
        if "depth" in channels:
            feats.append(self.depth)
        self.feat = torch.cat(feats, 1).contiguous()


@pytest.fixture(scope="module")
def small():
    scene, cam = WL.scene_small(0)
    return Prepared(scene, cam)


# --------------------------------------------------------------- forward ---
def test_project_point_bitexact(small):
    p = small
    uv_o, d_o = O.project_point(cpu(p.pos), cpu(p.intr), cpu(p.extr), p.W, p.H, nearest=0.2)
    assert torch.equal(cpu(p.uv), uv_o)
    assert torch.equal(cpu(p.depth), d_o)
    uv64, d64 = O.project_point(cpu(p.pos, torch.float64), cpu(p.intr, torch.float64),
                                cpu(p.extr, torch.float64), p.W, p.H, nearest=0.2)
    assert (cpu(p.uv, torch.float64) - uv64).abs().max() < 1e-3   # float32 rounding of pixel coords
    assert int(p.vis.sum()) > 0.9 * p.pos.shape[0]


def test_cov3d_and_ewa_bitexact(small):
    p = small
    cov_o = O.compute_cov3d(cpu(p.sc), cpu(p.q), cpu(p.vis))
    assert torch.equal(cpu(p.cov), cov_o)
    conic_o, rad_o, tiles_o = O.ewa_project(cpu(p.pos), cpu(p.cov), cpu(p.intr), cpu(p.extr), cpu(p.uv),
                                            p.W, p.H, cpu(p.vis))
    assert torch.equal(cpu(p.radius), rad_o)
    assert torch.equal(cpu(p.tiles), tiles_o)
    assert torch.equal(cpu(p.conic), conic_o)
    assert int((rad_o > 0).sum()) > 0


def test_sort_bitexact(small):
    p = small
    ids_o, rng_o = O.sort_gaussian(cpu(p.uv), cpu(p.depth), p.W, p.H, cpu(p.radius), cpu(p.tiles))
    assert p.ids.numel() == int(p.tiles.sum()) > 0
    assert torch.equal(cpu(p.ids), ids_o)
    assert torch.equal(cpu(p.rng), rng_o)
    ops.check_device_status()


def test_compute_sh_close(small):
    p = small
    ref = O.compute_sh(cpu(p.shc, torch.float64), cpu(p.dirs, torch.float64))
    assert (cpu(p.rgb_raw, torch.float64) - ref).abs().max() < IMG_ATOL


@pytest.mark.parametrize("K", [1, 4, 9, 16])
@pytest.mark.parametrize("layout", ["permuted", "contiguous", "strided"])
def test_compute_sh_layouts_and_grad(K, layout):
    g = torch.Generator().manual_seed(K)
    n = 3000
    base = torch.randn(n, K, 3, generator=g)
    if layout == "permuted":
        sh = base.to(DEV).permute(0, 2, 1)
    elif layout == "contiguous":
        sh = base.permute(0, 2, 1).contiguous().to(DEV)
    else:
        sh = torch.randn(n, 3, 2 * K, generator=g).to(DEV)[:, :, ::2]
    d = torch.randn(n, 3, generator=g)
    d = (d / d.norm(dim=1, keepdim=True)).to(DEV)
    sh = sh.detach().requires_grad_(True)
    d = d.requires_grad_(True)
    out = ops.compute_sh(sh, d)
    up = torch.randn(n, 3, generator=g).to(DEV)
    out.backward(up)
    sh64 = cpu(sh, torch.float64).requires_grad_(True)
    d64 = cpu(d, torch.float64).requires_grad_(True)
    ref = O.compute_sh(sh64, d64)
    ref.backward(cpu(up, torch.float64))
    assert (cpu(out, torch.float64) - ref).abs().max() < 1e-5 * max(1.0, float(ref.abs().max()))
    assert scaled_err(sh.grad, sh64.grad) < GRAD_RTOL
    assert scaled_err(d.grad, d64.grad) < GRAD_RTOL


def blend_inputs64(p):
    return [cpu(t, torch.float64) for t in (p.uv, p.conic, p.op, p.feat)]


def test_alpha_blending_forward_close(small):
    p = small
    img, fT, nc = ops.alpha_blending_with_state(p.uv, p.conic, p.op, p.feat, p.ids, p.rng, 0.0, p.W, p.H)
    u, c, o, f = blend_inputs64(p)
    ref, fT_o, nc_o = O.alpha_blending(u, c, o, f, cpu(p.ids), cpu(p.rng), 0.0, p.W, p.H, return_state=True)
    flagged = O.threshold_pixels(cpu(p.uv), cpu(p.conic), cpu(p.op), cpu(p.ids), cpu(p.rng), p.W, p.H)[0]
    assert_image_close(img, ref, flagged)
    assert bool((cpu(nc) == nc_o)[~flagged].all())
    assert_image_close(fT, fT_o, flagged, what="final T")


def test_alpha_blending_background(small):
    p = small
    img0 = ops.alpha_blending(p.uv, p.conic, p.op, p.feat, p.ids, p.rng, 0.0, p.W, p.H)
    img1, fT, _ = ops.alpha_blending_with_state(p.uv, p.conic, p.op, p.feat, p.ids, p.rng, 0.7, p.W, p.H)
    assert torch.allclose(img1 - img0, 0.7 * fT[None].expand_as(img0), atol=1e-6)


# -------------------------------------------------------------- backward ---
def test_alpha_blending_backward(small):
    p = small
    leaves = [t.detach().clone().requires_grad_(True) for t in (p.uv, p.conic, p.op, p.feat)]
    ndc = torch.zeros_like(p.uv, requires_grad=True)
    img = ops.alpha_blending(*leaves, p.ids, p.rng, 0.25, p.W, p.H, ndc)
    g = torch.Generator().manual_seed(7)
    up = torch.randn(img.shape, generator=g)
    img.backward(up.to(DEV))
    ref_leaves = [t.requires_grad_(True) for t in blend_inputs64(p)]
    ref = O.alpha_blending(*ref_leaves, cpu(p.ids), cpu(p.rng), 0.25, p.W, p.H)
    ref.backward(up.double())
    for name, a, b in zip(("uv", "conic", "opacity", "feature"), leaves, ref_leaves):
        e = scaled_err(a.grad, b.grad)
        assert e < GRAD_RTOL, (name, e)
    assert torch.equal(ndc.grad, leaves[0].grad)   # ndc receives the uv gradient


def test_projection_backward(small):
    p = small
    g = torch.Generator().manual_seed(11)
    pos = p.pos.detach().clone().requires_grad_(True)
    sc = p.sc.detach().clone().requires_grad_(True)
    q = p.q.detach().clone().requires_grad_(True)
    intr = p.intr.detach().clone().requires_grad_(True)
    extr = p.extr.detach().clone().requires_grad_(True)
    uv, depth = ops.project_point(pos, intr, extr, p.W, p.H, nearest=0.2)
    vis = depth != 0
    cov = ops.compute_cov3d(sc, q, vis)
    conic, radius, tiles = ops.ewa_project(pos, cov, intr, extr, uv, p.W, p.H, vis)
    ups = [torch.randn(t.shape, generator=g) for t in (uv, depth, conic)]
    torch.autograd.backward([uv, depth, conic], [u.to(DEV) for u in ups])

    r = [cpu(t, torch.float64).requires_grad_(True) for t in (p.pos, p.sc, p.q, p.intr, p.extr)]
    uv_o, d_o = O.project_point(r[0], r[3], r[4], p.W, p.H, nearest=0.2)
    vis_o = cpu(vis)
    cov_o = O.compute_cov3d(r[1], r[2], vis_o)
    conic_o = O.ewa_project(r[0], cov_o, r[3], r[4], cpu(uv), p.W, p.H, vis_o)[0]
    # cull decisions of the float64 rendition must match the GPU's
    keep = (cpu(radius) > 0)
    conic_o = torch.where(keep[:, None], conic_o, torch.zeros_like(conic_o))
    torch.autograd.backward([uv_o, d_o, conic_o], [u.double() for u in ups])
    for name, a, b in zip(("xyz", "scale", "quat", "intr", "extr"), (pos, sc, q, intr, extr), r):
        e = scaled_err(a.grad, b.grad)
        assert e < GRAD_RTOL, (name, e)


def _render_chain_gpu(p, leaves, bg=0.0):
    pos, sc, q, op, shs, intr, extr = leaves
    d = pos - p.center[None]
    d = d / d.norm(dim=1, keepdim=True)
    rgb = (ops.compute_sh(shs.permute(0, 2, 1), d) + 0.5).clamp(min=0)
    uv, depth = ops.project_point(pos, intr, extr, p.W, p.H, nearest=0.2)
    vis = depth != 0
    cov = ops.compute_cov3d(sc, q, vis)
    conic, radius, tiles = ops.ewa_project(pos, cov, intr, extr, uv, p.W, p.H, vis)
    ids, rng = ops.sort_gaussian(uv, depth, p.W, p.H, radius, tiles)
    feat = torch.cat([rgb, depth], 1)
    ndc = torch.zeros_like(uv, requires_grad=True)
    img = ops.alpha_blending(uv, conic, op, feat, ids, rng, bg, p.W, p.H, ndc)
    return img, ids, rng, vis, radius, ndc


def _blend_inputs_gpu(p, leaves):
    pos, sc, q, op, shs, intr, extr = leaves
    uv, depth = ops.project_point(pos, intr, extr, p.W, p.H, nearest=0.2)
    vis = depth != 0
    cov = ops.compute_cov3d(sc, q, vis)
    conic = ops.ewa_project(pos, cov, intr, extr, uv, p.W, p.H, vis)[0]
    return uv, conic, depth


def test_end_to_end_gradients_match_oracle(small):
    """Full MsplatRender chain on the small workload, gradients for every
    Gaussian parameter and the camera.  The loss is the mean squared error
    against a random target: an L1 loss has a sign discontinuity, so a float32
    and a float64 rendition can disagree on the sign at a pixel whose value
    is within rounding of its target, which says nothing about either."""
    p = small
    g = torch.Generator().manual_seed(21)
    target = torch.rand(4, p.H, p.W, generator=g)
    leaves = [t.detach().clone().requires_grad_(True) for t in (p.pos, p.sc, p.q, p.op, p.shs, p.intr, p.extr)]
    img, ids, rng, vis, radius, ndc = _render_chain_gpu(p, leaves)
    loss = ((img - target.to(DEV)) ** 2).mean()
    loss.backward()

    r = [cpu(t, torch.float64).requires_grad_(True) for t in (p.pos, p.sc, p.q, p.op, p.shs, p.intr, p.extr)]
    pos, sc, q, op, shs, intr, extr = r
    d = pos - cpu(p.center, torch.float64)[None]
    d = d / d.norm(dim=1, keepdim=True)
    rgb = (O.compute_sh(shs.permute(0, 2, 1), d) + 0.5).clamp(min=0)
    uv, depth = O.project_point(pos, intr, extr, p.W, p.H, nearest=0.2)
    vis_o = cpu(vis)
    cov = O.compute_cov3d(sc, q, vis_o)
    conic = O.ewa_project(pos, cov, intr, extr, uv.detach().float(), p.W, p.H, vis_o)[0]
    # The blend runs on the GPU's float32 intermediates (values substituted,
    # gradients flowing through the float64 chain), so that both sides take
    # their skip/stop decisions on the same inputs: a float64 uv that differs
    # in the 8th digit can flip a decision for a pair sitting on a threshold.
    with torch.no_grad():
        gd = dict(zip(("uv", "conic", "depth"), (cpu(t, torch.float64) for t in _blend_inputs_gpu(p, leaves))))
    uv = uv + (gd["uv"] - uv).detach()
    conic = conic + (gd["conic"] - conic).detach()
    depth = depth + (gd["depth"] - depth).detach()
    feat = torch.cat([rgb, depth], 1)
    img_o = O.alpha_blending(uv, conic, op, feat, cpu(ids), cpu(rng), 0.0, p.W, p.H)
    loss_o = ((img_o - target.double()) ** 2).mean()
    loss_o.backward()
    assert abs(float(loss.detach()) - float(loss_o.detach())) < 1e-5
    # A float32 and a float64 rendition may still take a different skip/stop
    # decision for a (pixel, splat) pair that sits on a threshold; the
    # Gaussians such pixels consider are excluded from the worst-entry bar.
    gflag = O.threshold_pixels(gd["uv"], gd["conic"], cpu(p.op), cpu(ids), cpu(rng), p.W, p.H)[2]
    for name, a, b in zip(("position", "scale", "rotation", "opacity", "shs", "intr", "extr"), leaves, r):
        assert_grad_close(a.grad, b.grad, gflag, what=name)


# ------------------------------------------------------------ edge cases ---
@pytest.mark.parametrize("W,H", [(250, 130), (16, 16), (10, 7), (33, 17)])
def test_odd_image_sizes(W, H):
    scene, _ = WL.scene_small(3, n=3000)
    g = torch.Generator().manual_seed(W * 1000 + H)
    cam = WL.make_camera(g, W, H, float(max(W, H)), 4.0)
    p = Prepared(scene, cam)
    ids_o, rng_o = O.sort_gaussian(cpu(p.uv), cpu(p.depth), W, H, cpu(p.radius), cpu(p.tiles))
    assert torch.equal(cpu(p.ids), ids_o) and torch.equal(cpu(p.rng), rng_o)
    img = ops.alpha_blending(p.uv, p.conic, p.op, p.feat, p.ids, p.rng, 0.1, W, H)
    ref = O.alpha_blending(*blend_inputs64(p), cpu(p.ids), cpu(p.rng), 0.1, W, H)
    assert img.shape == (4, H, W)
    flagged = O.threshold_pixels(cpu(p.uv), cpu(p.conic), cpu(p.op), cpu(p.ids), cpu(p.rng), W, H)[0]
    assert_image_close(img, ref, flagged)


def test_everything_culled_gives_background():
    scene, cam = WL.scene_small(4, n=500)
    p_pos = scene.position + 100.0   # all far outside the frustum extent
    scene = WL.Scene(p_pos, scene.log_scale, scene.quat_raw, scene.opacity_logit, scene.shs)
    p = Prepared(scene, cam)
    assert p.ids.numel() == 0 and int(p.rng.abs().sum()) == 0
    img = ops.alpha_blending(p.uv, p.conic, p.op, p.feat, p.ids, p.rng, 0.3, p.W, p.H)
    assert torch.all(img == 0.3)
    leaves = [t.detach().clone().requires_grad_(True) for t in (p.uv, p.conic, p.op, p.feat)]
    ops.alpha_blending(*leaves, p.ids, p.rng, 0.3, p.W, p.H).sum().backward()
    assert all(float(t.grad.abs().max()) == 0 for t in leaves)


@pytest.mark.parametrize("C", [1, 3, 7, 12, 26])
def test_channel_counts(small, C):
    p = small
    g = torch.Generator().manual_seed(C)
    feat = torch.rand(p.pos.shape[0], C, generator=g).to(DEV).requires_grad_(True)
    img = ops.alpha_blending(p.uv, p.conic, p.op, feat, p.ids, p.rng, 0.0, p.W, p.H)
    up = torch.randn(img.shape, generator=g)
    img.backward(up.to(DEV))
    u, c, o, _ = blend_inputs64(p)
    f64 = cpu(feat, torch.float64).requires_grad_(True)
    ref = O.alpha_blending(u, c, o, f64, cpu(p.ids), cpu(p.rng), 0.0, p.W, p.H)
    ref.backward(up.double())
    assert (cpu(img, torch.float64) - ref).abs().max() < IMG_ATOL
    assert scaled_err(feat.grad, f64.grad) < GRAD_RTOL


def test_side_stream_and_reuse(small):
    p = small
    ref = ops.alpha_blending(p.uv, p.conic, p.op, p.feat, p.ids, p.rng, 0.0, p.W, p.H)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ids, rng = ops.sort_gaussian(p.uv, p.depth, p.W, p.H, p.radius, p.tiles)
        img = ops.alpha_blending(p.uv, p.conic, p.op, p.feat, ids, rng, 0.0, p.W, p.H)
    s.synchronize()
    assert torch.equal(ids, p.ids) and torch.equal(img, ref)
    ops.check_device_status()


def test_bad_arguments_raise(small):
    p = small
    with pytest.raises(ValueError):
        ops.compute_sh(torch.zeros(p.dirs.shape[0], 3, 5, device=DEV), p.dirs)
    with pytest.raises(ValueError):
        ops.project_point(p.pos.cpu(), p.intr, p.extr, p.W, p.H)
    with pytest.raises(ValueError):
        ops.alpha_blending(p.uv, p.conic, p.op, p.feat, p.ids, p.rng[:-1], 0.0, p.W, p.H)
    with pytest.raises(ValueError):
        ops.sort_gaussian(p.uv, p.depth, p.W, p.H, p.radius.float(), p.tiles)


@pytest.mark.parametrize("bands", [None, 3, 16])
def test_recompute_backward_matches_stored(small, bands):
    """rasterize(recompute=True) re-runs the sort and blend forward in the
    backward, one band of tile rows at a time in both directions; image and
    gradients equal the stored mode (1e-4 relative L2 for gradients: the
    backward's float atomics may add in another order)."""
    p = small
    outs = {}
    for mode in (False, True):
        leaves = [t.detach().clone().requires_grad_(True) for t in (p.uv, p.conic, p.op, p.feat)]
        ndc = torch.zeros_like(p.uv, requires_grad=True)
        img = ops.rasterize(*leaves, p.depth, p.radius, p.tiles, 0.2, p.W, p.H, ndc, recompute=mode,
                            bands=bands)
        g = torch.Generator().manual_seed(5)
        img.backward(torch.randn(img.shape, generator=g).to(DEV))
        outs[mode] = (img.detach(), [t.grad for t in leaves], ndc.grad)
    assert torch.equal(outs[False][0], outs[True][0])
    for a, b in zip(outs[False][1], outs[True][1]):
        assert float((a - b).norm() / b.norm()) < 1e-4
    assert torch.equal(outs[True][2], outs[True][1][0])


def test_blend_batches_agree(small):
    """Every compiled per-block batch gives the same forward outputs (bit for
    bit) and the same gradients (float sums in another order: 1e-5)."""
    from pointrix_gb300 import autotune
    p = small
    C = p.feat.shape[1]
    key_f = autotune.workload_class("blend_fwd", C, p.W * p.H, p.ids.numel(), p.rng.shape[0])
    key_b = autotune.workload_class("blend_bwd", C, p.W * p.H, p.ids.numel(), p.rng.shape[0])
    up = torch.randn((C, p.H, p.W), generator=torch.Generator().manual_seed(3)).to(DEV)
    outs, grads = [], []
    try:
        for bf in ops._blend_batches(0):
            for bb in ops._blend_batches(1):
                autotune.reset()
                autotune._cache[key_f] = bf
                autotune._cache[key_b] = bb
                leaves = [t.detach().clone().requires_grad_(True) for t in (p.uv, p.conic, p.op, p.feat)]
                img, fT, nc = ops.alpha_blending_with_state(*leaves, p.ids, p.rng, 0.1, p.W, p.H)
                img.backward(up)
                outs.append((img.detach(), fT, nc))
                grads.append([t.grad for t in leaves])
    finally:
        autotune.reset()
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            assert torch.equal(a, b)
    for g in grads[1:]:
        for a, b in zip(g, grads[0]):
            assert scaled_err(a, b) < 1e-5
    ops.check_device_status()


def test_alpha_blending_pieces_matches_concatenation(small):
    """Pieces blend exactly like their concatenation; each piece gets the
    matching columns of the feature gradient."""
    p = small
    f = p.feat
    pieces = [f[:, :3].contiguous(), f[:, 3:4].contiguous()]
    up = torch.randn((f.shape[1], p.H, p.W), generator=torch.Generator().manual_seed(5)).to(DEV)
    leaves_a = [t.detach().clone().requires_grad_(True) for t in (p.uv, p.conic, p.op, f)]
    img_a = ops.alpha_blending(*leaves_a, p.ids, p.rng, 0.3, p.W, p.H)
    img_a.backward(up)
    leaves_b = [t.detach().clone().requires_grad_(True) for t in (p.uv, p.conic, p.op)]
    pieces_b = [t.detach().clone().requires_grad_(True) for t in pieces]
    ndc = torch.zeros_like(p.uv, requires_grad=True)
    img_b = ops.alpha_blending_pieces(*leaves_b, pieces_b, p.ids, p.rng, 0.3, p.W, p.H, ndc)
    img_b.backward(up)
    assert torch.equal(img_a, img_b)
    for a, b in zip(leaves_a[:3], leaves_b):
        assert scaled_err(b.grad, a.grad) < 1e-5
    assert scaled_err(torch.cat([t.grad for t in pieces_b], 1), leaves_a[3].grad) < 1e-5
    assert torch.equal(ndc.grad, leaves_b[0].grad)
    with pytest.raises(ValueError):
        ops.alpha_blending_pieces(p.uv, p.conic, p.op, [], p.ids, p.rng, 0.0, p.W, p.H)
    ops.check_device_status()


def test_blend_pair_census_counts_the_replayed_and_composited_pairs(small):
    """The measurement aid behind the benchmark's blend roofline: evaluated
    pairs = the sum of the contributor counts; composited pairs = the
    oracle's count of list entries before each pixel's last contributor
    that pass the alpha test (float64; threshold pairs may differ)."""
    p = small
    ev, comp = ops.blend_pair_census(p.uv, p.conic, p.op, p.feat, p.ids, p.rng, p.W, p.H)
    _, _, nc = ops.alpha_blending_with_state(p.uv, p.conic, p.op, p.feat, p.ids, p.rng, 0.0, p.W, p.H)
    assert ev == int(nc.long().sum())
    u, c, o, _ = blend_inputs64(p)
    gx, gy = O.tile_grid(p.W, p.H)
    ncc = cpu(nc).reshape(-1).long()
    ref = 0
    for t in range(gx * gy):
        s, e = int(p.rng[t, 0]), int(p.rng[t, 1])
        if e <= s:
            continue
        pxi, pyi, pix = O._tile_pixels(t, p.W, p.H)
        g = cpu(p.ids)[s:e].long()
        dx = u[g, 0][None] - pxi.double()[:, None]
        dy = u[g, 1][None] - pyi.double()[:, None]
        pw = -0.5 * (c[g, 0][None] * dx * dx + c[g, 2][None] * dy * dy) - c[g, 1][None] * dx * dy
        a = o.reshape(-1)[g][None] * torch.exp(pw)
        before = torch.arange(e - s)[None] < ncc[pix][:, None]
        ref += int(((pw <= 0) & (a >= 1 / 255) & before).sum())
    assert 0 < comp <= ev
    assert abs(comp - ref) <= max(2, 1e-4 * ref), (comp, ref)
    ops.check_device_status()


@pytest.mark.parametrize("bands", [1, 2, 5, 16])
@pytest.mark.parametrize("band_lists", [True, False])
def test_band_sort_lists_are_the_whole_image_lists(small, bands, band_lists, monkeypatch):
    """Each band's (band-local) tile lists are the whole image's lists of
    the same tiles, bit for bit; the bands cover every tile row once and
    their entry counts add up to K.  Both phase-two paths: over each band's
    own Gaussian list, and over the whole depth order."""
    p = small
    gx, gy = O.tile_grid(p.W, p.H)
    if not band_lists:
        monkeypatch.setattr(ops, "BAND_LIST_MAX", 0)
    bs = ops._BandSort(p.uv, p.depth, p.W, p.H, p.radius, p.tiles, bands)
    assert (bs.lists is not None) == band_lists
    assert bs.K == p.ids.numel()
    if band_lists:
        # band b's list: the Gaussians with an entry in its rows, in depth
        # order (depth, then id), from the float32 oracle's tile rectangles
        rad, uvc, dep = cpu(p.radius), cpu(p.uv), cpu(p.depth).reshape(-1)
        n = rad.numel()
        order = torch.tensor(sorted(range(n), key=lambda g: (float(dep[g]), g)))
        x0, x1, y0, y1 = O.tile_rect(uvc[:, 0], uvc[:, 1], rad.to(torch.float32), p.W, p.H)
        has = (rad > 0) & (x1 > x0)
        for i, (r0, r1, _) in enumerate(bs.plan):
            m = has & (torch.clamp(y1, max=r1) > torch.clamp(y0, min=r0))
            want = order[m[order]].tolist()
            got = cpu(bs.lists)[bs.list_off[i]:bs.list_off[i + 1]].tolist()
            assert got == want, (i, len(got), len(want))
    ids, rng = cpu(p.ids), cpu(p.rng).long()
    plan = bs.plan
    assert plan[0][0] == 0 and plan[-1][1] == gy and len(plan) <= min(bands, gy)
    assert all(a[1] == b[0] for a, b in zip(plan, plan[1:]))
    assert sum(k for _, _, k in plan) == bs.K
    for i, (r0, r1, k) in enumerate(plan):
        bi, br = (cpu(t) for t in bs.band(i))
        br = br.long()
        assert br.shape[0] == gx * (r1 - r0) and bi.numel() == k
        for tl in range(br.shape[0]):
            t = r0 * gx + tl
            assert torch.equal(bi[br[tl, 0]:br[tl, 1]], ids[rng[t, 0]:rng[t, 1]]), (r0, r1, tl)
    ops.check_device_status()
