"""Fused caller-side passes against the torch compositions they replace.

Bars: forward values within 1e-6 (relative to the largest entry) of the
float64 composition; gradients within 1e-5 relative to the largest
gradient entry (they are short float32 chains); the loss gradient equal to
torch's l1_loss + w * mse_loss gradient to 1 ulp.
"""
import pytest
import torch
import torch.nn.functional as F

from oracle import msplat_cpu as O
from pointrix_gb300 import fused, ops
from pointrix_gb300 import workloads as WL
from pointrix_gb300.optim import Adam
from pointrix_gb300.renderer import MsplatRender

pytestmark = pytest.mark.gpu
DEV = "cuda"


def rel(a, b):
    if b is None:          # no dependence in the reference: expect zeros
        return float(a.detach().abs().max())
    a, b = a.detach().double().cpu(), b.detach().double().cpu()
    return float((a - b).abs().max() / b.abs().max().clamp(min=1e-30))


def torch_activations(ls, q, lg):
    """The reference composition in float64 (gaussian_points.py:70-80,
    examples/supervise/model.py:50-62 with pose.py's matrix)."""
    s = torch.exp(ls)
    r = F.normalize(q, dim=-1)
    o = torch.sigmoid(lg)
    idx = torch.argmin(ls, dim=-1)
    w, x, y, z = r.unbind(-1)
    cols = torch.stack([
        torch.stack([x * x - y * y - z * z + w * w, 2 * (x * y + z * w), 2 * (x * z - y * w)], -1),
        torch.stack([2 * (x * y - z * w), -x * x + y * y - z * z + w * w, 2 * (y * z + x * w)], -1),
        torch.stack([2 * (x * z + y * w), 2 * (y * z - x * w), -x * x - y * y + z * z + w * w], -1),
    ], 1)                                           # [N, axis, 3]
    nrm = cols[torch.arange(ls.shape[0]), idx]
    return s, r, o, F.normalize(nrm, dim=-1)


def test_gaussian_activations_match_torch():
    g = torch.Generator().manual_seed(0)
    n = 50_000
    ls = torch.randn(n, 3, generator=g) * 0.7 - 4
    ls[:100, 1] = ls[:100, 0]                  # ties: the first minimum wins
    q = torch.randn(n, 4, generator=g)
    lg = torch.randn(n, 1, generator=g) * 1.5
    ups = [torch.randn(n, c, generator=g) for c in (3, 4, 1, 3)]
    leaves64 = [t.double().requires_grad_(True) for t in (ls, q, lg)]
    ref = torch_activations(*leaves64)
    torch.autograd.backward(ref, [u.double() for u in ups])
    leaves = [t.to(DEV).requires_grad_(True) for t in (ls, q, lg)]
    out = fused.gaussian_activations(*leaves)
    for a, b in zip(out, ref):
        assert rel(a, b) < 1e-6
    torch.autograd.backward(out, [u.to(DEV) for u in ups])
    for a, b in zip(leaves, leaves64):
        assert rel(a.grad, b.grad) < 1e-5
    # without the normal
    s, r, o, nrm = fused.gaussian_activations(*[t.detach() for t in leaves], normals=False)
    assert nrm is None and torch.equal(s, out[0]) and torch.equal(r, out[1])


@pytest.mark.parametrize("K,active", [(16, 16), (16, 4), (16, 9), (9, 9), (4, 1), (1, 1)])
def test_sh_rgb_matches_composition(K, active):
    g = torch.Generator().manual_seed(K * 10 + active)
    n = 20_000 + 13                            # a partial last warp block
    shs = torch.randn(n, K, 3, generator=g) * 0.3
    pos = torch.randn(n, 3, generator=g) * 1.5
    center = torch.tensor([0.3, -4.0, 2.5])
    up = torch.randn(n, 3, generator=g)
    # float64 composition: direction, mask, compute_sh, +0.5, clamp
    s64, p64, c64 = (t.double().requires_grad_(True) for t in (shs, pos, center))
    d = p64 - c64.reshape(1, 3)
    d = d / d.norm(dim=1, keepdim=True)
    mask = torch.zeros(1, 3, K, dtype=torch.float64)
    mask[..., :active] = 1
    ref = (O.compute_sh(s64.permute(0, 2, 1) * mask, d) + 0.5).clamp(min=0)
    ref.backward(up.double())
    sg, pg, cg = (t.to(DEV).requires_grad_(True) for t in (shs, pos, center))
    out = fused.sh_rgb(sg, pg, cg, active)
    assert rel(out, ref) < 1e-6
    out.backward(up.to(DEV))
    assert rel(sg.grad, s64.grad) < 1e-5
    assert float(sg.grad[:, active:].abs().max()) == 0.0 if active < K else True
    assert rel(pg.grad, p64.grad) < 1e-5
    assert rel(cg.grad, c64.grad) < 1e-5


def test_l1_l2_loss_matches_torch():
    g = torch.Generator().manual_seed(5)
    x = torch.rand(7, 106, 160, generator=g).to(DEV).requires_grad_(True)
    t = torch.rand(7, 106, 160, generator=g).to(DEV)
    t.view(-1)[:1000] = x.detach().view(-1)[:1000]     # zero differences: sign 0
    x2 = x.detach().clone().requires_grad_(True)
    ref = F.l1_loss(x2, t) + 0.2 * F.mse_loss(x2, t)
    ref.backward()
    loss = fused.l1_l2_loss(x, t, 0.2)
    assert abs(float(loss) - float(ref)) <= 1e-6 * float(ref)
    loss.backward()
    assert float((x.grad - x2.grad).abs().max()) <= 2 ** -23 * float(x2.grad.abs().max())
    # an odd length (scalar tail) and a scaled upstream gradient
    y = torch.rand(1001, generator=g).to(DEV).requires_grad_(True)
    u = torch.rand(1001, generator=g).to(DEV)
    (3.0 * fused.l1_l2_loss(y, u, 0.5)).backward()
    y2 = y.detach().clone().requires_grad_(True)
    (3.0 * (F.l1_loss(y2, u) + 0.5 * F.mse_loss(y2, u))).backward()
    assert rel(y.grad, y2.grad) < 1e-6


def test_capturable_adam_matches_host_steps():
    g = torch.Generator().manual_seed(2)
    ps = [torch.randn(1000, 3, generator=g).to(DEV) for _ in range(3)]
    grads = [[torch.randn(1000, 3, generator=g).to(DEV) for _ in ps] for _ in range(5)]
    runs = []
    for capturable in (False, True):
        leaves = [p.clone().requires_grad_(True) for p in ps]
        opt = Adam([{"params": leaves[:2], "lr": 1e-2}, {"params": leaves[2:], "lr": 5e-3}],
                   capturable=capturable)
        for step in grads:
            for p, gr in zip(leaves, step):
                p.grad = gr.clone()
            opt.step()
        runs.append(leaves)
    for a, b in zip(*runs):
        assert rel(b, a) < 1e-6


def test_renderer_fused_colour_matches_unfused():
    scene, cam = WL.scene_small(0)
    cam = cam.to(DEV)
    outs, grads = [], []
    for fused_on in (True, False):
        leaves = [t.to(DEV).requires_grad_(True) for t in scene.activated()]
        pos, sc, q, op, shs = leaves
        shs3 = shs.detach().repeat(1, 16, 1).contiguous().requires_grad_(True)  # K = 16
        r = MsplatRender(MsplatRender.Config(render_depth=True, fused_view_colour=fused_on))
        r.sh_degree = 2
        out = r.render_iter(cam.H, cam.W, cam.extr, cam.intr, cam.center, pos, op, sc, q, shs3)
        img = out["rendered_features"]
        img.backward(torch.ones_like(img))
        outs.append(img.detach())
        grads.append([pos.grad, shs3.grad])
    assert float((outs[0] - outs[1]).abs().max()) < 1e-5
    for a, b in zip(*grads):
        assert rel(a, b) < 1e-4
    ops.check_device_status()


def test_densification_stats_match_controller():
    """One kernel against the controller's masked torch update
    (pointrix/controller/gs.py:318-333), two views, normalize_grad on."""
    from pointrix_gb300.densify import DensificationStats
    g = torch.Generator().manual_seed(8)
    n, W, H = 30_000, 640, 480
    st = DensificationStats(n, DEV, normalize_grad=True)
    ga, ac, mr = torch.zeros(n, 1), torch.zeros(n, 1), torch.zeros(n)
    for step in range(3):
        uvs, rads = [], []
        for v in range(2):
            p = torch.zeros(n, 2, requires_grad=True)
            p.grad = torch.randn(n, 2, generator=g) * 1e-3
            r = torch.randint(-2, 30, (n,), generator=g).clamp(min=0).to(torch.int32)
            uvs.append(p); rads.append(r)
        # reference update (accumulate_viewspace_grad + preprocess)
        vg = uvs[0].grad.clone() + uvs[1].grad
        vg[..., 0] *= W / 2.0
        vg[..., 1] *= H / 2.0
        radii = torch.stack(rads).max(dim=0).values
        vis = torch.stack([r > 0 for r in rads]).any(dim=0)
        mr[vis] = torch.max(mr[vis], radii[vis])
        ga[vis] += torch.norm(vg[vis, :2], dim=-1, keepdim=True)
        ac[vis] += 1
        dev_uvs = [t.detach().to(DEV).requires_grad_(True) for t in uvs]
        for a, b in zip(dev_uvs, uvs):
            a.grad = b.grad.to(DEV)
        st.preprocess([r.to(DEV) for r in rads], dev_uvs, W, H)
    assert torch.equal(st.acc_steps.cpu(), ac) and torch.equal(st.max_radii.cpu(), mr)
    assert rel(st.grad_accum, ga) < 1e-6
    avg = st.average_grad()
    assert not bool(avg.isnan().any())


def _ssim_reference(x, y):
    """pointrix/model/loss.py:ssim in float64 (conv2d with the separable
    Gaussian window, zero padding 5, groups = channels)."""
    import math
    g = torch.tensor([math.exp(-(k - 5) ** 2 / (2 * 1.5 ** 2)) for k in range(11)],
                     dtype=torch.float64)
    g = g / g.sum()
    win = (g[:, None] @ g[None, :])[None, None]
    x4, y4 = (t if t.dim() == 4 else t[None] for t in (x, y))
    C = x4.shape[1]
    w = win.expand(C, 1, 11, 11).contiguous()
    conv = lambda t: F.conv2d(t, w, padding=5, groups=C)  # noqa: E731
    mu1, mu2 = conv(x4), conv(y4)
    s11 = conv(x4 * x4) - mu1 ** 2
    s22 = conv(y4 * y4) - mu2 ** 2
    s12 = conv(x4 * y4) - mu1 * mu2
    C1, C2 = 0.01 ** 2, 0.03 ** 2
    m = ((2 * mu1 * mu2 + C1) * (2 * s12 + C2)) / ((mu1 ** 2 + mu2 ** 2 + C1) * (s11 + s22 + C2))
    return m.mean()


@pytest.mark.parametrize("shape", [(3, 70, 101), (2, 3, 33, 64), (1, 32, 32)])
def test_ssim_matches_reference(shape):
    g = torch.Generator().manual_seed(sum(shape))
    y = torch.rand(*shape, generator=g)
    x = (y + 0.1 * torch.randn(*shape, generator=g)).clamp(0, 1)
    x64 = x.double().requires_grad_(True)
    ref = _ssim_reference(x64, y.double())
    (2.0 * ref).backward()
    xg = x.to(DEV).requires_grad_(True)
    out = fused.ssim(xg, y.to(DEV))
    assert abs(float(out) - float(ref)) < 1e-6
    (2.0 * out).backward()
    assert rel(xg.grad, x64.grad) < 1e-5
    ops.check_device_status()


def test_preprocess_matches_three_operators():
    """Fused project_point + compute_cov3d + ewa_project: every forward output
    bit-identical to the three operators, gradients (position, scales,
    quaternions, intrinsics, extrinsics) within 1e-5 of the chained ones."""
    scene, cam = WL.scene_train_view(1, n=200_000)
    g = torch.Generator().manual_seed(4)
    runs = []
    for fused_on in (True, False):
        pos, sc, q, op, shs = (t.to(DEV) for t in scene.activated())
        pos, sc, q = (t.detach().requires_grad_(True) for t in (pos, sc, q))
        intr = cam.intr.to(DEV).requires_grad_(True)
        E = cam.extr.to(DEV).requires_grad_(True)
        extr = E[:3, :]
        if fused_on:
            uv, depth, conic, radius, tiles = fused.preprocess(pos, sc, q, intr, extr, cam.W, cam.H)
        else:
            uv, depth = ops.project_point(pos, intr, extr, cam.W, cam.H)
            vis = depth != 0
            cov = ops.compute_cov3d(sc, q, vis)
            conic, radius, tiles = ops.ewa_project(pos, cov, intr, extr, uv, cam.W, cam.H, vis)
        gen = torch.Generator().manual_seed(11)
        ups = [torch.randn(t.shape, generator=gen).to(DEV) for t in (uv, depth, conic)]
        torch.autograd.backward([uv, depth, conic], ups)
        runs.append(([uv, depth, conic, radius, tiles], [pos.grad, sc.grad, q.grad, intr.grad, E.grad]))
    for a, b in zip(runs[0][0], runs[1][0]):
        assert torch.equal(a, b)
    for a, b in zip(runs[0][1], runs[1][1]):
        assert rel(a, b) < 1e-5
    ops.check_device_status()


def test_sh_rgb_views_matches_per_view():
    """Colour of several views in one pass equals the per-view fused colour;
    gradients (summed over views for sh and position, per view for the
    centres) within 1e-5."""
    g = torch.Generator().manual_seed(21)
    n, K, V = 30_000 + 7, 16, 5
    shs = (torch.randn(n, K, 3, generator=g) * 0.3).to(DEV)
    pos = (torch.randn(n, 3, generator=g) * 1.5).to(DEV)
    centres = (torch.randn(V, 3, generator=g) * 4.0).to(DEV)
    ups = torch.randn(V, n, 3, generator=g).to(DEV)
    a = [t.clone().requires_grad_(True) for t in (shs, pos, centres)]
    out = fused.sh_rgb_views(a[0], a[1], a[2], 9)
    out.backward(ups)
    b = [t.clone().requires_grad_(True) for t in (shs, pos, centres)]
    ref = torch.stack([fused.sh_rgb(b[0], b[1], b[2][v], 9) for v in range(V)])
    ref.backward(ups)
    assert torch.equal(out, ref.detach())
    for x, y in zip(a, b):
        assert rel(x.grad, y.grad) < 1e-5
    ops.check_device_status()


def test_camera_pose_matches_torch_composition():
    """fused.camera_pose against the torch composition (quaternion
    normalisation, homogeneous rotation, [R t; 0 1], -R^T t): values and the
    gradients of both outputs to 1e-5."""
    g = torch.Generator().manual_seed(9)
    q0 = torch.randn(4, generator=g) * 2.0
    t0 = torch.randn(3, generator=g) * 3.0
    dE = torch.randn(4, 4, generator=g).to(DEV)
    dc = torch.randn(3, generator=g).to(DEV)
    q, t = q0.to(DEV).requires_grad_(True), t0.to(DEV).requires_grad_(True)
    E, c = fused.camera_pose(q, t)
    ((E * dE).sum() + (c * dc).sum()).backward()
    qr, tr = q0.to(DEV).requires_grad_(True), t0.to(DEV).requires_grad_(True)
    R = WL.rotation_from_unit_quat(qr / qr.norm())
    Er = torch.cat([torch.cat([R, tr[:, None]], 1), torch.tensor([[0.0, 0, 0, 1]], device=DEV)], 0)
    cr = -(R.T @ tr)
    ((Er * dE).sum() + (cr * dc).sum()).backward()
    assert torch.allclose(E, Er, atol=1e-6) and torch.allclose(c, cr, atol=1e-5)
    assert torch.allclose(q.grad, qr.grad, rtol=1e-5, atol=1e-5)
    assert torch.allclose(t.grad, tr.grad, rtol=1e-5, atol=1e-5)
    # one output unused: its gradient arrives as None
    q2, t2 = q0.to(DEV).requires_grad_(True), t0.to(DEV).requires_grad_(True)
    E2, _ = fused.camera_pose(q2, t2)
    (E2 * dE).sum().backward()
    q3, t3 = q0.to(DEV).requires_grad_(True), t0.to(DEV).requires_grad_(True)
    R3 = WL.rotation_from_unit_quat(q3 / q3.norm())
    E3 = torch.cat([torch.cat([R3, t3[:, None]], 1), torch.tensor([[0.0, 0, 0, 1]], device=DEV)], 0)
    (E3 * dE).sum().backward()
    assert torch.allclose(q2.grad, q3.grad, rtol=1e-5, atol=1e-5)
    assert torch.allclose(t2.grad, t3.grad, rtol=1e-5, atol=1e-5)
