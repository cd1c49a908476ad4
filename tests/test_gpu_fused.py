"""Fused caller-side passes against the torch compositions they replace.

Bars: forward values within 1e-6 (relative to the largest entry) of the
float64 composition; gradients within 1e-5 relative to the largest
gradient entry (they are short float32 chains); the loss gradient equal to
torch's l1_loss + w * mse_loss gradient to 1 ulp.
"""
import os

import pytest
import torch
import torch.nn.functional as F

from oracle import msplat_cpu as O
from pointrix_gb300 import fused, ops
from pointrix_gb300 import workloads as WL
from pointrix_gb300.optim import Adam
from pointrix_gb300.camera import unitquat_to_rotmat as cam_rotmat
from pointrix_gb300.renderer import MsplatRender
from tests import refload

pytestmark = pytest.mark.gpu
DEV = "cuda"


def rel(a, b):
    if b is None:          # no dependence in the reference: expect zeros
        return float(a.detach().abs().max())
    a, b = a.detach().double().cpu(), b.detach().double().cpu()
    return float((a - b).abs().max() / b.abs().max().clamp(min=1e-30))


def _rotmat():
    """``pointrix/utils/pose.py:unitquat_to_rotmat`` itself where the reference
    is installed, else the camera model's form (equal to it bit for bit on the
    fixture, ``tests/test_reference_glue.py``)."""
    pose = refload.pose()
    return pose.unitquat_to_rotmat if pose is not None else cam_rotmat


def torch_activations(ls, q, lg):
    """The reference composition in float64 (gaussian_points.py:70-80,
    examples/supervise/model.py:50-62 with pose.py's matrix)."""
    s = torch.exp(ls)
    r = F.normalize(q, dim=-1)
    o = torch.sigmoid(lg)
    idx = torch.argmin(ls, dim=-1)
    cols = _rotmat()(r).transpose(-1, -2)           # [N, axis, 3]
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
    assert abs(float(loss.detach()) - float(ref)) <= 1e-6 * float(ref)
    loss.backward()
    assert float((x.grad - x2.grad).abs().max()) <= 2 ** -23 * float(x2.grad.abs().max())
    # an odd length (scalar tail) and a scaled upstream gradient
    y = torch.rand(1001, generator=g).to(DEV).requires_grad_(True)
    u = torch.rand(1001, generator=g).to(DEV)
    (3.0 * fused.l1_l2_loss(y, u, 0.5)).backward()
    y2 = y.detach().clone().requires_grad_(True)
    (3.0 * (F.l1_loss(y2, u) + 0.5 * F.mse_loss(y2, u))).backward()
    assert rel(y.grad, y2.grad) < 1e-6


def test_l1_l2_loss_gradient_from_the_forward_pass():
    """The gradient the forward writes for an upstream 1, and the backward's
    rewrite for any other upstream gradient, equal the plain backward
    (pgb_l1_l2_loss_backward) bit for bit; a retained graph's second
    backward recomputes it.  Odd length: the scalar tail too."""
    from pointrix_gb300 import _lib
    g = torch.Generator().manual_seed(9)
    x = torch.rand(7, 53, 81, generator=g).to(DEV)
    t = torch.rand(7, 53, 81, generator=g).to(DEV)
    t.view(-1)[:500] = x.view(-1)[:500]                # zero differences: sign 0
    stream = torch.cuda.current_stream().cuda_stream

    def plain(dl):
        dx = torch.empty_like(x)
        d = torch.tensor([dl], dtype=torch.float32, device=DEV)
        _lib.call("pgb_l1_l2_loss_backward", x.data_ptr(), t.data_ptr(), x.numel(), 0.2,
                  d.data_ptr(), dx.data_ptr(), stream)
        return dx

    for dl in (1.0, 2.5, -0.75):
        xr = x.clone().requires_grad_(True)
        loss = fused.l1_l2_loss(xr, t, 0.2)
        (dl * loss).backward(retain_graph=True)
        assert torch.equal(xr.grad, plain(dl)), dl
        xr.grad = None
        (dl * loss).backward()
        assert torch.equal(xr.grad, plain(dl)), dl
    # no gradient wanted: the plain forward, the same loss
    with torch.no_grad():
        l0 = fused.l1_l2_loss(x, t, 0.2)
    assert float(l0) == float(fused.l1_l2_loss(x.clone().requires_grad_(True), t, 0.2).detach())


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
    for a, b, p0 in zip(*runs, ps):
        assert float((a - p0).abs().max()) > 1e-4      # the steps moved the parameters
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


GLUE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference", "glue.pt")


def _glue():
    return torch.load(GLUE, weights_only=False)


def _reference_controller(n, W, H):
    """The reference's ``DensificationController`` (``pointrix/controller/gs.py``)
    with only the state its ``preprocess`` reads; None where the reference is
    not installed."""
    gs = refload.gs_controller()
    if gs is None:
        return None
    from types import SimpleNamespace
    ctrl = object.__new__(gs.DensificationController)
    ctrl.cfg = SimpleNamespace(normalize_grad=True)
    ctrl.width, ctrl.height = W, H
    ctrl.grad_accum = torch.zeros(n, 1)
    ctrl.acc_steps = torch.zeros(n, 1)
    ctrl.max_radii = torch.zeros(n)
    return ctrl


def _stats_step(st, rads, grads, W, H):
    dev_uvs = []
    for gr in grads:
        p = torch.zeros(gr.shape, device=DEV, requires_grad=True)
        p.grad = gr.to(DEV)
        dev_uvs.append(p)
    st.preprocess([r.to(DEV) for r in rads], dev_uvs, W, H)


def test_densification_stats_match_controller_fixture():
    """One kernel against the reference controller's masked torch update
    (``preprocess`` + ``accumulate_viewspace_grad``, pointrix/controller/gs.py:
    260-284, 318-333), as recorded by executing it: two views per step,
    normalize_grad on, three steps."""
    from pointrix_gb300.densify import DensificationStats
    c = _glue()["controller"]
    st = DensificationStats(c["n"], DEV, normalize_grad=True)
    for step in c["steps"]:
        _stats_step(st, step["radii"], step["uv_grads"], c["W"], c["H"])
        assert torch.equal(st.acc_steps.cpu(), step["acc_steps"])
        assert torch.equal(st.max_radii.cpu(), step["max_radii"])
        assert rel(st.grad_accum, step["grad_accum"]) < 1e-6
    assert not bool(st.average_grad().isnan().any())


@pytest.mark.skipif(refload.pointrix_dir() is None, reason="reference source not installed")
def test_densification_stats_match_controller_live():
    """The same against the reference controller run here, 30,000 points."""
    from pointrix_gb300.densify import DensificationStats
    g = torch.Generator().manual_seed(8)
    n, W, H = 30_000, 640, 480
    ctrl = _reference_controller(n, W, H)
    st = DensificationStats(n, DEV, normalize_grad=True)
    for _ in range(3):
        uvs, rads = [], []
        for _v in range(2):
            p = torch.zeros(n, 2, requires_grad=True)
            p.grad = torch.randn(n, 2, generator=g) * 1e-3
            uvs.append(p)
            rads.append(torch.randint(-2, 30, (n,), generator=g).clamp(min=0).to(torch.int32))
        vis = torch.cat([(r > 0).unsqueeze(0) for r in rads]).any(dim=0)
        radii = torch.cat([r.unsqueeze(0) for r in rads], 0).max(dim=0).values
        ctrl.preprocess(visibility=vis, radii=radii, uv_points=uvs)
        _stats_step(st, rads, [p.grad for p in uvs], W, H)
    assert torch.equal(st.acc_steps.cpu(), ctrl.acc_steps)
    assert torch.equal(st.max_radii.cpu(), ctrl.max_radii)
    assert rel(st.grad_accum, ctrl.grad_accum) < 1e-6


def test_ssim_matches_reference_fixture():
    """Fused SSIM against the value and gradient the reference's ``ssim``
    (pointrix/model/loss.py:71-125) gave in float64."""
    c = _glue()["ssim"]
    xg = c["x"].float().to(DEV).requires_grad_(True)
    out = fused.ssim(xg, c["y"].float().to(DEV))
    assert abs(float(out) - float(c["value"])) < 1e-6
    out.backward()
    assert rel(xg.grad, c["grad"]) < 1e-5
    ops.check_device_status()


@pytest.mark.skipif(refload.pointrix_dir() is None, reason="reference source not installed")
@pytest.mark.parametrize("shape", [(3, 70, 101), (2, 3, 33, 64), (1, 32, 32)])
def test_ssim_matches_reference_live(shape):
    ssim_ref = refload.loss().ssim
    g = torch.Generator().manual_seed(sum(shape))
    y = torch.rand(*shape, generator=g)
    x = (y + 0.1 * torch.randn(*shape, generator=g)).clamp(0, 1)
    x64 = x.double().requires_grad_(True)
    ref = ssim_ref(x64, y.double())
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


def test_preprocess_views_matches_per_view_preprocess():
    """The batched projection of V views: each view's outputs equal the
    single-view preprocess bit for bit; the Gaussian gradients (summed over
    views in the kernel) and every camera's gradients equal the per-view
    calls' autograd sums within 1e-5."""
    g = torch.Generator().manual_seed(12)
    scene = WL.scene_sh3(12, 60_000)
    cams = [WL.make_camera(g, W, H, 0.72 * W, 4.5) for W, H in ((320, 240), (200, 150), (257, 190))]
    pos, sc, q, _, _ = (t.to(DEV) for t in scene.activated())
    leaves = lambda: [t.detach().clone().requires_grad_(True) for t in (pos, sc, q)]  # noqa: E731
    intr = [c.intr.to(DEV).reshape(4).clone().requires_grad_(True) for c in cams]
    extr = [c.extr[:3].to(DEV).contiguous().requires_grad_(True) for c in cams]
    sizes = [(c.W, c.H) for c in cams]
    ups = [torch.randn(len(cams) * pos.shape[0], k, generator=g).to(DEV) for k in (2, 1, 3)]
    la = leaves()
    outs = fused.preprocess_views(*la, torch.stack(intr), torch.stack(extr), sizes)
    torch.autograd.backward(list(outs[:3]), ups)
    ga = [t.grad.clone() for t in la] + [t.grad.clone() for t in intr + extr]
    for t in intr + extr:
        t.grad = None
    lb = leaves()
    per = [fused.preprocess(*lb, intr[v], extr[v], W, H) for v, (W, H) in enumerate(sizes)]
    for k in range(5):
        assert torch.equal(outs[k], torch.cat([p[k] for p in per])), k
    n = pos.shape[0]
    torch.autograd.backward([p[k] for p in per for k in range(3)],
                            [u[v * n:(v + 1) * n] for v in range(len(cams)) for u in ups])
    gb = [t.grad for t in lb] + [t.grad for t in intr + extr]
    for a, b in zip(ga, gb):
        assert rel(a, b) < 1e-5
    ops.check_device_status()
