"""Fused caller-side passes of the training step (no msplat counterpart).

Around the msplat operators, a Pointrix training step spends a dozen torch
kernels each on the parameter activations and the normal feature
(``pointrix/model/point_cloud/gaussian_points.py:70-80``,
``examples/supervise/model.py:50-62``), on the view colour glue of
``MsplatRender.render_iter`` (``pointrix/model/renderer/msplat.py:94-105``)
and on the loss.  Each function here does the same arithmetic in one kernel
forward and one backward:

* :func:`gaussian_activations` -- exp(log_scale), F.normalize(quat),
  sigmoid(logit) and the shortest-axis normal;
* :func:`sh_rgb` -- clamp(compute_sh(masked sh, normalize(xyz - center)) +
  0.5, min=0), with gradients to sh, xyz and the camera centre;
* :func:`l1_l2_loss` -- mean|x - t| + w mean((x - t)^2);
* :func:`ssim` -- the SSIM of ``pointrix/model/loss.py:71-125`` (one tiled
  kernel forward, one backward);
* :func:`preprocess` -- ``project_point``, ``compute_cov3d`` and
  ``ewa_project`` as ``render_iter`` chains them
  (``pointrix/model/renderer/msplat.py:109-130``), outputs bit-identical to
  the three operators.
"""
from __future__ import annotations

import torch

from . import _lib
from ._lib import call
from .ops import EXTENT_DEFAULT, NEAREST_DEFAULT, _c, _extr34, _intr4, _ptr, _stream, _timed

__all__ = ["gaussian_activations", "sh_rgb", "sh_rgb_views", "sh_rgb_supported", "l1_l2_loss",
           "ssim", "preprocess", "camera_pose"]


def _aligned(t: torch.Tensor) -> bool:
    return t.data_ptr() % 16 == 0


def _c16(t: torch.Tensor) -> torch.Tensor:
    """Contiguous float32 with a 16-byte aligned start (copied if not)."""
    t = _c(t)
    return t if _aligned(t) else t.clone()


# ---------------------------------------------------------------------------
class _Activate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, log_scale, quat, logit, normals):
        n = log_scale.shape[0]
        dev = log_scale.device
        scaling = torch.empty(n, 3, dtype=torch.float32, device=dev)
        rotation = torch.empty(n, 4, dtype=torch.float32, device=dev)
        opacity = torch.empty(logit.shape, dtype=torch.float32, device=dev)
        normal = torch.empty(n, 3, dtype=torch.float32, device=dev) if normals else None
        with _timed("gaussian_activate_fwd", dev, 1 if n else 0):
            call("pgb_gaussian_activate_forward", _ptr(log_scale), _ptr(quat), _ptr(logit), n,
                 _ptr(scaling), _ptr(rotation), _ptr(opacity), _ptr(normal) if normals else None,
                 _stream(dev))
        ctx.save_for_backward(log_scale, quat, logit)
        if normal is None:
            normal = torch.empty(0, 3, dtype=torch.float32, device=dev)
            ctx.mark_non_differentiable(normal)
        return scaling, rotation, opacity, normal

    @staticmethod
    def backward(ctx, d_scaling, d_rotation, d_opacity, d_normal):
        log_scale, quat, logit = ctx.saved_tensors
        n = log_scale.shape[0]
        dev = log_scale.device
        d_ls = torch.empty_like(log_scale)
        d_q = torch.empty_like(quat)
        d_lg = torch.empty_like(logit)

        def g(t, aligned=False):
            if t is None or t.numel() == 0:
                return None
            return _c16(t) if aligned else _c(t)

        d_scaling, d_rotation = g(d_scaling), g(d_rotation, True)
        d_opacity, d_normal = g(d_opacity), g(d_normal)
        with _timed("gaussian_activate_bwd", dev, 1 if n else 0):
            call("pgb_gaussian_activate_backward", _ptr(log_scale), _ptr(quat), _ptr(logit), n,
                 _ptr(d_scaling) if d_scaling is not None else None,
                 _ptr(d_rotation) if d_rotation is not None else None,
                 _ptr(d_opacity) if d_opacity is not None else None,
                 _ptr(d_normal) if d_normal is not None else None,
                 _ptr(d_ls), _ptr(d_q), _ptr(d_lg), _stream(dev))
        return d_ls, d_q, d_lg, None


def gaussian_activations(log_scale, quat, opacity_logit, normals=True):
    """(scaling [N,3], rotation [N,4], opacity (shape of the logit), normal
    [N,3] or None) from the stored Gaussian parameters: exp, F.normalize
    (eps 1e-12), sigmoid, and normalize(R(rotation)[:, argmin(log_scale)])
    with R the wxyz unit-quaternion matrix.  Differentiable in all three
    inputs."""
    if log_scale.dim() != 2 or log_scale.shape[1] != 3:
        raise ValueError(f"log_scale must be [N,3], got {tuple(log_scale.shape)}")
    n = log_scale.shape[0]
    if tuple(quat.shape) != (n, 4):
        raise ValueError(f"quat must be [N,4], got {tuple(quat.shape)}")
    if opacity_logit.numel() != n:
        raise ValueError("opacity_logit must hold N values")
    for name, t in (("log_scale", log_scale), ("quat", quat), ("opacity_logit", opacity_logit)):
        if not t.is_cuda or t.dtype != torch.float32:
            raise ValueError(f"{name} must be a CUDA float32 tensor")
    s, r, o, nrm = _Activate.apply(_c(log_scale), _c16(quat), _c(opacity_logit), bool(normals))
    return s, r, o, (nrm if normals else None)


# ---------------------------------------------------------------------------
_SH_K = (1, 4, 9, 16)


def sh_rgb_supported(shs) -> bool:
    """True when ``shs`` ([N,K,3]) is dense storage the fused kernel reads."""
    return (shs.is_cuda and shs.dtype == torch.float32 and shs.dim() == 3 and shs.shape[2] == 3
            and shs.shape[1] in _SH_K and shs.is_contiguous() and _aligned(shs))


class _ShRgb(torch.autograd.Function):
    @staticmethod
    def forward(ctx, shs, xyz, center, active):
        n, K = shs.shape[0], shs.shape[1]
        dev = shs.device
        rgb = torch.empty(n, 3, dtype=torch.float32, device=dev)
        with _timed("sh_rgb_fwd", dev, 1 if n else 0):
            call("pgb_sh_rgb_forward", _ptr(shs), n, K, active, _ptr(xyz), _ptr(center), _ptr(rgb),
                 _stream(dev))
        ctx.save_for_backward(shs, xyz, center)
        ctx.active = active
        return rgb

    @staticmethod
    def backward(ctx, d_rgb):
        shs, xyz, center = ctx.saved_tensors
        n, K = shs.shape[0], shs.shape[1]
        dev = shs.device
        d_sh = torch.empty_like(shs)
        d_xyz = torch.empty_like(xyz)
        d_center = torch.empty(3, dtype=torch.float32, device=dev)
        nf = _lib.lib().pgb_sh_rgb_scratch_floats(n)
        scratch = torch.empty(max(nf, 1), dtype=torch.float32, device=dev)
        with _timed("sh_rgb_bwd", dev, 2 if n else 0):
            call("pgb_sh_rgb_backward", _ptr(shs), n, K, ctx.active, _ptr(xyz), _ptr(center),
                 _ptr(_c(d_rgb)), _ptr(d_sh), _ptr(d_xyz), _ptr(d_center), _ptr(scratch), nf,
                 _stream(dev))
        return d_sh, d_xyz, d_center, None


def sh_rgb(shs, position, camera_center, active=None):
    """clamp(compute_sh(shs.permute(0,2,1) * mask, normalize(position -
    center)) + 0.5, min=0) -> [N,3], the mask keeping the first ``active``
    coefficients (all when None).  ``shs`` is the [N,K,3] storage (see
    :func:`sh_rgb_supported`); gradients flow to shs, position and the
    camera centre ([3] or any shape of 3 elements)."""
    if not sh_rgb_supported(shs):
        raise ValueError("sh_rgb needs dense, 16-byte aligned CUDA float32 shs [N,K,3], K in 1/4/9/16")
    n, K = shs.shape[0], shs.shape[1]
    if tuple(position.shape) != (n, 3):
        raise ValueError(f"position must be [N,3], got {tuple(position.shape)}")
    if camera_center.numel() != 3:
        raise ValueError("camera_center must hold 3 values")
    active = K if active is None else max(0, min(int(active), K))
    return _ShRgb.apply(shs, _c(position), _c(camera_center.reshape(3)), active)


class _ShRgbViews(torch.autograd.Function):
    @staticmethod
    def forward(ctx, shs, xyz, centres, active):
        n, K = shs.shape[0], shs.shape[1]
        V = centres.shape[0]
        dev = shs.device
        rgb = torch.empty(V, n, 3, dtype=torch.float32, device=dev)
        with _timed("sh_rgb_views_fwd", dev, 1 if n else 0):
            call("pgb_sh_rgb_views_forward", _ptr(shs), n, K, active, _ptr(xyz), _ptr(centres), V,
                 _ptr(rgb), _stream(dev))
        ctx.save_for_backward(shs, xyz, centres)
        ctx.active = active
        return rgb

    @staticmethod
    def backward(ctx, d_rgb):
        shs, xyz, centres = ctx.saved_tensors
        n, K = shs.shape[0], shs.shape[1]
        V = centres.shape[0]
        dev = shs.device
        d_sh = torch.empty_like(shs)
        d_xyz = torch.empty_like(xyz)
        d_c = torch.empty(V, 3, dtype=torch.float32, device=dev)
        nf = _lib.lib().pgb_sh_rgb_views_scratch_floats(n)
        scratch = torch.empty(max(nf, 1), dtype=torch.float32, device=dev)
        with _timed("sh_rgb_views_bwd", dev, 2 if n else 0):
            call("pgb_sh_rgb_views_backward", _ptr(shs), n, K, ctx.active, _ptr(xyz), _ptr(centres),
                 V, _ptr(_c(d_rgb)), _ptr(d_sh), _ptr(d_xyz), _ptr(d_c), _ptr(scratch), nf,
                 _stream(dev))
        return d_sh, d_xyz, d_c, None


def sh_rgb_views(shs, position, centres, active=None):
    """:func:`sh_rgb` for V camera centres ([V,3], V <= 64) in one pass over
    the coefficients -> [V,N,3]; gradients to shs and position are summed
    over the views, each centre gets its own."""
    if not sh_rgb_supported(shs):
        raise ValueError("sh_rgb_views needs dense, 16-byte aligned CUDA float32 shs [N,K,3]")
    n, K = shs.shape[0], shs.shape[1]
    if tuple(position.shape) != (n, 3):
        raise ValueError(f"position must be [N,3], got {tuple(position.shape)}")
    if centres.dim() != 2 or centres.shape[1] != 3 or not 1 <= centres.shape[0] <= 64:
        raise ValueError(f"centres must be [V,3] with 1 <= V <= 64, got {tuple(centres.shape)}")
    active = K if active is None else max(0, min(int(active), K))
    return _ShRgbViews.apply(shs, _c(position), _c(centres), active)


# ---------------------------------------------------------------------------
class _L1L2(torch.autograd.Function):
    """When x needs a gradient, the forward also writes the gradient for an
    upstream 1 in the same pass over x and t (a training step's loss is its
    output, so that is the gradient it gets); the first backward hands that
    buffer over and only rewrites it if the upstream gradient is not 1 (a
    check on the device, so the step stays capturable).  A second backward
    through a retained graph recomputes from x and t."""

    @staticmethod
    def forward(ctx, x, t, w):
        n = x.numel()
        dev = x.device
        nd = _lib.lib().pgb_l1_l2_loss_scratch_doubles(n)
        scratch = torch.empty(nd, dtype=torch.float64, device=dev)
        loss = torch.empty((), dtype=torch.float32, device=dev)
        ctx.dx_unit = None
        with _timed("l1_l2_loss_fwd", dev, 2):
            if ctx.needs_input_grad[0]:
                ctx.dx_unit = torch.empty_like(x)
                call("pgb_l1_l2_loss_forward_grad", _ptr(x), _ptr(t), n, w, _ptr(scratch), nd,
                     _ptr(loss), _ptr(ctx.dx_unit), _stream(dev))
            else:
                call("pgb_l1_l2_loss_forward", _ptr(x), _ptr(t), n, w, _ptr(scratch), nd,
                     _ptr(loss), _stream(dev))
        ctx.save_for_backward(x, t)
        ctx.w = w
        return loss

    @staticmethod
    def backward(ctx, d_loss):
        x, t = ctx.saved_tensors
        dev = x.device
        dx, ctx.dx_unit = ctx.dx_unit, None
        with _timed("l1_l2_loss_bwd", dev, 1):
            if dx is not None:
                call("pgb_l1_l2_loss_backward_unit", _ptr(x), _ptr(t), x.numel(), ctx.w,
                     _ptr(_c(d_loss.reshape(1))), _ptr(dx), _stream(dev))
            else:
                dx = torch.empty_like(x)
                call("pgb_l1_l2_loss_backward", _ptr(x), _ptr(t), x.numel(), ctx.w,
                     _ptr(_c(d_loss.reshape(1))), _ptr(dx), _stream(dev))
        return dx, None, None


def l1_l2_loss(x, target, w_l2=0.0):
    """mean|x - target| + w_l2 * mean((x - target)^2) as a 0-dim tensor;
    differentiable in ``x`` (the same gradient as torch's l1_loss +
    w_l2 * mse_loss)."""
    if x.shape != target.shape:
        raise ValueError(f"shape mismatch {tuple(x.shape)} vs {tuple(target.shape)}")
    if x.numel() == 0:
        raise ValueError("l1_l2_loss of an empty tensor")
    if not (x.is_cuda and target.is_cuda and x.dtype == torch.float32 and target.dtype == torch.float32):
        raise ValueError("l1_l2_loss takes CUDA float32 tensors")
    return _L1L2.apply(_c16(x), _c16(target.detach()), float(w_l2))


# ---------------------------------------------------------------------------
class _Ssim(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, planes, H, W):
        dev = x.device
        nd = int(_lib.lib().pgb_ssim_scratch_doubles(planes, H, W))
        scratch = torch.empty(max(nd, 1), dtype=torch.float64, device=dev)
        out = torch.empty((), dtype=torch.float32, device=dev)
        with _timed("ssim_fwd", dev, 2):
            call("pgb_ssim_forward", _ptr(x), _ptr(y), planes, H, W, _ptr(scratch), nd, _ptr(out),
                 _stream(dev))
        ctx.save_for_backward(x, y)
        ctx.dims = (planes, H, W)
        return out

    @staticmethod
    def backward(ctx, d_out):
        x, y = ctx.saved_tensors
        planes, H, W = ctx.dims
        dx = torch.empty_like(x)
        with _timed("ssim_bwd", x.device, 1):
            call("pgb_ssim_backward", _ptr(x), _ptr(y), planes, H, W, _ptr(_c(d_out.reshape(1))),
                 _ptr(dx), _stream(x.device))
        return dx, None, None, None, None


def ssim(img1, img2, window_size=11, size_average=True):
    """SSIM of ``img1`` against the target ``img2`` ([C,H,W] or [B,C,H,W]),
    as ``pointrix/model/loss.py:ssim`` with its defaults (11x11 window,
    sigma 1.5, mean over everything); differentiable in ``img1`` (``img2`` is
    treated as a constant target)."""
    if window_size != 11 or not size_average:
        raise ValueError("fused ssim supports window_size=11, size_average=True")
    if img1.shape != img2.shape or img1.dim() not in (3, 4):
        raise ValueError(f"ssim takes two [C,H,W] or [B,C,H,W] images of one shape, got "
                         f"{tuple(img1.shape)} and {tuple(img2.shape)}")
    if not (img1.is_cuda and img2.is_cuda and img1.dtype == torch.float32
            and img2.dtype == torch.float32):
        raise ValueError("ssim takes CUDA float32 images")
    H, W = img1.shape[-2], img1.shape[-1]
    planes = img1.numel() // (H * W)
    return _Ssim.apply(_c(img1), _c(img2.detach()), planes, H, W)


# ---------------------------------------------------------------------------
class _Preprocess(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, scales, quats, intr, extr, W, H, nearest, extent):
        n = xyz.shape[0]
        dev = xyz.device
        uv = torch.empty(n, 2, dtype=torch.float32, device=dev)
        depth = torch.empty(n, 1, dtype=torch.float32, device=dev)
        conic = torch.empty(n, 3, dtype=torch.float32, device=dev)
        radius = torch.empty(n, dtype=torch.int32, device=dev)
        tiles = torch.empty(n, dtype=torch.int32, device=dev)
        with _timed("preprocess_fwd", dev, 1 if n else 0):
            call("pgb_preprocess_forward", _ptr(xyz), _ptr(scales), _ptr(quats), n, _ptr(intr),
                 _ptr(extr), W, H, nearest, extent, _ptr(uv), _ptr(depth), _ptr(conic),
                 _ptr(radius), _ptr(tiles), _stream(dev))
        ctx.save_for_backward(xyz, scales, quats, intr, extr, radius)
        ctx.cfg = (W, H, nearest, extent)
        ctx.mark_non_differentiable(radius, tiles)
        ctx.set_materialize_grads(False)  # no zero tensors for radius / tiles
        return uv, depth, conic, radius, tiles

    @staticmethod
    def backward(ctx, d_uv, d_depth, d_conic, _d_radius, _d_tiles):
        xyz, scales, quats, intr, extr, radius = ctx.saved_tensors
        W, H, nearest, extent = ctx.cfg
        n = xyz.shape[0]
        dev = xyz.device
        g = lambda t, *shape: torch.zeros(*shape, device=dev) if t is None else _c(t)  # noqa: E731
        d_uv, d_depth, d_conic = g(d_uv, n, 2), g(d_depth, n, 1), g(d_conic, n, 3)
        d_xyz, d_scales, d_quats = torch.empty_like(xyz), torch.empty_like(scales), torch.empty_like(quats)
        d_intr = torch.empty(4, dtype=torch.float32, device=dev)
        d_extr = torch.empty(3, 4, dtype=torch.float32, device=dev)
        nbytes = _lib.lib().pgb_camera_grad_scratch_bytes()
        scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        with _timed("preprocess_bwd", dev, 2):
            call("pgb_preprocess_backward", _ptr(xyz), _ptr(scales), _ptr(quats), n, _ptr(intr),
                 _ptr(extr), W, H, nearest, extent, _ptr(radius), _ptr(d_uv), _ptr(d_depth),
                 _ptr(d_conic), _ptr(d_xyz), _ptr(d_scales), _ptr(d_quats), _ptr(d_intr),
                 _ptr(d_extr), _ptr(scratch), nbytes, _stream(dev))
        return d_xyz, d_scales, d_quats, d_intr, d_extr, None, None, None, None


def preprocess(position, scaling, rotation, intr, extr, W, H, nearest=NEAREST_DEFAULT,
               extent=EXTENT_DEFAULT):
    """(uv [N,2], depth [N,1], conic [N,3], radius [N], tiles_touched [N]) of
    ``project_point`` -> ``compute_cov3d(visible = depth != 0)`` ->
    ``ewa_project`` in one kernel each way; the same values, bit for bit, as
    the three operators, and the same gradients up to summation order.
    ``intr`` is [4] or [1,4], ``extr`` the world->camera [3,4]."""
    n = position.shape[0]
    for name, t, last in (("position", position, 3), ("scaling", scaling, 3), ("rotation", rotation, 4)):
        if t.dim() != 2 or t.shape[0] != n or t.shape[1] != last:
            raise ValueError(f"{name} must be [N,{last}], got {tuple(t.shape)}")
        if not (t.is_cuda and t.dtype == torch.float32):
            raise ValueError(f"{name} must be a CUDA float32 tensor")
    return _Preprocess.apply(_c(position), _c(scaling), _c16(rotation), _intr4(intr), _extr34(extr),
                             int(W), int(H), float(nearest), float(extent))


class _PreprocessViews(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xyz, scales, quats, intrs, extrs, sizes, nearest, extent):
        n = xyz.shape[0]
        V = len(sizes)
        dev = xyz.device
        uv = torch.empty(V * n, 2, dtype=torch.float32, device=dev)
        depth = torch.empty(V * n, 1, dtype=torch.float32, device=dev)
        conic = torch.empty(V * n, 3, dtype=torch.float32, device=dev)
        radius = torch.empty(V * n, dtype=torch.int32, device=dev)
        tiles = torch.empty(V * n, dtype=torch.int32, device=dev)
        sz = _sizes_table(sizes)
        with _timed("preprocess_fwd", dev, 1 if n else 0):
            call("pgb_preprocess_views_forward", _ptr(xyz), _ptr(scales), _ptr(quats), n,
                 _ptr(intrs), _ptr(extrs), sz, V, nearest, extent, _ptr(uv), _ptr(depth),
                 _ptr(conic), _ptr(radius), _ptr(tiles), _stream(dev))
        ctx.save_for_backward(xyz, scales, quats, intrs, extrs, radius)
        ctx.cfg = (tuple(sizes), nearest, extent)
        ctx.mark_non_differentiable(radius, tiles)
        ctx.set_materialize_grads(False)  # no zero tensors for radius / tiles
        return uv, depth, conic, radius, tiles

    @staticmethod
    def backward(ctx, d_uv, d_depth, d_conic, _d_radius, _d_tiles):
        xyz, scales, quats, intrs, extrs, radius = ctx.saved_tensors
        sizes, nearest, extent = ctx.cfg
        n, V = xyz.shape[0], len(sizes)
        dev = xyz.device
        g = lambda t, *shape: torch.zeros(*shape, device=dev) if t is None else _c(t)  # noqa: E731
        d_uv, d_depth, d_conic = g(d_uv, V * n, 2), g(d_depth, V * n, 1), g(d_conic, V * n, 3)
        d_xyz, d_scales, d_quats = torch.empty_like(xyz), torch.empty_like(scales), torch.empty_like(quats)
        d_intrs = torch.empty(V, 4, dtype=torch.float32, device=dev)
        d_extrs = torch.empty(V, 3, 4, dtype=torch.float32, device=dev)
        nbytes = _lib.lib().pgb_camera_grad_views_scratch_bytes(V)
        scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        with _timed("preprocess_bwd", dev, 2):
            call("pgb_preprocess_views_backward", _ptr(xyz), _ptr(scales), _ptr(quats), n,
                 _ptr(intrs), _ptr(extrs), _sizes_table(sizes), V, nearest, extent, _ptr(radius),
                 _ptr(d_uv), _ptr(d_depth), _ptr(d_conic), _ptr(d_xyz), _ptr(d_scales),
                 _ptr(d_quats), _ptr(d_intrs), _ptr(d_extrs), _ptr(scratch), nbytes, _stream(dev))
        return d_xyz, d_scales, d_quats, d_intrs, d_extrs, None, None, None


def _sizes_table(sizes):
    import ctypes
    arr = (ctypes.c_int32 * (2 * len(sizes)))()
    for i, (W, H) in enumerate(sizes):
        arr[2 * i], arr[2 * i + 1] = int(W), int(H)
    return arr


def preprocess_views(position, scaling, rotation, intrs, extrs, sizes, nearest=NEAREST_DEFAULT,
                     extent=EXTENT_DEFAULT):
    """:func:`preprocess` for V views at once: ``intrs`` [V,4], ``extrs``
    [V,3,4], ``sizes`` [(W, H)] * V; returns view-major uv [V*N,2], depth
    [V*N,1], conic [V*N,3], radius [V*N], tiles_touched [V*N] (each view's
    block equal bit for bit to its single-view call).  One kernel each way:
    the backward sums the Gaussian gradients over the views itself, so the
    V per-view gradients are never materialised and added."""
    n = position.shape[0]
    V = len(sizes)
    if V < 1 or V > 64:
        raise ValueError(f"preprocess_views takes 1..64 views, got {V}")
    for name, t, last in (("position", position, 3), ("scaling", scaling, 3), ("rotation", rotation, 4)):
        if t.dim() != 2 or t.shape[0] != n or t.shape[1] != last:
            raise ValueError(f"{name} must be [N,{last}], got {tuple(t.shape)}")
        if not (t.is_cuda and t.dtype == torch.float32):
            raise ValueError(f"{name} must be a CUDA float32 tensor")
    intrs = _c(intrs.reshape(V, 4))
    extrs = _c(extrs.reshape(V, 3, 4))
    return _PreprocessViews.apply(_c(position), _c(scaling), _c16(rotation), intrs, extrs,
                                  [tuple(map(int, s)) for s in sizes], float(nearest), float(extent))


# ---------------------------------------------------------------------------
# camera pose of a differentiable camera
# ---------------------------------------------------------------------------
class _CameraPose(torch.autograd.Function):
    @staticmethod
    def forward(ctx, quat, translation):
        dev = quat.device
        E = torch.empty(4, 4, dtype=torch.float32, device=dev)
        centre = torch.empty(3, dtype=torch.float32, device=dev)
        with _timed("camera_pose_fwd", dev, 1):
            call("pgb_camera_pose_forward", _ptr(quat), _ptr(translation), _ptr(E), _ptr(centre),
                 _stream(dev))
        ctx.save_for_backward(quat, translation)
        return E, centre

    @staticmethod
    def backward(ctx, dE, dcentre):
        quat, translation = ctx.saved_tensors
        dev = quat.device
        dq = torch.empty(4, dtype=torch.float32, device=dev)
        dt = torch.empty(3, dtype=torch.float32, device=dev)
        dE = None if dE is None else dE.contiguous()
        dcentre = None if dcentre is None else dcentre.contiguous()
        with _timed("camera_pose_bwd", dev, 1):
            call("pgb_camera_pose_backward", _ptr(quat), _ptr(translation), _ptr(dE),
                 _ptr(dcentre), _ptr(dq), _ptr(dt), _stream(dev))
        return dq, dt


def camera_pose(quat, translation):
    """(world->camera [4,4], camera centre [3]) of a camera stored as a wxyz
    quaternion [4] (normalised here) and a translation [3]: the rotation of
    ``pointrix/utils/pose.py:40-84`` applied to q / |q|, E = [R t; 0 0 0 1],
    centre = -R^T t; one kernel each way (the torch composition is a dozen
    kernels forward and as many backward)."""
    for name, t, k in (("quat", quat, 4), ("translation", translation, 3)):
        if t.numel() != k or not (t.is_cuda and t.dtype == torch.float32):
            raise ValueError(f"{name} must be a CUDA float32 tensor of {k} values")
    return _CameraPose.apply(quat.reshape(4).contiguous(), translation.reshape(3).contiguous())
