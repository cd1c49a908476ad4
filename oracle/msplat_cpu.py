"""CPU oracle for the msplat operator path behind Pointrix's ``MsplatRender``.

TEST INFRASTRUCTURE ONLY.  The shipped package never imports this module; the
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use
it as the checker.

Parity unpinned.  The operator backend the reference calls is the git
submodule ``pointrix-project/msplat`` (``.gitmodules:1-3``); its directory is
empty in the reference tree, its pinned commit is unknown, and the reference
ships no tests, golden vectors or fixtures for it.  This module therefore
restates the published algorithms -- EWA splatting (Zwicker et al. 2001), 3D
Gaussian Splatting (Kerbl et al. 2023) and real spherical harmonics -- under
the contracts fixed by the reference's call sites:

* ``pointrix/model/renderer/msplat.py:94-158``   (``MsplatRender.render_iter``)
* ``pointrix/model/renderer/utils/renderer_utils.py:30-71`` (feature packing)
* ``pointrix/model/point_cloud/gaussian_points.py:70-86`` (activations)
* ``pointrix/utils/pose.py:40-84``               (wxyz quaternions)
* ``pointrix/controller/gs.py:260-284``          (``ndc.grad`` is the raw
  pixel-space uv gradient: the controller rescales it by W/2, H/2 itself)

Conventions the call sites leave open are fixed here (module constants and
docstrings below) and mirrored by the CUDA kernels:

* pixel (i, j) has its centre at the integer coordinate (i, j);
* ``project_point`` culls ``depth <= nearest`` (default 0.2) and centres whose
  normalised offset ``|2u/W - 1|`` or ``|2v/H - 1|`` is not below ``extent``
  (default 1.3); culled points get uv = 0 and depth = 0;
* ``ewa_project`` clamps x/z and y/z to 1.3 tan(fov/2), adds a 0.3 px^2
  low-pass dilation to the 2D covariance diagonal, culls det <= 0, takes the
  radius ceil(3 sqrt(lambda_max)) with lambda_max = mid + sqrt(max(0.1,
  mid^2 - det)), capped at 2^20 px, and the 16x16 tile rectangle
  [trunc(clamp((u - r)/16, 0, gx)), trunc(clamp((u + r + 15)/16, 0, gx))),
  likewise for v; a Gaussian touching no tile gets radius 0;
* ``sort_gaussian`` emits one entry per (Gaussian, tile) in Gaussian-id order
  and row-major tile order, with the key (tile_id << 32) | float_bits(depth),
  and sorts stably; ``tile_range[t] = [start, end)``, ``[0, 0]`` for an empty
  tile;
* ``alpha_blending``: alpha = min(0.99, o exp(power)), power = -(a dx^2 +
  c dy^2)/2 - b dx dy with d = uv - pixel; a Gaussian is skipped when power > 0
  or alpha < 1/255; a pixel stops before the Gaussian that would take its
  transmittance below 1e-4; ``out = sum f alpha T + T_final bg``;
* ``compute_sh`` returns the raw real-SH sum (no +0.5, no clamp), degree
  ``sqrt(K) - 1``, with the basis and signs of the 3DGS renderer.

Every function is written elementwise with a fixed operation order.  Run in
float32 it reproduces the CUDA kernels' integer outputs (radius, tile counts,
sorted ids, tile ranges) bit for bit, because the kernels that produce them are
compiled without FMA contraction and use the same order; run in float64 it is
the precision reference for float outputs and, through torch autograd, for
every gradient.
"""
from __future__ import annotations

import math

import numpy as np
import torch

TILE = 16
NEAREST_DEFAULT = 0.2
EXTENT_DEFAULT = 1.3
FOV_CLAMP = 1.3
DILATION = 0.3
EIG_FLOOR = 0.1
RADIUS_CAP = 1048576.0
ALPHA_MAX = 0.99
ALPHA_MIN = 1.0 / 255.0
T_MIN = 1e-4
# splats per step of the oracle's blend loop over a tile's list
BLEND_CHUNK = 256

# Real spherical-harmonic normalisation constants, from their closed forms.
SH_C0 = 0.5 / math.sqrt(math.pi)
SH_C1 = math.sqrt(3.0) / (2.0 * math.sqrt(math.pi))
SH_C2 = (
    0.5 * math.sqrt(15.0 / math.pi),
    -0.5 * math.sqrt(15.0 / math.pi),
    0.25 * math.sqrt(5.0 / math.pi),
    -0.5 * math.sqrt(15.0 / math.pi),
    0.25 * math.sqrt(15.0 / math.pi),
)
SH_C3 = (
    -0.25 * math.sqrt(35.0 / (2.0 * math.pi)),
    0.5 * math.sqrt(105.0 / math.pi),
    -0.25 * math.sqrt(21.0 / (2.0 * math.pi)),
    0.25 * math.sqrt(7.0 / math.pi),
    -0.25 * math.sqrt(21.0 / (2.0 * math.pi)),
    0.25 * math.sqrt(105.0 / math.pi),
    -0.25 * math.sqrt(35.0 / (2.0 * math.pi)),
)


def tile_grid(W: int, H: int) -> tuple[int, int]:
    return (W + TILE - 1) // TILE, (H + TILE - 1) // TILE


def _s(v, like: torch.Tensor) -> torch.Tensor:
    """A scalar as a 0-dim tensor of the working dtype, so that every
    arithmetic step below is carried out (and rounded) in that dtype."""
    return torch.tensor(v, dtype=like.dtype)


def _cam_point(xyz: torch.Tensor, extr: torch.Tensor):
    """p = R x + t, summed left to right: ((R0 x + R1 y) + R2 z) + t."""
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    e = extr
    px = e[0, 0] * x + e[0, 1] * y + e[0, 2] * z + e[0, 3]
    py = e[1, 0] * x + e[1, 1] * y + e[1, 2] * z + e[1, 3]
    pz = e[2, 0] * x + e[2, 1] * y + e[2, 2] * z + e[2, 3]
    return px, py, pz


# ---------------------------------------------------------------------------
# compute_sh  (call site pointrix/model/renderer/msplat.py:104)
# ---------------------------------------------------------------------------
def sh_basis(dirs: torch.Tensor, K: int) -> torch.Tensor:
    """Real SH basis Y_k(d) for k < K, d a unit direction [N,3] -> [N,K]."""
    x, y, z = dirs[:, 0], dirs[:, 1], dirs[:, 2]
    ys = [torch.full_like(x, SH_C0)]
    if K > 1:
        ys += [-SH_C1 * y, SH_C1 * z, -SH_C1 * x]
    if K > 4:
        xx, yy, zz = x * x, y * y, z * z
        ys += [
            SH_C2[0] * (x * y),
            SH_C2[1] * (y * z),
            SH_C2[2] * (2.0 * zz - xx - yy),
            SH_C2[3] * (x * z),
            SH_C2[4] * (xx - yy),
        ]
    if K > 9:
        ys += [
            SH_C3[0] * y * (3.0 * xx - yy),
            SH_C3[1] * (x * y) * z,
            SH_C3[2] * y * (4.0 * zz - xx - yy),
            SH_C3[3] * z * (2.0 * zz - 3.0 * xx - 3.0 * yy),
            SH_C3[4] * x * (4.0 * zz - xx - yy),
            SH_C3[5] * z * (xx - yy),
            SH_C3[6] * x * (xx - 3.0 * yy),
        ]
    return torch.stack(ys, dim=1)


def compute_sh(sh: torch.Tensor, dirs: torch.Tensor) -> torch.Tensor:
    """sh [N,3,K] (K in 1,4,9,16), dirs [N,3] -> raw SH colour [N,3]."""
    K = sh.shape[-1]
    if K not in (1, 4, 9, 16):
        raise ValueError(f"compute_sh: K={K} is not (deg+1)^2 for deg<=3")
    basis = sh_basis(dirs, K)                      # [N,K]
    return (sh * basis[:, None, :]).sum(-1)


# ---------------------------------------------------------------------------
# project_point  (call site pointrix/model/renderer/msplat.py:109-113)
# ---------------------------------------------------------------------------
def project_point(xyz, intr, extr, W, H, nearest=NEAREST_DEFAULT, extent=EXTENT_DEFAULT):
    """xyz [N,3], intr [4] or [1,4] = (fx, fy, cx, cy), extr [3,4] world->camera.

    Returns uv [N,2] and depth [N,1]; culled points have uv = 0, depth = 0.
    """
    f = intr.reshape(4)
    fx, fy, cx, cy = f[0], f[1], f[2], f[3]
    px, py, pz = _cam_point(xyz, extr)
    near_ok = pz > _s(nearest, pz)
    pzs = torch.where(near_ok, pz, torch.ones_like(pz))
    u = fx * px / pzs + cx
    v = fy * py / pzs + cy
    hw = _s(0.5 * W, pz)
    hh = _s(0.5 * H, pz)
    ext = _s(extent, pz)
    vis = near_ok & ((u - hw).abs() < ext * hw) & ((v - hh).abs() < ext * hh)
    zero = torch.zeros_like(u)
    uv = torch.stack([torch.where(vis, u, zero), torch.where(vis, v, zero)], dim=1)
    depth = torch.where(vis, pz, zero)[:, None]
    return uv, depth


# ---------------------------------------------------------------------------
# compute_cov3d  (call site pointrix/model/renderer/msplat.py:118)
# ---------------------------------------------------------------------------
def quat_to_rot(q: torch.Tensor):
    """Rotation matrix entries of a unit wxyz quaternion (no normalisation)."""
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    xx, yy, zz = x * x, y * y, z * z
    xy, xz, yz = x * y, x * z, y * z
    wx, wy, wz = w * x, w * y, w * z
    one = _s(1.0, q)
    return (
        (one - 2.0 * (yy + zz), 2.0 * (xy - wz), 2.0 * (xz + wy)),
        (2.0 * (xy + wz), one - 2.0 * (xx + zz), 2.0 * (yz - wx)),
        (2.0 * (xz - wy), 2.0 * (yz + wx), one - 2.0 * (xx + yy)),
    )


def compute_cov3d(scales, uquats, visible):
    """Sigma = (R S)(R S)^T, upper triangle (xx, xy, xz, yy, yz, zz) [N,6];
    rows where ``visible`` is false are zero."""
    R = quat_to_rot(uquats)
    s = (scales[:, 0], scales[:, 1], scales[:, 2])
    M = [[R[i][j] * s[j] for j in range(3)] for i in range(3)]

    def sig(i, j):
        return M[i][0] * M[j][0] + M[i][1] * M[j][1] + M[i][2] * M[j][2]

    cov = torch.stack([sig(0, 0), sig(0, 1), sig(0, 2), sig(1, 1), sig(1, 2), sig(2, 2)], 1)
    vis = visible.reshape(-1).bool()
    return torch.where(vis[:, None], cov, torch.zeros_like(cov))


# ---------------------------------------------------------------------------
# ewa_project  (call site pointrix/model/renderer/msplat.py:121-130)
# ---------------------------------------------------------------------------
def tile_rect(u, v, r, W, H):
    """Tile rectangle [xmin, xmax) x [ymin, ymax) of a disc of radius r at
    (u, v); all float steps in the dtype of ``u``."""
    gx, gy = tile_grid(W, H)
    t = _s(float(TILE), u)
    c = _s(float(TILE - 1), u)
    zero = _s(0.0, u)

    def clampi(val, hi):
        return torch.minimum(torch.maximum(val, zero), _s(float(hi), u)).to(torch.int32)

    xmin = clampi((u - r) / t, gx)
    xmax = clampi((u + r + c) / t, gx)
    ymin = clampi((v - r) / t, gy)
    ymax = clampi((v + r + c) / t, gy)
    return xmin, xmax, ymin, ymax


def ewa_project(xyz, cov3d, intr, extr, uv, W, H, visible):
    """EWA projection of the 3D covariance to an image-space conic.

    Returns conic [N,3] = inverse 2D covariance (a, b, c), radius [N] int32
    and tiles_touched [N] int32; culled Gaussians get zeros.
    """
    dt = xyz.dtype
    f = intr.reshape(4)
    fx, fy = f[0], f[1]
    px, py, pz = _cam_point(xyz, extr)
    vis = visible.reshape(-1).bool()
    pzs = torch.where(vis, pz, torch.ones_like(pz))
    limx = _s(FOV_CLAMP, pz) * (_s(0.5 * W, pz) / fx)
    limy = _s(FOV_CLAMP, pz) * (_s(0.5 * H, pz) / fy)
    tx = torch.minimum(torch.maximum(px / pzs, -limx), limx) * pzs
    ty = torch.minimum(torch.maximum(py / pzs, -limy), limy) * pzs
    pz2 = pzs * pzs
    J00 = fx / pzs
    J02 = -(fx * tx) / pz2
    J11 = fy / pzs
    J12 = -(fy * ty) / pz2
    e = extr
    T0 = (J00 * e[0, 0] + J02 * e[2, 0], J00 * e[0, 1] + J02 * e[2, 1], J00 * e[0, 2] + J02 * e[2, 2])
    T1 = (J11 * e[1, 0] + J12 * e[2, 0], J11 * e[1, 1] + J12 * e[2, 1], J11 * e[1, 2] + J12 * e[2, 2])
    s00, s01, s02, s11, s12, s22 = (cov3d[:, i] for i in range(6))
    V0 = (s00 * T0[0] + s01 * T0[1] + s02 * T0[2],
          s01 * T0[0] + s11 * T0[1] + s12 * T0[2],
          s02 * T0[0] + s12 * T0[1] + s22 * T0[2])
    V1 = (s00 * T1[0] + s01 * T1[1] + s02 * T1[2],
          s01 * T1[0] + s11 * T1[1] + s12 * T1[2],
          s02 * T1[0] + s12 * T1[1] + s22 * T1[2])
    dil = _s(DILATION, pz)
    a = T0[0] * V0[0] + T0[1] * V0[1] + T0[2] * V0[2] + dil
    b = T1[0] * V0[0] + T1[1] * V0[1] + T1[2] * V0[2]
    c = T1[0] * V1[0] + T1[1] * V1[1] + T1[2] * V1[2] + dil
    det = a * c - b * b
    ok = vis & (det > 0)
    dets = torch.where(ok, det, torch.ones_like(det))
    inv = _s(1.0, pz) / dets
    conic = torch.stack([c * inv, -b * inv, a * inv], dim=1)

    with torch.no_grad():
        a_, c_, det_ = a.detach(), c.detach(), det.detach()
        mid = _s(0.5, pz) * (a_ + c_)
        disc = torch.maximum(_s(EIG_FLOOR, pz), mid * mid - det_)
        lam = mid + torch.sqrt(disc)
        rf = torch.ceil(_s(3.0, pz) * torch.sqrt(lam))
        rf = torch.minimum(rf, _s(RADIUS_CAP, pz))
        rf = torch.where(ok, rf, torch.zeros_like(rf))
        u = uv[:, 0].detach().to(dt)
        v = uv[:, 1].detach().to(dt)
        xmin, xmax, ymin, ymax = tile_rect(u, v, rf, W, H)
        tiles = (xmax - xmin) * (ymax - ymin)
        ok = ok & (tiles > 0)
        radius = torch.where(ok, rf.to(torch.int32), torch.zeros_like(tiles))
        tiles = torch.where(ok, tiles, torch.zeros_like(tiles))
    conic = torch.where(ok[:, None], conic, torch.zeros_like(conic))
    return conic, radius, tiles


# ---------------------------------------------------------------------------
# sort_gaussian  (call site pointrix/model/renderer/msplat.py:133-135)
# ---------------------------------------------------------------------------
def duplicate_with_keys(uv, depth, W, H, radius, tiles_touched):
    """One (key, gaussian id) pair per touched tile, in Gaussian-id order and
    row-major tile order; key = (tile_id << 32) | float_bits(depth)."""
    gx, gy = tile_grid(W, H)
    # rectangles in the dtype the radius/tiles were derived in (float32 for
    # the bit-exact rendition, float64 for the float64 one)
    fdt = np.float64 if uv.dtype == torch.float64 else np.float32
    uv32 = np.ascontiguousarray(uv.detach().cpu().numpy().astype(fdt, copy=False))
    d32 = np.ascontiguousarray(depth.detach().cpu().numpy().reshape(-1).astype(np.float32, copy=False))
    rad = radius.detach().cpu().numpy().reshape(-1).astype(np.int64)
    tt = tiles_touched.detach().cpu().numpy().reshape(-1).astype(np.int64)
    gid = np.nonzero(rad > 0)[0]
    u = uv32[gid, 0]
    v = uv32[gid, 1]
    r = rad[gid].astype(fdt)
    t16, t15 = fdt(TILE), fdt(TILE - 1)
    z = fdt(0)
    xmin = np.clip((u - r) / t16, z, fdt(gx)).astype(np.int64)
    xmax = np.clip((u + r + t15) / t16, z, fdt(gx)).astype(np.int64)
    ymin = np.clip((v - r) / t16, z, fdt(gy)).astype(np.int64)
    ymax = np.clip((v + r + t15) / t16, z, fdt(gy)).astype(np.int64)
    wrect = xmax - xmin
    cnt = wrect * (ymax - ymin)
    if not np.array_equal(cnt, tt[gid]):
        raise ValueError("sort_gaussian: tiles_touched disagrees with the uv/radius rectangles")
    K = int(cnt.sum())
    rep = np.repeat(np.arange(len(gid)), cnt)
    starts = np.concatenate([[0], np.cumsum(cnt)[:-1]]).astype(np.int64)
    k = np.arange(K, dtype=np.int64) - starts[rep]
    w = np.maximum(wrect[rep], 1)
    tx = xmin[rep] + k % w
    ty = ymin[rep] + k // w
    tile = (ty * gx + tx).astype(np.uint64)
    dbits = d32.view(np.uint32)[gid[rep]].astype(np.uint64)
    keys = (tile << np.uint64(32)) | dbits
    vals = gid[rep].astype(np.int64)
    return keys, vals


def sort_gaussian(uv, depth, W, H, radius, tiles_touched):
    """Returns gaussian_ids_sorted [K] int32 and tile_range [T,2] int32."""
    gx, gy = tile_grid(W, H)
    T = gx * gy
    keys, vals = duplicate_with_keys(uv, depth, W, H, radius, tiles_touched)
    order = np.argsort(keys, kind="stable")
    ids = vals[order].astype(np.int32)
    tile_of = (keys[order] >> np.uint64(32)).astype(np.int64)
    counts = np.bincount(tile_of, minlength=T)
    ends = np.cumsum(counts)
    starts = ends - counts
    rng = np.stack([starts, ends], 1).astype(np.int32)
    rng[counts == 0] = 0
    return torch.from_numpy(ids), torch.from_numpy(rng)


# ---------------------------------------------------------------------------
# alpha_blending  (call site pointrix/model/renderer/msplat.py:148-151)
# ---------------------------------------------------------------------------
def _tile_pixels(t, W, H):
    """Pixel coordinates (x, y) and flat indices of tile ``t``, row-major."""
    gx, _ = tile_grid(W, H)
    ly, lx = torch.meshgrid(torch.arange(TILE), torch.arange(TILE), indexing="ij")
    pxi = (t % gx) * TILE + lx.reshape(-1)
    pyi = (t // gx) * TILE + ly.reshape(-1)
    inside = (pxi < W) & (pyi < H)
    pxi, pyi = pxi[inside], pyi[inside]
    return pxi, pyi, pyi * W + pxi


def blend_tile(uv, conic, opacity, feature, g, pxi, pyi):
    """One tile's compositing: the pixels (pxi, pyi) over the depth-sorted
    splats ``g`` (indices into the per-Gaussian inputs).  Returns
    (colour [P,C] before the background, final T [P], index of the last
    contributor in ``g`` [P], -1 for none); differentiable in the inputs.

    The list is walked in chunks of BLEND_CHUNK, the transmittance carried
    across chunks; the walk stops once every pixel has stopped (nothing later
    in the list can contribute)."""
    dt = feature.dtype
    C = feature.shape[1]
    amin, amax, tmin = _s(ALPHA_MIN, feature), _s(ALPHA_MAX, feature), _s(T_MIN, feature)
    half = _s(0.5, feature)
    pxf = pxi.to(dt)[:, None]
    pyf = pyi.to(dt)[:, None]
    P = pxi.numel()
    Tprev = torch.ones(P, dtype=dt)
    col = torch.zeros(P, C, dtype=dt)
    last = torch.full((P,), -1, dtype=torch.long)
    Tf = torch.ones(P, dtype=dt)
    n = g.numel()
    for c0 in range(0, n, BLEND_CHUNK):
        gc = g[c0:c0 + BLEND_CHUNK]
        dx = uv[gc, 0].to(dt)[None, :] - pxf
        dy = uv[gc, 1].to(dt)[None, :] - pyf
        ca, cb, cc = (conic[gc, i].to(dt)[None, :] for i in range(3))
        power = -half * (ca * dx * dx + cc * dy * dy) - cb * dx * dy
        o = opacity.reshape(-1)[gc].to(dt)[None, :]
        alpha = torch.minimum(amax, o * torch.exp(power))
        valid = (power <= 0) & (alpha >= amin)
        a_v = torch.where(valid, alpha, torch.zeros_like(alpha))
        Tinc = Tprev[:, None] * torch.cumprod(1.0 - a_v, dim=1)
        Texc = torch.cat([Tprev[:, None], Tinc[:, :-1]], dim=1)
        incl = valid & (Tinc.detach() >= tmin)
        w = torch.where(incl, a_v * Texc, torch.zeros_like(a_v))
        col = col + w @ feature[gc].to(dt)
        idx = torch.arange(c0, c0 + gc.numel())[None, :].expand_as(incl)
        lastc = torch.where(incl, idx, torch.full_like(idx, -1)).max(dim=1).values
        has = lastc >= 0
        Tf = torch.where(has, Tinc.gather(1, (lastc - c0).clamp(min=0)[:, None])[:, 0], Tf)
        last = torch.where(has, lastc, last)
        Tprev = Tinc[:, -1]
        if bool((Tprev.detach() < tmin).all()):
            break
    return col, Tf, last


def alpha_blending(uv, conic, opacity, feature, ids, tile_range, bg, W, H,
                   tiles=None, return_state=False):
    """Front-to-back compositing of ``feature`` [N,C] over 16x16 tiles.

    Returns the image [C,H,W]; with ``return_state`` also the final
    transmittance [H,W] and the per-pixel count of list entries up to and
    including the last contributor [H,W].  ``tiles`` restricts the work to a
    subset of tile ids (the rest of the image is left at ``bg``), which the
    tests use to check sampled tiles of a full-size view.

    Differentiable (torch autograd) in uv, conic, opacity and feature.
    """
    dt = feature.dtype
    C = feature.shape[1]
    gx, gy = tile_grid(W, H)
    ids = ids.long()
    rng = tile_range.long()
    out = torch.full((C, H * W), float(bg), dtype=dt)
    finalT = torch.ones(H * W, dtype=dt)
    ncon = torch.zeros(H * W, dtype=torch.int32)
    pieces = []
    for t in (range(gx * gy) if tiles is None else tiles):
        t = int(t)
        s, e = int(rng[t, 0]), int(rng[t, 1])
        if e <= s:
            continue
        pxi, pyi, pix = _tile_pixels(t, W, H)
        col, Tf, last = blend_tile(uv, conic, opacity, feature, ids[s:e], pxi, pyi)
        pieces.append((pix, col + Tf[:, None] * bg, Tf))
        ncon[pix] = (last + 1).to(torch.int32)
    if pieces:
        pix_all = torch.cat([p[0] for p in pieces])
        col_all = torch.cat([p[1] for p in pieces])
        T_all = torch.cat([p[2] for p in pieces])
        out = out.index_copy(1, pix_all, col_all.t())
        finalT = finalT.index_copy(0, pix_all, T_all)
    out = out.reshape(C, H, W)
    if return_state:
        return out, finalT.reshape(H, W), ncon.reshape(H, W)
    return out


def blend_loss_grad(uv, conic, opacity, feature, ids, tile_range, bg, W, H, pixel_loss,
                    workers=1):
    """The blend and the gradient of a per-pixel loss, tile by tile, in
    bounded memory (a full-size view's autograd graph over all tiles would
    not fit): each tile is composited with autograd on copies of its splats'
    inputs, its share of the loss is back-propagated at once and the
    gradients are summed into per-Gaussian buffers.  ``pixel_loss(img [C,P],
    pix [P])`` returns that tile's scalar share (the loss must be a sum over
    pixels).  ``workers`` threads take tiles in turn.  Returns (loss,
    image [C,H,W], d_uv, d_conic, d_opacity, d_feature), all detached."""
    import threading
    from concurrent.futures import ThreadPoolExecutor

    dt = feature.dtype
    C = feature.shape[1]
    gx, gy = tile_grid(W, H)
    ids = ids.long()
    rng = tile_range.long()
    U, Cn, Op, F = (x.detach() for x in (uv, conic, opacity.reshape(-1, 1), feature))
    grads = [torch.zeros_like(x) for x in (U, Cn, Op, F)]
    out = torch.full((C, H * W), float(bg), dtype=dt)
    lock = threading.Lock()
    total = [0.0]

    def one(t):
        s, e = int(rng[t, 0]), int(rng[t, 1])
        pxi, pyi, pix = _tile_pixels(t, W, H)
        if e <= s:
            with torch.no_grad():
                img = torch.full((C, pix.numel()), float(bg), dtype=dt)
            loss = pixel_loss(img, pix)
            with lock:
                total[0] += float(loss)
            return
        g = ids[s:e]               # a splat is listed at most once per tile
        leaves = [x[g].clone().requires_grad_(True) for x in (U, Cn, Op, F)]
        col, Tf, _ = blend_tile(*leaves, torch.arange(g.numel()), pxi, pyi)
        img = (col + Tf[:, None] * bg).t()
        loss = pixel_loss(img, pix)
        gl = torch.autograd.grad(loss, leaves, allow_unused=True)
        with lock:
            total[0] += float(loss.detach())
            out[:, pix] = img.detach()
            for buf, gr in zip(grads, gl):
                if gr is not None:
                    buf.index_add_(0, g, gr)

    tiles = range(gx * gy)
    if workers > 1:
        with ThreadPoolExecutor(workers) as ex:
            list(ex.map(one, tiles))
    else:
        for t in tiles:
            one(t)
    return (total[0], out.reshape(C, H, W), grads[0], grads[1], grads[2].reshape(opacity.shape),
            grads[3])


def threshold_pixels(uv, conic, opacity, ids, tile_range, W, H, tiles=None,
                     rel_alpha=1e-5, rel_T=1e-4, rel_clamp=1e-5):
    """Where a float32 and a float64 rendition may legitimately disagree.

    Evaluates, in float64, every (pixel, splat) pair that a pixel considers
    (up to and including the pair at which it stops) and flags the pixel when
    one of its pairs sits within a relative margin of a decision threshold of
    the blend contract (``alpha_blending`` above):

    * the skip test alpha >= 1/255 (``|o e^power - 1/255| <= rel_alpha/255``);
    * the stop test T (1 - alpha) < 1e-4 (``|T (1 - alpha) - 1e-4| <=
      rel_T 1e-4``; T carries the rounding of every earlier factor, hence
      the wider margin);
    * the 0.99 clamp (``|o e^power - 0.99| <= rel_clamp``), where the image is
      continuous but its gradient jumps -- flagged in the second mask only.

    The margins are ten to a hundred times the relative error of a float32
    evaluation of one pair's power, exponential and transmittance.  Returns
    ``(pix [H,W] bool, pix_grad [H,W] bool, gauss [N] bool)``: pixels whose
    value may flip, pixels whose gradient may jump (a superset), and the
    Gaussians any gradient-flagged pixel considers.
    """
    dt = torch.float64
    n = uv.shape[0]
    gx, gy = tile_grid(W, H)
    ids = ids.long()
    rng = tile_range.long()
    pix_flag = torch.zeros(H * W, dtype=torch.bool)
    grad_flag = torch.zeros(H * W, dtype=torch.bool)
    gauss = torch.zeros(n, dtype=torch.bool)
    ly, lx = torch.meshgrid(torch.arange(TILE), torch.arange(TILE), indexing="ij")
    ly, lx = ly.reshape(-1), lx.reshape(-1)
    u64, c64 = uv.detach().to(dt), conic.detach().to(dt)
    o64 = opacity.detach().reshape(-1).to(dt)
    for t in (range(gx * gy) if tiles is None else tiles):
        t = int(t)
        s, e = int(rng[t, 0]), int(rng[t, 1])
        if e <= s:
            continue
        tx, ty = t % gx, t // gx
        pxi, pyi = tx * TILE + lx, ty * TILE + ly
        inside = (pxi < W) & (pyi < H)
        pxi, pyi = pxi[inside], pyi[inside]
        pix = pyi * W + pxi
        g = ids[s:e]
        dx = u64[g, 0][None, :] - pxi.to(dt)[:, None]
        dy = u64[g, 1][None, :] - pyi.to(dt)[:, None]
        ca, cb, cc = (c64[g, i][None, :] for i in range(3))
        power = -0.5 * (ca * dx * dx + cc * dy * dy) - cb * dx * dy
        araw = o64[g][None, :] * torch.exp(power)
        alpha = araw.clamp(max=ALPHA_MAX)
        valid = (power <= 0) & (alpha >= ALPHA_MIN)
        a_v = torch.where(valid, alpha, torch.zeros_like(alpha))
        Tinc = torch.cumprod(1.0 - a_v, dim=1)
        stops = valid & (Tinc < T_MIN)
        # a pair is considered when no earlier pair stopped the pixel
        stopped_before = torch.cumsum(stops.int(), dim=1) - stops.int() > 0
        considered = ~stopped_before
        near_skip = (araw - ALPHA_MIN).abs() <= rel_alpha * ALPHA_MIN
        near_stop = valid & ((Tinc - T_MIN).abs() <= rel_T * T_MIN)
        near_clamp = (araw - ALPHA_MAX).abs() <= rel_clamp * ALPHA_MAX
        f_val = ((near_skip | near_stop) & considered).any(dim=1)
        f_grad = f_val | (near_clamp & valid & considered).any(dim=1)
        pix_flag[pix[f_val]] = True
        grad_flag[pix[f_grad]] = True
        if bool(f_grad.any()):
            touched = considered[f_grad].any(dim=0)
            gauss[g[touched]] = True
    return pix_flag.reshape(H, W), grad_flag.reshape(H, W), gauss


# ---------------------------------------------------------------------------
# The whole per-view path, as MsplatRender.render_iter chains it
# (pointrix/model/renderer/msplat.py:94-151)
# ---------------------------------------------------------------------------
def render_view(xyz, scales, uquats, opacity, sh, extra_features, campos, intr, extr,
                W, H, bg=0.0, nearest=NEAREST_DEFAULT, sh_degree=None, depth_feature=True):
    """Renders one view; returns (image [C,H,W], uv, radius, aux dict).

    ``sh`` is [N,K,3] as ``GaussianPointCloud.get_shs`` stores it; features
    are rgb (+ depth when ``depth_feature``) (+ ``extra_features``).
    """
    d = xyz - campos[None, :]
    d = d / d.norm(dim=1, keepdim=True)
    shc = sh.permute(0, 2, 1)
    if sh_degree is not None:
        mask = torch.zeros_like(shc)
        mask[..., : (sh_degree + 1) ** 2] = 1.0
        shc = shc * mask
    rgb = (compute_sh(shc, d) + 0.5).clamp(min=0.0)
    uv, depth = project_point(xyz, intr, extr, W, H, nearest=nearest)
    vis = depth != 0
    cov = compute_cov3d(scales, uquats, vis)
    conic, radius, tiles = ewa_project(xyz, cov, intr, extr, uv, W, H, vis)
    ids, rng = sort_gaussian(uv, depth, W, H, radius, tiles)
    feats = [rgb]
    if depth_feature:
        feats.append(depth)
    if extra_features is not None:
        feats.append(extra_features)
    f = torch.cat(feats, dim=-1)
    img = alpha_blending(uv, conic, opacity, f, ids, rng, bg, W, H)
    return img, uv, radius, {"ids": ids, "tile_range": rng, "conic": conic, "depth": depth, "tiles": tiles}
