"""Seeded synthetic scenes and cameras for the five benchmark workloads.

No dataset is read: every workload is generated from a ``torch.Generator`` with
the shapes and distributions the workload definitions name.  Parameters are
returned in the storage layout Pointrix's ``GaussianPointCloud`` keeps and in
the activated form ``MsplatRender.render_iter`` receives
(``pointrix/model/point_cloud/gaussian_points.py:70-86``):

* ``position`` [N,3], ``scaling`` = exp(log-scale) [N,3],
* ``rotation`` unit wxyz quaternion [N,4], ``opacity`` = sigmoid(logit) [N,1],
* ``shs`` [N,K,3] (DC first, ``get_shs`` layout).

Cameras are OpenCV-style (x right, y down, z forward) world->camera matrices
looking at the origin, with intrinsics ``[fx, fy, cx, cy]``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import torch

SH_C0 = 0.5 / math.sqrt(math.pi)


@dataclass
class Camera:
    W: int
    H: int
    intr: torch.Tensor          # [1,4] fx, fy, cx, cy
    extr: torch.Tensor          # [4,4] world -> camera
    center: torch.Tensor        # [3]

    def to(self, device):
        return Camera(self.W, self.H, self.intr.to(device), self.extr.to(device), self.center.to(device))


@dataclass
class Scene:
    position: torch.Tensor
    log_scale: torch.Tensor
    quat_raw: torch.Tensor
    opacity_logit: torch.Tensor
    shs: torch.Tensor
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.position.shape[0]

    def to(self, device):
        return Scene(*(t.to(device) for t in (self.position, self.log_scale, self.quat_raw,
                                               self.opacity_logit, self.shs)), dict(self.extra))

    def activated(self):
        """(position, scaling, rotation, opacity, shs) as the renderer receives them."""
        q = self.quat_raw / self.quat_raw.norm(dim=1, keepdim=True)
        return (self.position, torch.exp(self.log_scale), q,
                torch.sigmoid(self.opacity_logit), self.shs)

    def leaves(self):
        """Fresh leaf copies with requires_grad, for a training step."""
        return Scene(*(t.detach().clone().requires_grad_(True) for t in
                       (self.position, self.log_scale, self.quat_raw, self.opacity_logit, self.shs)),
                     dict(self.extra))


def look_at(center: torch.Tensor) -> torch.Tensor:
    """World->camera [4,4] for a camera at ``center`` looking at the origin."""
    c = center.double()
    z = -c / c.norm()
    up = torch.tensor([0.0, 0.0, 1.0], dtype=torch.float64)
    if abs(float(z @ up)) > 0.99:
        up = torch.tensor([0.0, 1.0, 0.0], dtype=torch.float64)
    x = torch.linalg.cross(z, up)
    x = x / x.norm()
    y = torch.linalg.cross(z, x)
    R = torch.stack([x, y, z])
    E = torch.eye(4, dtype=torch.float64)
    E[:3, :3] = R
    E[:3, 3] = -R @ c
    return E.float()


def random_direction(g: torch.Generator) -> torch.Tensor:
    d = torch.randn(3, generator=g, dtype=torch.float64)
    return d / d.norm()


def make_camera(g: torch.Generator, W: int, H: int, f: float, radius: float) -> Camera:
    center = (random_direction(g) * radius).float()
    intr = torch.tensor([[f, f, W / 2.0, H / 2.0]], dtype=torch.float32)
    return Camera(W, H, intr, look_at(center), center)


def _quats(g, n):
    return torch.randn(n, 4, generator=g)


def scene_small(seed: int = 0, n: int = 16384) -> tuple[Scene, Camera]:
    """16,384 Gaussians, SH degree 0 with RGB ~U[0,1]; means ~U[-1,1]^3,
    log-scales ~N(-4.5, 0.5), quaternions normalised N(0,1)^4, opacity
    sigmoid(N(0,1)); one 256x256 camera, f=256, at radius 4."""
    g = torch.Generator().manual_seed(seed)
    pos = torch.rand(n, 3, generator=g) * 2 - 1
    logs = torch.randn(n, 3, generator=g) * 0.5 - 4.5
    q = _quats(g, n)
    op = torch.randn(n, 1, generator=g)
    rgb = torch.rand(n, 3, generator=g)
    shs = ((rgb - 0.5) / SH_C0)[:, None, :]
    cam = make_camera(g, 256, 256, 256.0, 4.0)
    return Scene(pos, logs, q, op, shs), cam


def scene_sh3(seed: int, n: int) -> Scene:
    """SH degree 3 scene: DC ~N(0,0.3), higher bands ~N(0,0.05); means
    ~N(0,1.5^2)^3, log-scales ~N(-4,0.7), random unit quaternions, opacity
    sigmoid(N(0,1.5))."""
    g = torch.Generator().manual_seed(seed)
    pos = torch.randn(n, 3, generator=g) * 1.5
    logs = torch.randn(n, 3, generator=g) * 0.7 - 4.0
    q = _quats(g, n)
    op = torch.randn(n, 1, generator=g) * 1.5
    shs = torch.randn(n, 16, 3, generator=g) * 0.05
    shs[:, 0, :] = torch.randn(n, 3, generator=g) * 0.3
    return Scene(pos, logs, q, op, shs)


def scene_train_view(seed: int = 1, n: int = 1_000_000) -> tuple[Scene, Camera]:
    """Single-view training step: 1M Gaussians SH3, one 1600x1060 camera,
    focal 1150 px, at radius 5."""
    s = scene_sh3(seed, n)
    g = torch.Generator().manual_seed(seed + 1000)
    return s, make_camera(g, 1600, 1060, 1150.0, 5.0)


MULTIVIEW_RES = ((640, 480), (1280, 720), (1600, 1060), (1920, 1080))


def cameras_multiview(seed: int = 2, views: int = 16, radius: float = 5.0, f_scale: float = 0.72):
    """``views`` cameras on a radius-5 sphere, resolutions uniform over
    640x480, 1280x720, 1600x1060 and 1920x1080 (focal = f_scale * W)."""
    g = torch.Generator().manual_seed(seed)
    cams = []
    for _ in range(views):
        W, H = MULTIVIEW_RES[int(torch.randint(0, len(MULTIVIEW_RES), (1,), generator=g))]
        cams.append(make_camera(g, W, H, f_scale * W, radius))
    return cams


def _quat_pair_to_rot() -> torch.Tensor:
    """[16, 9]: row-major rotation entries of a unit wxyz quaternion as linear
    combinations of the products q_a q_b (index 4a + b), in the homogeneous
    form of ``pointrix/utils/pose.py:40-84``."""
    W_, X, Y, Z = 0, 1, 2, 3
    terms = [
        {(W_, W_): 1, (X, X): 1, (Y, Y): -1, (Z, Z): -1},   # R00
        {(X, Y): 2, (W_, Z): -2},                            # R01
        {(X, Z): 2, (W_, Y): 2},                             # R02
        {(X, Y): 2, (W_, Z): 2},                             # R10
        {(W_, W_): 1, (X, X): -1, (Y, Y): 1, (Z, Z): -1},   # R11
        {(Y, Z): 2, (W_, X): -2},                            # R12
        {(X, Z): 2, (W_, Y): -2},                            # R20
        {(Y, Z): 2, (W_, X): 2},                             # R21
        {(W_, W_): 1, (X, X): -1, (Y, Y): -1, (Z, Z): 1},   # R22
    ]
    A = torch.zeros(16, 9)
    for j, t in enumerate(terms):
        for (a, b), c in t.items():
            A[4 * a + b, j] = c
    return A


_QQ_TO_R = _quat_pair_to_rot()
_QQ_TO_R_ON: dict = {}


def rotation_from_unit_quat(q: torch.Tensor) -> torch.Tensor:
    """Rotation matrices [..., 3, 3] of unit wxyz quaternions [..., 4]: one
    outer product and one small matmul (few kernels, also in backward)."""
    key = (q.device, q.dtype)
    A = _QQ_TO_R_ON.get(key)
    if A is None:
        A = _QQ_TO_R_ON[key] = _QQ_TO_R.to(q.device, q.dtype)
    qq = (q[..., :, None] * q[..., None, :]).reshape(*q.shape[:-1], 16)
    return (qq @ A).reshape(*q.shape[:-1], 3, 3)


def normals_from_scene(scaling: torch.Tensor, rotation: torch.Tensor) -> torch.Tensor:
    """Shortest-axis normal, rotated into world space (the normal feature of
    ``examples/supervise/model.py:50-62``: column argmin(scale) of R(q))."""
    idx = torch.argmin(scaling.detach(), dim=-1)
    R = rotation_from_unit_quat(rotation)                     # [N, 3, 3]
    n = R.gather(2, idx[:, None, None].expand(-1, 3, 1))[..., 0]
    return torch.nn.functional.normalize(n, dim=-1)
