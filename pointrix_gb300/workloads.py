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


def normals_from_scene(scaling: torch.Tensor, rotation: torch.Tensor) -> torch.Tensor:
    """Shortest-axis normal, rotated into world space (the normal feature of
    ``examples/supervise/model.py:50-62``)."""
    idx = torch.argmin(scaling.detach(), dim=-1)
    w, x, y, z = rotation.unbind(-1)
    cols = torch.stack([
        torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y + w * z), 2 * (x * z - w * y)], -1),
        torch.stack([2 * (x * y - w * z), 1 - 2 * (x * x + z * z), 2 * (y * z + w * x)], -1),
        torch.stack([2 * (x * z + w * y), 2 * (y * z - w * x), 1 - 2 * (x * x + y * y)], -1),
    ], 1)                                              # [N, 3 (column), 3]
    n = cols.gather(1, idx[:, None, None].expand(-1, 1, 3))[:, 0]
    return torch.nn.functional.normalize(n, dim=-1)
