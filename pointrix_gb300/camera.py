"""The cameras of a scene, as Pointrix's ``CameraModel`` plug-in holds them.

``pointrix/model/camera/camera_model.py:19-210`` keeps one wxyz unit
quaternion, one translation and one ``[fx, fy, cx, cy]`` per camera (trainable
when ``enable_training``), built from the dataset's world->camera matrices,
and the training step asks it for the batch's extrinsics, intrinsics and
camera centres (``pointrix/model/base_model.py:73-78``).  :class:`CameraModel`
here has the same configuration, setup and accessors, computed the same way
(``extrinsic_matrices`` = [R(q/|q|) t; 0 0 0 1], ``camera_centers`` = -R^T t,
the rotation of ``pointrix/utils/pose.py:40-84``).  :meth:`CameraModel.poses`
returns both matrices and centres at once, on a CUDA device through the
library's camera-pose kernel (one launch each way per camera instead of the
torch composition's dozen).

The dataset matrices become quaternions by Shepperd's method (S. W.
Shepperd, "Quaternion from rotation matrix", J. Guidance and Control 1(3),
1978): of the four squared-component formulas the one with the largest
value is taken, so the division that yields the other three components is
well conditioned.  A rotation has two quaternions, q and -q; the one with
w >= 0 is returned (the rotation, and so every output above, is the same for
both).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch
from torch import nn


def rotmat_to_unitquat(R) -> np.ndarray:
    """wxyz unit quaternion of a 3x3 rotation matrix (float64)."""
    R = np.asarray(R, dtype=np.float64)
    if R.shape != (3, 3):
        raise ValueError("a rotation matrix is 3x3")
    tr = R[0, 0] + R[1, 1] + R[2, 2]
    pick = int(np.argmax([tr, R[0, 0], R[1, 1], R[2, 2]]))
    if pick == 0:
        w = 0.5 * np.sqrt(1.0 + tr)
        s = 0.25 / w
        q = [w, (R[2, 1] - R[1, 2]) * s, (R[0, 2] - R[2, 0]) * s, (R[1, 0] - R[0, 1]) * s]
    elif pick == 1:
        x = 0.5 * np.sqrt(1.0 + R[0, 0] - R[1, 1] - R[2, 2])
        s = 0.25 / x
        q = [(R[2, 1] - R[1, 2]) * s, x, (R[0, 1] + R[1, 0]) * s, (R[0, 2] + R[2, 0]) * s]
    elif pick == 2:
        y = 0.5 * np.sqrt(1.0 - R[0, 0] + R[1, 1] - R[2, 2])
        s = 0.25 / y
        q = [(R[0, 2] - R[2, 0]) * s, (R[0, 1] + R[1, 0]) * s, y, (R[1, 2] + R[2, 1]) * s]
    else:
        z = 0.5 * np.sqrt(1.0 - R[0, 0] - R[1, 1] + R[2, 2])
        s = 0.25 / z
        q = [(R[1, 0] - R[0, 1]) * s, (R[0, 2] + R[2, 0]) * s, (R[1, 2] + R[2, 1]) * s, z]
    q = np.asarray(q)
    q /= np.linalg.norm(q)
    return -q if q[0] < 0 else q


def unitquat_to_rotmat(q: torch.Tensor) -> torch.Tensor:
    """[..., 3, 3] rotation of wxyz unit quaternions [..., 4], entry by entry
    as ``pointrix/utils/pose.py:40-84`` forms it."""
    w, x, y, z = q.unbind(-1)
    x2, y2, z2, w2 = x * x, y * y, z * z, w * w
    xy, zw, xz, yw, yz, xw = x * y, z * w, x * z, y * w, y * z, x * w
    rows = [
        [x2 - y2 - z2 + w2, 2 * (xy - zw), 2 * (xz + yw)],
        [2 * (xy + zw), -x2 + y2 - z2 + w2, 2 * (yz - xw)],
        [2 * (xz - yw), 2 * (yz + xw), -x2 - y2 + z2 + w2],
    ]
    return torch.stack([torch.stack(r, -1) for r in rows], -2)


@dataclass
class CameraPrior:
    """One dataset camera: world->camera [4,4], ``[fx, fy, cx, cy]`` and the
    image size (the fields ``CameraModel.setup`` reads from Pointrix's
    ``CameraPrior``)."""
    extrinsic_matrix: np.ndarray
    intrinsic_params: np.ndarray
    image_width: int
    image_height: int


class CameraModel:
    """Pointrix's ``CameraModel`` (``camera_model.py:19-210``): the cameras
    of one split of a dataset, trainable when ``enable_training``."""

    @dataclass
    class Config:
        name: str = "CameraModel"
        enable_training: bool = False
        scene_scale: float = 1.0

    def __init__(self, cfg: "CameraModel.Config | dict | None" = None):
        self.cfg = cfg if isinstance(cfg, CameraModel.Config) else CameraModel.Config(**(cfg or {}))

    def setup(self, camerasprior, device="cuda") -> None:
        """One quaternion, translation and intrinsics vector per camera, as
        float32 tensors on ``device`` (``nn.Parameter`` leaves there when
        trainable); the image size is the last camera's
        (``camera_model.py:38-69``)."""
        self.qrots, self.tvecs, self.intrs = [], [], []
        self.enable_training = self.cfg.enable_training
        dev = torch.device(device)
        for prior in camerasprior:
            E = np.asarray(prior.extrinsic_matrix, dtype=np.float64)
            if E.shape not in ((4, 4), (3, 4)):
                raise ValueError("extrinsic_matrix must be 4x4 or 3x4")
            intr = np.asarray(prior.intrinsic_params, dtype=np.float64).reshape(-1)
            if intr.shape != (4,):
                raise ValueError("intrinsic_params must hold [fx, fy, cx, cy]")
            self.width, self.height = prior.image_width, prior.image_height
            for store, value in ((self.qrots, rotmat_to_unitquat(E[:3, :3])),
                                 (self.tvecs, E[:3, 3]), (self.intrs, intr)):
                t = torch.tensor(value, dtype=torch.float32, device=dev)
                store.append(nn.Parameter(t) if self.enable_training else t)

    def __len__(self) -> int:
        return len(self.qrots)

    def parameters(self):
        """Every camera's quaternion, translation and intrinsics."""
        return [*self.qrots, *self.tvecs, *self.intrs]

    def intrinsic_params(self, idx_list) -> torch.Tensor:
        return torch.stack([self.intrs[i] for i in idx_list], dim=0)

    def translation_vectors(self, idx_list) -> torch.Tensor:
        return torch.stack([self.tvecs[i] for i in idx_list], dim=0)

    def rotation_matrices(self, idx_list) -> torch.Tensor:
        q = torch.stack([self.qrots[i] for i in idx_list], dim=0)
        return unitquat_to_rotmat(torch.nn.functional.normalize(q, dim=-1))

    def extrinsic_matrices(self, idx_list) -> torch.Tensor:
        """[C,4,4] world->camera matrices [R t; 0 0 0 1]."""
        R = self.rotation_matrices(idx_list)
        Rt = torch.cat([R, self.translation_vectors(idx_list).unsqueeze(-1)], dim=-1)
        bottom = torch.tensor([0.0, 0.0, 0.0, 1.0], dtype=Rt.dtype, device=Rt.device)
        return torch.cat([Rt, bottom.expand(Rt.shape[0], 1, 4)], dim=-2)

    def camera_centers(self, idx_list) -> torch.Tensor:
        """[C,3] camera centres -R^T t."""
        R = self.rotation_matrices(idx_list)
        t = self.translation_vectors(idx_list).unsqueeze(-1)
        return torch.matmul(-R.transpose(-1, -2), t).squeeze(-1)

    def poses(self, idx_list):
        """(extrinsic_matrices, camera_centers) of the cameras in one call;
        on a CUDA device one camera-pose kernel per camera each way."""
        idx = list(idx_list)
        if idx and self.qrots[idx[0]].is_cuda:
            from . import fused

            E, c = zip(*(fused.camera_pose(self.qrots[i], self.tvecs[i]) for i in idx))
            return torch.stack(E, 0), torch.stack(c, 0)
        return self.extrinsic_matrices(idx), self.camera_centers(idx)

    @property
    def image_height(self) -> int:
        return self.height

    @property
    def image_width(self) -> int:
        return self.width
