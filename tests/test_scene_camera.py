"""The scene's cameras (``pointrix/model/camera/camera_model.py:19-210``):
rotation matrix -> quaternion by Shepperd's method (all four branches,
known answers), the accessors on CPU against the dataset matrices, the
trainable cameras' gradients, and on the GPU the camera-pose kernel path of
``poses`` against the torch composition."""
import math

import numpy as np
import pytest
import torch

from pointrix_gb300.camera import CameraModel, CameraPrior, rotmat_to_unitquat, unitquat_to_rotmat
from pointrix_gb300 import ops


def _rot(q):
    q = torch.as_tensor(q, dtype=torch.float64)
    return unitquat_to_rotmat(q / q.norm()).numpy()


@pytest.mark.parametrize("R,q", [
    (np.eye(3), [1, 0, 0, 0]),
    (np.diag([1.0, -1, -1]), [0, 1, 0, 0]),      # 180 deg about x: the R00 branch
    (np.diag([-1.0, 1, -1]), [0, 0, 1, 0]),      # about y: the R11 branch
    (np.diag([-1.0, -1, 1]), [0, 0, 0, 1]),      # about z: the R22 branch
    ([[0.0, -1, 0], [1, 0, 0], [0, 0, 1]], [math.sqrt(0.5), 0, 0, math.sqrt(0.5)]),  # 90 about z
])
def test_known_rotations(R, q):
    assert np.allclose(rotmat_to_unitquat(R), q, atol=1e-15)


def test_round_trip_over_every_branch():
    g = np.random.default_rng(0)
    picks = set()
    for _ in range(2000):
        q = g.standard_normal(4)
        q /= np.linalg.norm(q)
        R = _rot(q)
        picks.add(int(np.argmax([np.trace(R), R[0, 0], R[1, 1], R[2, 2]])))
        back = rotmat_to_unitquat(R)
        assert back[0] >= 0 and abs(np.linalg.norm(back) - 1) < 1e-15
        assert np.allclose(back, q if q[0] >= 0 else -q, atol=1e-12)
    assert picks == {0, 1, 2, 3}


def _priors(n=5, seed=1):
    g = np.random.default_rng(seed)
    out = []
    for i in range(n):
        E = np.eye(4)
        E[:3, :3] = _rot(g.standard_normal(4))
        E[:3, 3] = g.standard_normal(3) * 3
        intr = np.array([800.0 + i, 810.0, 320.0, 240.0 + i])
        out.append(CameraPrior(E, intr, 640 + i, 480 + i))
    return out


def test_accessors_reproduce_the_dataset_cameras():
    priors = _priors()
    cams = CameraModel()
    cams.setup(priors, device="cpu")
    assert len(cams) == 5 and (cams.image_width, cams.image_height) == (644, 484)
    idx = [3, 0, 4]
    E = cams.extrinsic_matrices(idx)
    assert E.shape == (3, 4, 4) and E.dtype == torch.float32
    for j, i in enumerate(idx):
        assert np.allclose(E[j].numpy(), priors[i].extrinsic_matrix, atol=2e-6)
        R, t = priors[i].extrinsic_matrix[:3, :3], priors[i].extrinsic_matrix[:3, 3]
        assert np.allclose(cams.camera_centers(idx)[j].numpy(), -R.T @ t, atol=1e-5)
        assert np.array_equal(cams.intrinsic_params(idx)[j].numpy(),
                              priors[i].intrinsic_params.astype(np.float32))
    E2, c2 = cams.poses(idx)
    assert torch.equal(E2, E) and torch.equal(c2, cams.camera_centers(idx))
    with pytest.raises(ValueError, match="fx, fy"):
        CameraModel().setup([CameraPrior(np.eye(4), np.ones(3), 4, 4)], device="cpu")


def test_trainable_cameras_are_leaves_with_gradients():
    cams = CameraModel(dict(enable_training=True))
    cams.setup(_priors(3), device="cpu")
    params = cams.parameters()
    assert len(params) == 9 and all(p.is_leaf and p.requires_grad for p in params)
    E, c = cams.poses([1, 2])
    (E.sum() + c.square().sum() + cams.intrinsic_params([1]).sum()).backward()
    assert cams.qrots[0].grad is None and cams.tvecs[0].grad is None
    for p in (cams.qrots[1], cams.tvecs[2], cams.intrs[1]):
        assert p.grad is not None and bool(p.grad.abs().sum() > 0)


@pytest.mark.gpu
def test_poses_on_the_gpu_match_the_composition():
    """``poses`` through the camera-pose kernel against the accessors' torch
    composition: values and gradients to 1e-5."""
    priors = _priors(4, seed=3)
    cams, ref = CameraModel(dict(enable_training=True)), CameraModel(dict(enable_training=True))
    cams.setup(priors, device="cuda")
    ref.setup(priors, device="cuda")
    idx = [2, 0, 3]
    g = torch.Generator().manual_seed(4)
    dE, dc = torch.randn(3, 4, 4, generator=g).cuda(), torch.randn(3, 3, generator=g).cuda()
    E, c = cams.poses(idx)
    Er, cr = ref.extrinsic_matrices(idx), ref.camera_centers(idx)
    ((E * dE).sum() + (c * dc).sum()).backward()
    ((Er * dE).sum() + (cr * dc).sum()).backward()
    assert torch.allclose(E, Er, atol=1e-6) and torch.allclose(c, cr, atol=1e-5)
    for a, b in zip(cams.parameters(), ref.parameters()):
        if b.grad is None:
            assert a.grad is None
        else:
            assert torch.allclose(a.grad, b.grad, rtol=1e-5, atol=1e-5)
    ops.check_device_status()
