"""The renderer's glue and the oracle, held to the reference's own code (CPU).

Two sources, the same functions:

* the fixture ``tests/golden/reference/glue.pt``, which
  ``tests/golden/make_reference_golden.py`` made by executing the reference's
  ``RenderFeatures``, ``unitquat_to_rotmat``/``quat_to_rotmat``, ``ssim``,
  ``DensificationController.preprocess`` and ``MsplatRender.render_iter``/
  ``render_batch`` (these tests always run);
* the reference files themselves, loaded by ``tests/refload.py`` from the
  offline install (these tests skip where it is absent).
"""
import os

import pytest
import torch

from oracle import msplat_cpu as O
from oracle import msplat_ops
from pointrix_gb300 import workloads as WL
from pointrix_gb300.camera import unitquat_to_rotmat as cam_rotmat
from pointrix_gb300.renderer import MsplatRender, RenderFeatures
from tests import refload

GLUE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference", "glue.pt")
live = pytest.mark.skipif(refload.pointrix_dir() is None,
                          reason="reference source not installed (baseline/_ref)")


@pytest.fixture(scope="module")
def glue():
    return torch.load(GLUE, weights_only=False)


# ------------------------------------------------------------- fixture ---
def test_render_features_reproduce_reference(glue):
    f = glue["features"]
    rf = RenderFeatures(rgb=f["rgb"], depth=f["depth"], normal=f["normal"])
    assert torch.equal(rf.combine(), f["combined"])
    parts = rf.split(f["image"])
    assert list(parts) == list(f["split"])
    for k, v in f["split"].items():
        assert torch.equal(parts[k], v), k


def test_quaternion_rotations_reproduce_reference(glue):
    """Every quaternion -> rotation of this repository -- the oracle's (used by
    compute_cov3d), the camera model's and the workloads' matmul form --
    against ``pointrix/utils/pose.py:unitquat_to_rotmat``."""
    p = glue["pose"]
    ref = p["unitquat_to_rotmat"]
    R = O.quat_to_rot(p["unit"])
    mine = torch.stack([torch.stack(list(r), 1) for r in R], 1)
    assert torch.allclose(mine, ref, atol=1e-14)
    assert torch.equal(cam_rotmat(p["unit"]), ref)
    assert torch.allclose(WL.rotation_from_unit_quat(p["unit"]), ref, atol=1e-14)
    # quat_to_rotmat normalises first (pose.py:86-118)
    assert torch.allclose(cam_rotmat(p["q"] / p["q"].norm(dim=1, keepdim=True)), p["quat_to_rotmat"],
                          atol=1e-15)


def test_fixture_integer_outputs_are_the_float32_oracle(glue):
    """The fixture's radii come from the reference's render_iter around the
    float32 oracle; the oracle's own chain gives the same integers."""
    sc, ri = glue["scene"], glue["render_iter"]
    extr = sc["extr"][0][:3]
    uv, depth = O.project_point(sc["position"], sc["intr"], extr, sc["W"], sc["H"], nearest=0.2)
    cov = O.compute_cov3d(sc["scaling"], sc["rotation"], depth != 0)
    _, radius, _ = O.ewa_project(sc["position"], cov, sc["intr"], extr, uv, sc["W"], sc["H"], depth != 0)
    assert torch.equal(radius, ri["radii"])
    assert torch.equal(radius > 0, ri["visibility"])


# ---------------------------------------------------------------- live ---
@live
def test_fixture_is_the_installed_reference(glue):
    """The installed reference files are the ones the fixture was made from,
    and re-running the generator reproduces it."""
    from tests.golden import make_reference_golden as gen

    assert gen.digests(refload.pointrix_dir()) == glue["digests"]
    nthreads = torch.get_num_threads()
    torch.set_num_threads(1)
    try:
        fresh = gen.make_all()
    finally:
        torch.set_num_threads(nthreads)

    def same(a, b, path):
        if isinstance(a, dict):
            assert set(a) == set(b), path
            for k in a:
                same(a[k], b[k], f"{path}.{k}")
        elif isinstance(a, (list, tuple)):
            for i, (x, y) in enumerate(zip(a, b)):
                same(x, y, f"{path}[{i}]")
        elif torch.is_tensor(a) and a.is_floating_point():
            assert torch.allclose(a, b, rtol=1e-12, atol=1e-14), path
        elif torch.is_tensor(a):
            assert torch.equal(a, b), path
        else:
            assert a == b, path

    same(fresh, glue, "glue")


@live
def test_render_features_is_the_reference_class():
    ru = refload.renderer_utils()
    g = torch.Generator().manual_seed(5)
    feats = dict(rgb=torch.rand(9, 3, generator=g), depth=torch.rand(9, 1, generator=g),
                 normal=torch.rand(9, 3, generator=g))
    ref = ru.RenderFeatures(**feats, note="not a tensor")
    mine = RenderFeatures(**feats, note="not a tensor")
    assert torch.equal(mine.combine(), ref.combine())
    img = torch.rand(7, 4, 5, generator=g)
    a, b = mine.split(img), ref.split(img)
    assert list(a) == list(b) and all(torch.equal(a[k], b[k]) for k in a)


@live
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_oracle_chain_is_the_reference_render_iter(dtype):
    """The reference's render_iter with ``import msplat`` bound to the oracle's
    operators gives what the oracle's own chain (``render_view``, which the
    tests and the smoke use) gives: the oracle's glue is the reference's."""
    mod = refload.msplat_renderer(msplat_ops)
    r = refload.make_render(mod, render_depth=True)
    r.sh_degree = 2
    scene, cam = WL.scene_small(2, n=2000)
    pos, sc, q, op = (t.to(dtype) for t in scene.activated()[:4])
    shs = WL.scene_sh3(2, 2000).shs.to(dtype)
    with refload.cuda_calls_stay_on_cpu():
        out = r.render_iter(cam.H, cam.W, cam.extr.to(dtype), cam.intr.to(dtype),
                            cam.center.to(dtype), pos, op, sc, q, shs)
    img = torch.cat([out["rendered_features_split"]["rgb"], out["rendered_features_split"]["depth"]])
    ref, _, radius, _ = O.render_view(pos, sc, q, op, shs, None, cam.center.to(dtype),
                                      cam.intr.to(dtype), cam.extr[:3].to(dtype), cam.W, cam.H,
                                      sh_degree=2)
    assert torch.equal(out["radii"], radius)
    assert torch.equal(out["visibility"], radius > 0)
    assert torch.equal(img, ref)


@live
def test_render_batch_is_the_reference_loop(monkeypatch):
    """Our ``render_batch`` and the reference's (``msplat.py:160-213``) with
    the same per-view stub: identical slicing, stacking and aggregation."""
    mod = refload.msplat_renderer(msplat_ops)
    B, N, H, W = 3, 6, 4, 5

    def fake_iter(self, **kw):
        i = int(kw["camera_center"][0])
        return {"rendered_features_split": {"rgb": torch.full((3, H, W), float(i)),
                                            "depth": kw["extrinsic_matrix"][:1, :1].expand(1, H, W) + i},
                "uv_points": torch.full((N, 2), float(i)),
                "visibility": (torch.arange(N) % (i + 2)) == 0,
                "radii": (torch.arange(N, dtype=torch.int32) * (i + 1)) % 7}

    monkeypatch.setattr(MsplatRender, "render_iter", fake_iter)
    monkeypatch.setattr(mod.MsplatRender, "render_iter", fake_iter)
    rd = {"extrinsic_matrix": torch.randn(B, 4, 4), "camera_center": torch.arange(B).float()[:, None].expand(B, 3),
          "intrinsic_params": torch.tensor([[10.0, 10.0, 2.0, 2.0]]), "shs": torch.zeros(N, 16, 3),
          "height": H, "width": W}
    mine = MsplatRender().render_batch(dict(rd))
    ref = refload.make_render(mod).render_batch(dict(rd))
    assert list(mine) == list(ref)
    for k in ref:
        if k == "uv_points":
            assert all(torch.equal(a, b) for a, b in zip(mine[k], ref[k]))
        else:
            assert torch.equal(mine[k], ref[k]), k


@live
def test_renderer_config_schedule_and_state_match_reference():
    mod = refload.msplat_renderer(msplat_ops)
    ref_cfg = mod.MsplatRender.Config()
    mine_cfg = MsplatRender.Config()
    for f in ("update_sh_iter", "max_sh_degree", "render_depth"):
        assert getattr(mine_cfg, f) == getattr(ref_cfg, f), f
    ref = refload.make_render(mod, max_sh_degree=2)
    ref.cfg.update_sh_iter = 7
    mine = MsplatRender(dict(update_sh_iter=7, max_sh_degree=2))
    for step in range(1, 40):
        ref.update_sh_degree(step)
        mine.update_sh_degree(step)
        assert ref.sh_degree == mine.sh_degree, step
    assert mine.state_dict() == ref.state_dict()
    assert mine.bg_color == ref.bg_color
