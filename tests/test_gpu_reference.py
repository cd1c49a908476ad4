"""The GB300 renderer against the reference's own renderer code (GPU).

* Fixture: ``tests/golden/reference/glue.pt`` holds what the reference's
  ``MsplatRender.render_iter`` and ``render_batch``
  (``pointrix/model/renderer/msplat.py:51-213``) and the example
  ``MsplatNormalRender`` (``examples/supervise/renderer.py:25-102``) gave,
  executed around the CPU oracle (float32 geometry, float64 colour and
  blend).  ``pointrix_gb300.renderer.MsplatRender`` on the GPU must give the
  same radii and visibility bit for bit, the same images within 1e-5 abs,
  and the same gradients within 1e-4 (``tests/bars.py``).
* Live: where the reference is installed (``baseline/_ref``), its
  ``MsplatRender`` runs unmodified with ``import msplat`` resolved to this
  repository's shim (``msplat/__init__.py``) -- the drop-in as Pointrix
  would use it -- and must render bit-identical images to
  ``pointrix_gb300.renderer.MsplatRender`` with the same operators
  (unfused glue), and within the bars with the fused default.
"""
import os

import pytest
import torch

import msplat as shim
from pointrix_gb300 import ops
from pointrix_gb300 import workloads as WL
from pointrix_gb300.renderer import MsplatRender
from tests import refload
from tests.bars import assert_grad_close, assert_image_close

pytestmark = pytest.mark.gpu
DEV = "cuda"
GLUE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference", "glue.pt")
live = pytest.mark.skipif(refload.pointrix_dir() is None,
                          reason="reference source not installed (baseline/_ref)")
CONFIGS = {
    "fused": dict(),
    "unfused": dict(fused_view_colour=False, fused_preprocess=False),
    "capacity": dict(sort_capacity=1 << 16),
}
PARAMS = ("position", "opacity", "scaling", "rotation", "shs")


@pytest.fixture(scope="module")
def glue():
    return torch.load(GLUE, weights_only=False)


def _leaves(sc):
    return {k: sc[k].to(DEV).clone().requires_grad_(True) for k in PARAMS}


@pytest.mark.parametrize("config", list(CONFIGS))
def test_render_iter_matches_reference_fixture(glue, config):
    sc, ref = glue["scene"], glue["render_iter"]
    r = MsplatRender(MsplatRender.Config(render_depth=True, **CONFIGS[config]))
    r.sh_degree = ref["sh_degree"]
    lv = _leaves(sc)
    extr = sc["extr"][0].to(DEV).clone().requires_grad_(True)
    intr = sc["intr"].to(DEV).clone().requires_grad_(True)
    out = r.render_iter(sc["H"], sc["W"], extr, intr, sc["center"][0].to(DEV), lv["position"],
                        lv["opacity"], lv["scaling"], lv["rotation"], lv["shs"])
    assert torch.equal(out["radii"].cpu(), ref["radii"])
    assert torch.equal(out["visibility"].cpu(), ref["visibility"])
    split = out["rendered_features_split"]
    assert list(split) == ["rgb", "depth"]
    flags = ref["flags"]
    assert_image_close(split["rgb"], ref["rgb"], flags["pix"], what="rgb")
    assert_image_close(split["depth"], ref["depth"], flags["pix"], what="depth")
    img = torch.cat([split["rgb"], split["depth"]])
    loss = ((img - sc["targets"][0].to(DEV)) ** 2).mean()
    loss.backward()
    assert abs(float(loss) - float(ref["loss"])) < 1e-6
    for k in PARAMS:
        assert_grad_close(lv[k].grad, ref["grads"][k], flags["gauss"], what=k)
    assert_grad_close(extr.grad, ref["grads"]["extr"], what="extr")
    assert_grad_close(intr.grad, ref["grads"]["intr"], what="intr")
    assert_grad_close(out["uv_points"].grad, ref["grads"]["uv_points"], flags["gauss"], what="ndc")
    ops.check_device_status()


def test_render_batch_matches_reference_fixture(glue):
    sc, ref = glue["scene"], glue["render_batch"]
    r = MsplatRender(MsplatRender.Config(render_depth=True))
    r.sh_degree = 3
    lv = _leaves(sc)
    rd = dict(height=sc["H"], width=sc["W"], extrinsic_matrix=sc["extr"].to(DEV),
              intrinsic_params=sc["intr"].to(DEV), camera_center=sc["center"].to(DEV), **lv)
    out = r.render_batch(rd)
    assert torch.equal(out["radii"].cpu(), ref["radii"])
    assert torch.equal(out["visibility"].cpu(), ref["visibility"])
    for v in range(2):
        pix = ref["flags"][v]["pix"]
        assert_image_close(out["rgb"][v], ref["rgb"][v], pix, what=f"rgb view {v}")
        assert_image_close(out["depth"][v], ref["depth"][v], pix, what=f"depth view {v}")
    img = torch.cat([out["rgb"], out["depth"]], 1)
    loss = ((img - torch.stack(sc["targets"]).to(DEV)) ** 2).mean()
    loss.backward()
    gauss = ref["flags"][0]["gauss"] | ref["flags"][1]["gauss"]
    for k in PARAMS:
        assert_grad_close(lv[k].grad, ref["grads"][k], gauss, what=k)
    for v in range(2):
        assert_grad_close(out["uv_points"][v].grad, ref["grads"]["uv_points"][v], gauss, what="ndc")
    ops.check_device_status()


@pytest.mark.skipif(refload.examples_dir() is None, reason="reference example not installed")
def test_reference_normal_renderer_through_shim_matches_fixture(glue):
    """``MsplatNormalRender`` (rgb + normal features, no ``+0.5``, its own
    normal post-processing) executed unmodified on this repository's msplat
    shim, against the same code executed around the oracle."""
    sc, ref = glue["scene"], glue["normal"]
    mod = refload.normal_renderer(shim)
    r = refload.make_render(mod, cls="MsplatNormalRender", white_bg=True)
    lv = _leaves(sc)
    normals = sc["normals"].to(DEV).clone().requires_grad_(True)
    out = r.render_iter(sc["H"], sc["W"], sc["extr"][0].to(DEV), sc["intr"].to(DEV),
                        sc["center"][0].to(DEV), lv["position"], lv["opacity"], lv["scaling"],
                        lv["rotation"], lv["shs"], normals=normals)
    assert torch.equal(out["radii"].cpu(), ref["radii"])
    rgb, nrm = out["rendered_features_split"]["rgb"], out["rendered_features_split"]["normal"]
    assert_image_close(rgb, ref["rgb"], what="rgb")
    assert_image_close(nrm, ref["normal"], what="normal")
    t = sc["targets"][0].to(DEV)
    loss = ((rgb - t[:3]) ** 2).mean() + ((nrm - t[1:]) ** 2).mean()
    loss.backward()
    for k in PARAMS:
        assert_grad_close(lv[k].grad, ref["grads"][k], what=k)
    assert_grad_close(normals.grad, ref["grads"]["normals"], what="normals")
    ops.check_device_status()


# ---------------------------------------------- the reference on the shim ---
def _config1():
    scene, cam = WL.scene_small(0)
    pos, sc, q, op, shs = (t.to(DEV) for t in scene.activated())
    return dict(pos=pos, sc=sc, q=q, op=op, shs=shs, cam=cam.to(DEV))


def _run(renderer, c, sh_degree, target=None):
    lv = {k: c[k].clone().requires_grad_(True) for k in ("pos", "sc", "q", "op", "shs")}
    cam = c["cam"]
    out = renderer.render_iter(cam.H, cam.W, cam.extr, cam.intr, cam.center, lv["pos"], lv["op"],
                               lv["sc"], lv["q"], lv["shs"])
    img = torch.cat([out["rendered_features_split"]["rgb"], out["rendered_features_split"]["depth"]])
    if target is not None:
        (img - target).abs().mean().backward()
    return img.detach(), out, lv


@live
@pytest.mark.parametrize("sh_degree", [0, 3])
def test_reference_renderer_through_shim_matches_ours(sh_degree):
    """The 16,384-Gaussian 256x256 workload (RGB + depth, L1 loss), with the
    SH coefficients of degree 3 and the warm-up mask at ``sh_degree``."""
    mod = refload.msplat_renderer(shim)
    c = _config1()
    c["shs"] = WL.scene_sh3(0, c["pos"].shape[0]).shs.to(DEV)
    g = torch.Generator().manual_seed(3)
    target = torch.rand(4, c["cam"].H, c["cam"].W, generator=g).to(DEV)
    ref = refload.make_render(mod, render_depth=True)
    ref.sh_degree = sh_degree
    img_r, out_r, lv_r = _run(ref, c, sh_degree, target)
    for cfg, exact in (("unfused", True), ("fused", False)):
        mine = MsplatRender(MsplatRender.Config(render_depth=True, **CONFIGS[cfg]))
        mine.sh_degree = sh_degree
        img_m, out_m, lv_m = _run(mine, c, sh_degree, target)
        assert torch.equal(out_m["radii"], out_r["radii"]), cfg
        assert torch.equal(out_m["visibility"], out_r["visibility"]), cfg
        if exact:
            # the same operators in the same order: the same image bits; the
            # gradients are sums of float atomics, whose order varies by run
            assert torch.equal(img_m, img_r), cfg
            assert_grad_close(out_m["uv_points"].grad, out_r["uv_points"].grad, rtol=1e-5, what="ndc")
            for k in lv_r:
                assert_grad_close(lv_m[k].grad, lv_r[k].grad, rtol=1e-5, what=f"{cfg} {k}")
        else:
            assert_image_close(img_m, img_r, what=cfg)
            for k in lv_r:
                assert_grad_close(lv_m[k].grad, lv_r[k].grad, what=f"{cfg} {k}")
    ops.check_device_status()


@live
def test_reference_render_batch_through_shim_matches_ours():
    mod = refload.msplat_renderer(shim)
    c = _config1()
    g = torch.Generator().manual_seed(4)
    cams = [WL.make_camera(g, 192, 160, 200.0, 4.0) for _ in range(3)]
    rd = dict(height=160, width=192, extrinsic_matrix=torch.stack([k.extr for k in cams]).to(DEV),
              intrinsic_params=cams[0].intr.to(DEV), camera_center=torch.stack([k.center for k in cams]).to(DEV))
    outs = []
    for r in (refload.make_render(mod, render_depth=True),
              MsplatRender(MsplatRender.Config(render_depth=True, **CONFIGS["unfused"]))):
        lv = {k: c[k].clone().requires_grad_(True) for k in ("pos", "sc", "q", "op", "shs")}
        o = r.render_batch(dict(rd, position=lv["pos"], scaling=lv["sc"], rotation=lv["q"],
                                opacity=lv["op"], shs=lv["shs"]))
        (o["rgb"].square().mean() + o["depth"].mean()).backward()
        outs.append((o, lv))
    (o_r, lv_r), (o_m, lv_m) = outs
    for k in ("rgb", "depth", "visibility", "radii"):
        assert torch.equal(o_m[k], o_r[k]), k
    for a, b in zip(o_m["uv_points"], o_r["uv_points"]):
        assert_grad_close(a.grad, b.grad, rtol=1e-5, what="ndc")
    for k in lv_r:   # float atomics: summation order varies by run
        assert_grad_close(lv_m[k].grad, lv_r[k].grad, rtol=1e-5, what=k)
    ops.check_device_status()
