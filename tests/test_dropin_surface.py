"""The drop-in surface, on CPU: every call form Pointrix makes on ``msplat``
binds to the operators of ``import msplat``; each operator refuses host
tensors with an error instead of computing anywhere but on the GPU; and the
renderer's host logic (configuration defaults, SH warm-up schedule, state
dict, feature packing) behaves as Pointrix's ``MsplatRender``."""
import inspect

import pytest
import torch

import msplat
from pointrix_gb300 import ops
from pointrix_gb300.renderer import MsplatRender, RenderFeatures

_ = object()  # stands for any argument: only the call's shape is bound

# (operator, positional count, keywords) of each call in the reference
CALL_FORMS = [
    # pointrix/model/renderer/msplat.py
    ("compute_sh", 2, ()),                      # :104
    ("project_point", 5, ("nearest",)),         # :109-113
    ("compute_cov3d", 3, ()),                   # :118
    ("ewa_project", 8, ()),                     # :121-130
    ("sort_gaussian", 6, ()),                   # :133-135
    ("alpha_blending", 10, ()),                 # :148-151 (ndc positional)
    # examples/supervise/renderer.py
    ("compute_sh", 2, ()),                      # :42
    ("project_point", 5, ()),                   # :45-49 (nearest defaulted)
    ("compute_cov3d", 3, ()),                   # :54
    ("ewa_project", 8, ()),                     # :57-66
    ("sort_gaussian", 6, ()),                   # :69-71
    ("alpha_blending", 10, ()),                 # :83-86
    # the form without the ndc gradient sink
    ("alpha_blending", 9, ()),
]


@pytest.mark.parametrize("name,npos,kws", CALL_FORMS)
def test_reference_call_forms_bind(name, npos, kws):
    fn = getattr(msplat, name)
    assert fn is getattr(ops, name)
    inspect.signature(fn).bind(*([_] * npos), **{k: _ for k in kws})


def test_project_point_defaults():
    p = inspect.signature(msplat.project_point).parameters
    assert p["nearest"].default == 0.2 and p["extent"].default == 1.3


def _host_calls():
    n, W, H = 8, 32, 16
    f = torch.zeros
    i32 = dict(dtype=torch.int32)
    intr, extr = torch.tensor([20.0, 20.0, 16.0, 8.0]), torch.eye(4)[:3].contiguous()
    uv, depth = f(n, 2), f(n, 1)
    vis = torch.ones(n, 1, dtype=torch.bool)
    radius, tiles = f(n, 1, **i32), f(n, 1, **i32)
    ids, rng = f(0, **i32), f(4, 2, **i32)
    return [
        ("compute_sh", (f(n, 3, 16), f(n, 3))),
        ("project_point", (f(n, 3), intr, extr, W, H)),
        ("compute_cov3d", (f(n, 3), f(n, 4), vis)),
        ("ewa_project", (f(n, 3), f(n, 6), intr, extr, uv, W, H, vis)),
        ("sort_gaussian", (uv, depth, W, H, radius, tiles)),
        ("alpha_blending", (uv, f(n, 3), f(n, 1), f(n, 3), ids, rng, 0.0, W, H)),
    ]


@pytest.mark.parametrize("name,args", _host_calls(), ids=lambda v: v if isinstance(v, str) else "")
def test_operators_refuse_host_tensors(name, args):
    with pytest.raises(ValueError, match="CUDA tensor"):
        getattr(msplat, name)(*args)


def test_renderer_defaults_match_pointrix():
    cfg = MsplatRender.Config()  # pointrix/model/renderer/msplat.py:29-31
    assert (cfg.update_sh_iter, cfg.max_sh_degree, cfg.render_depth) == (1000, 3, False)


def test_sh_warm_up_schedule_and_state_dict():
    r = MsplatRender(dict(update_sh_iter=10, max_sh_degree=2))
    r.setup(white_bg=True, device="cpu")
    assert r.sh_degree == 0 and r.bg_color == 1.0
    degrees = []
    for step in range(1, 61):  # pointrix/model/renderer/msplat.py:215-226
        r.update_sh_degree(step)
        degrees.append(r.sh_degree)
    assert degrees[8] == 0 and degrees[9] == 1 and degrees[19] == 2 and degrees[-1] == 2
    s = r.state_dict()
    r2 = MsplatRender()
    r2.setup(white_bg=False, device="cpu")
    r2.load_state_dict(s)
    assert r2.sh_degree == 2 and r2.bg_color == 0.0


def test_render_features_pack_in_keyword_order():
    n = 5
    rgb, depth, normal = torch.rand(n, 3), torch.rand(n, 1), torch.rand(n, 3)
    rf = RenderFeatures(rgb=rgb, depth=depth, normal=normal, note="not a tensor")
    packed = rf.combine()  # pointrix/model/renderer/utils/renderer_utils.py:30-46
    assert torch.equal(packed, torch.cat([rgb, depth, normal], 1))
    img = torch.arange(7 * 2 * 3, dtype=torch.float32).reshape(7, 2, 3)
    parts = rf.split(img)  # renderer_utils.py:48-71
    assert list(parts) == ["rgb", "depth", "normal"]
    assert torch.equal(parts["rgb"], img[:3]) and torch.equal(parts["depth"], img[3:4])
    assert torch.equal(parts["normal"], img[4:])
