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


def test_render_batch_aggregates_views_as_pointrix(monkeypatch):
    """render_batch (pointrix/model/renderer/msplat.py:160-213) with
    render_iter stubbed: per-view slices of the batched keys only, features
    stacked per name, uv_points kept as a list, visibility any() and radii
    max() over the views."""
    B, N, H, W = 3, 5, 4, 6
    seen = []

    def fake_iter(self, **kw):
        i = len(seen)
        seen.append(kw)
        return {"rendered_features_split": {"rgb": torch.full((3, H, W), float(i)),
                                            "depth": torch.full((1, H, W), 10.0 + i)},
                "uv_points": torch.full((N, 2), float(i)),
                "visibility": torch.arange(N) == i,
                "radii": torch.arange(N, dtype=torch.int32) * (i + 1)}

    monkeypatch.setattr(MsplatRender, "render_iter", fake_iter)
    r = MsplatRender()
    extr = torch.randn(B, 4, 4)
    centres = torch.randn(B, 3)
    intr = torch.tensor([[100.0, 100.0, 3.0, 2.0]])
    shs = torch.zeros(N, 16, 3)
    out = r.render_batch({"extrinsic_matrix": extr, "camera_center": centres,
                          "intrinsic_params": intr, "shs": shs, "height": H, "width": W})
    assert len(seen) == B
    for i, kw in enumerate(seen):
        assert torch.equal(kw["extrinsic_matrix"], extr[i])
        assert torch.equal(kw["camera_center"], centres[i])
        assert kw["intrinsic_params"] is intr and kw["shs"] is shs  # not sliced
    assert out["rgb"].shape == (B, 3, H, W) and out["depth"].shape == (B, 1, H, W)
    assert [float(out["rgb"][i, 0, 0, 0]) for i in range(B)] == [0.0, 1.0, 2.0]
    assert isinstance(out["uv_points"], list) and len(out["uv_points"]) == B
    assert out["visibility"].tolist() == [True, True, True, False, False]
    assert torch.equal(out["radii"], torch.arange(N, dtype=torch.int32) * B)


def test_band_grouping_of_tile_rows():
    """The recompute mode's bands: consecutive tile rows grouped up to the
    target, covering every row once, entry counts preserved."""
    from pointrix_gb300.ops import band_rows, group_rows
    rows = [3, 9, 0, 4, 4, 4, 12, 1]
    for kw in (dict(max_entries=10), dict(bands=3), dict(bands=1), dict(max_entries=1)):
        plan = group_rows(rows, **kw)
        assert plan[0][0] == 0 and plan[-1][1] == len(rows)
        assert all(a[1] == b[0] and a[0] < a[1] for a, b in zip(plan, plan[1:]))
        assert [k for *_, k in plan] == [sum(rows[a:b]) for a, b, _ in plan]
    assert len(group_rows(rows, bands=3)) == 3
    assert group_rows(rows, bands=1) == [(0, 8, 37)]
    assert band_rows(100, 16 * 9, bands=3) == [(0, 3), (3, 6), (6, 9)]


def test_band_list_scratch_and_limits():
    """The band lists' scratch query (no GPU needed): one count per band and
    block of 4,096 depth positions, 256-byte rounded; 0 for band counts
    outside 1..256 (the banded sort then keeps its whole-order path)."""
    from pointrix_gb300 import _lib
    lib = _lib.lib()
    q = lib.pgb_band_lists_scratch_bytes
    assert ops.BAND_LIST_MAX == 256
    assert q(0, 1) == 256 and q(4096, 1) == 256
    assert q(4097, 13) == 256                      # 2 blocks x 13 bands x 4 B
    assert q(6_000_000, 13) == -(-(13 * 1465 * 4) // 256) * 256
    assert q(100, 0) == 0 and q(100, 257) == 0 and q(-1, 4) == 0
    assert q(10_000_000, 256) >= 256 * ((10_000_000 + 4095) // 4096) * 4


class _FakeEvent:
    def __init__(self, done):
        self.done = done
        self.queried = 0

    def query(self):
        self.queried += 1
        return self.done

    def synchronize(self):
        self.done = True


def test_deferred_status_checks_drain_in_order_and_raise():
    """The deferred device-status read-backs: a non-blocking drain checks
    the completed ones in order and stops at the first still pending
    (keeping it and everything after it unqueried, ahead of later
    deferrals); a completed non-zero word raises; a blocking drain waits
    for all."""
    import numpy as np
    import torch
    from pointrix_gb300 import _lib, ops

    def word(code):
        return torch.from_numpy(np.array([code, 0, 0], dtype=np.int64))

    saved = list(ops._pending)
    try:
        done1, pend, after = _FakeEvent(True), _FakeEvent(False), _FakeEvent(True)
        ops._pending[:] = [(done1, word(0), "a"), (pend, word(0), "b"), (after, word(0), "c")]
        ops._drain_pending(block=False)
        assert [w for _, _, w in ops._pending] == ["b", "c"]
        assert after.queried == 0            # not queried behind a pending one
        ops._pending.append((_FakeEvent(True), word(0), "d"))
        ops._drain_pending(block=True)
        assert ops._pending == []
        ops._pending[:] = [(_FakeEvent(True), word(0), "ok"), (_FakeEvent(True), word(6), "bad")]
        with pytest.raises(_lib.PgbError, match="bad"):
            ops._drain_pending(block=False)
        assert ops._pending == []
    finally:
        ops._pending[:] = saved
