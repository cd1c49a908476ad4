"""sort_gaussian beyond the single-image default: capacity mode (K kept on
the device, no host read-back), CUDA-graph capture of sort + blend, and tile
grids that need the 9-bit and the three-pass tile sorts.  Sorted ids and tile
ranges are compared bit-exactly with the oracle or with the host-K sort."""
import pytest
import torch

from oracle import msplat_cpu as O
from pointrix_gb300 import _lib, ops
from pointrix_gb300 import workloads as WL

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _render_inputs(pos, sc, q, op, shs, intr, extr, W, H):
    uv, depth = ops.project_point(pos, intr, extr, W, H)
    vis = depth != 0
    cov = ops.compute_cov3d(sc, q, vis)
    conic, radius, tiles = ops.ewa_project(pos, cov, intr, extr, uv, W, H, vis)
    rgb = (ops.compute_sh(shs.permute(0, 2, 1), pos / pos.norm(dim=1, keepdim=True)) + 0.5).clamp(min=0)
    return dict(uv=uv, depth=depth, radius=radius, tiles=tiles, conic=conic, op=op,
                feat=torch.cat([rgb, depth], 1), W=W, H=H)


def _prepare(n, W, H, seed, f=None):
    scene, _ = WL.scene_small(seed, n=n)
    g = torch.Generator().manual_seed(seed + 17)
    cam = WL.make_camera(g, W, H, float(f or max(W, H)), 4.0)
    leaves = [t.to(DEV) for t in scene.activated()]
    intr, extr = cam.intr.to(DEV), cam.extr[:3].to(DEV).contiguous()
    p = _render_inputs(*leaves, intr, extr, W, H)
    p["leaves"], p["intr"], p["extr"] = leaves, intr, extr
    return p


def _sort(p, capacity=None):
    return ops.sort_gaussian(p["uv"], p["depth"], p["W"], p["H"], p["radius"], p["tiles"],
                             capacity=capacity)


@pytest.fixture(scope="module")
def small():
    return _prepare(16384, 256, 256, 0, f=256)


@pytest.mark.parametrize("extra", [0, 1, 1000, -1])
def test_capacity_matches_exact_sort(small, extra):
    ids, rng = _sort(small)
    K = ids.numel()
    cap = 3 * K if extra < 0 else K + extra
    ids_c, rng_c = _sort(small, capacity=cap)
    assert ids_c.numel() == cap
    assert torch.equal(ids_c[:K], ids) and torch.equal(rng_c, rng)
    ops.check_device_status()


def test_capacity_overflow_reports_and_leaves_tiles_empty(small):
    ids, _ = _sort(small)
    K = ids.numel()
    for cap in (K - 1, K // 3, 0):
        _, rng = _sort(small, capacity=cap)
        assert int(rng.abs().sum()) == 0
        with pytest.raises(_lib.PgbError):
            ops.check_device_status()
    ops.check_device_status()   # the failure was reported once and cleared


@pytest.mark.parametrize("W,H", [(4800, 4800), (8400, 8400)])
def test_large_tile_grids_match_oracle(W, H):
    """90,000 tiles take two 9-bit tile passes, 275,625 tiles three 8-bit
    passes; both must give the oracle's ids and ranges."""
    p = _prepare(3000, W, H, 5)
    T = ((W + 15) // 16) * ((H + 15) // 16)
    assert ops._tile_passes(T) == (2 if T <= (1 << 18) else 3)
    ids, rng = _sort(p)
    cpu = lambda t: t.detach().cpu()  # noqa: E731
    ids_o, rng_o = O.sort_gaussian(cpu(p["uv"]), cpu(p["depth"]), W, H, cpu(p["radius"]),
                                   cpu(p["tiles"]))
    assert ids.numel() > 0 and int(rng[:, 0].max()) > 0
    assert torch.equal(cpu(ids), ids_o) and torch.equal(cpu(rng), rng_o)
    ids_c, rng_c = _sort(p, capacity=ids.numel() + 77)
    assert torch.equal(ids_c[:ids.numel()], ids) and torch.equal(rng_c, rng)
    ops.check_device_status()


def test_sort_and_blend_replay_in_a_cuda_graph(small):
    """Projection, capacity-mode sort and blend captured once and replayed on
    new Gaussian positions copied into the captured input: every replay
    equals the eager result for those positions."""
    p = small
    W, H = p["W"], p["H"]
    ids, _ = _sort(p)
    cap = 2 * ids.numel()
    pos0, sc, q, op, shs = p["leaves"]
    static_pos = pos0.clone()

    def run(pos, capacity):
        r = _render_inputs(pos, sc, q, op, shs, p["intr"], p["extr"], W, H)
        i, rng = ops.sort_gaussian(r["uv"], r["depth"], W, H, r["radius"], r["tiles"],
                                   capacity=capacity)
        return ops.alpha_blending(r["uv"], r["conic"], r["op"], r["feat"], i, rng, 0.0, W, H)

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(2):
            run(static_pos, cap)
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        out = run(static_pos, cap)
    g = torch.Generator(device=DEV).manual_seed(9)
    for step in range(3):
        pos_new = pos0 + 0.02 * torch.randn(pos0.shape, generator=g, device=DEV)
        static_pos.copy_(pos_new)
        graph.replay()
        torch.cuda.synchronize()
        ref = run(pos_new, None)
        assert torch.equal(out, ref), step
    ops.check_device_status()
