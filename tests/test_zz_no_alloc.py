"""The allocation-free sort entry point, called through the C ABI.

``pgb_sort_gaussian_noalloc`` serves callers that cannot allocate device
memory (a host application that owns the GPU memory budget, or a hot path
that must not enter the CUDA allocator): its scratch is a fixed static device
array.  These tests check it against the allocating entry points
(``pgb_sort_gaussian_begin``/``finish`` through ``ops.sort_gaussian``) on
calls in a row -- the static scratch keeps the previous call's contents, so
the second call shows that everything that must start at zero is cleared --
with the same bit-exact bar as the other sort tests.  This file is collected
last so that a failure here cannot stop the rest of the suite.
"""
import ctypes as C

import pytest
import torch

from pointrix_gb300 import _lib, ops
from pointrix_gb300 import workloads as WL

pytestmark = pytest.mark.gpu
PGB_ERR_INVALID, PGB_ERR_OVERFLOW = 1, 3
MAX_GAUSSIANS = 262144


def sort_inputs(seed, n, W, H, f, radius, log_scale_shift=0.0):
    scene, _ = WL.scene_small(seed, n=n)
    scene.log_scale += log_scale_shift
    g = torch.Generator().manual_seed(100 + seed)
    cam = WL.make_camera(g, W, H, f, radius)
    pos, sc, q, op, shs = (t.cuda() for t in scene.activated())
    intr, extr = cam.intr.cuda(), cam.extr[:3].cuda().contiguous()
    uv, depth = ops.project_point(pos, intr, extr, W, H)
    vis = depth != 0
    cov = ops.compute_cov3d(sc, q, vis)
    _, rad, tiles = ops.ewa_project(pos, cov, intr, extr, uv, W, H, vis)
    return uv.contiguous(), depth.contiguous(), rad.contiguous(), tiles.contiguous(), W, H


def call_noalloc(uv, depth, rad, tiles, W, H, capacity):
    n = uv.shape[0]
    T = ((W + 15) // 16) * ((H + 15) // 16)
    ids = torch.full((max(capacity, 1),), -1, dtype=torch.int32, device="cuda")
    rng = torch.full((T, 2), -7, dtype=torch.int32, device="cuda")
    k = C.c_int64(-2)
    status = _lib.lib().pgb_sort_gaussian_noalloc(
        uv.data_ptr(), depth.data_ptr(), rad.data_ptr(), tiles.data_ptr(), n, W, H, ids.data_ptr(),
        capacity, rng.data_ptr(), C.byref(k), torch.cuda.current_stream().cuda_stream)
    return status, k.value, ids, rng


@pytest.mark.parametrize("case", [
    (0, 16384, 256, 256, 256.0, 4.0),      # the small workload's scene and camera
    (5, 60000, 640, 480, 460.0, 4.5),
])
def test_noalloc_matches_allocating_sort_on_calls_in_a_row(case):
    uv, depth, rad, tiles, W, H = sort_inputs(*case)
    ids_ref, rng_ref = ops.sort_gaussian(uv, depth, W, H, rad, tiles)
    K = ids_ref.numel()
    assert K > 0
    for _ in range(2):
        status, k, ids, rng = call_noalloc(uv, depth, rad, tiles, W, H, K + 64)
        assert status == 0, _lib.lib().pgb_status_string(status)
        assert k == K
        assert torch.equal(ids[:K], ids_ref)
        assert torch.equal(rng, rng_ref)
        assert bool((ids[K:] == -1).all())          # nothing written past K


def test_noalloc_rejects_sizes_beyond_its_limits():
    uv, depth, rad, tiles, W, H = sort_inputs(0, 16384, 256, 256, 256.0, 4.0)
    K = int(tiles[rad > 0].sum())
    # output buffer smaller than K: refused after phase one, K reported
    status, k, ids, _ = call_noalloc(uv, depth, rad, tiles, W, H, K - 1)
    assert status == PGB_ERR_OVERFLOW and k == K
    assert bool((ids == -1).all())
    # more Gaussians than the static scratch is sized for: refused up front
    big = MAX_GAUSSIANS + 1
    z2 = torch.zeros(big, 2, device="cuda")
    z1 = torch.zeros(big, device="cuda")
    zi = torch.zeros(big, dtype=torch.int32, device="cuda")
    status, k, _, _ = call_noalloc(z2, z1, zi, zi, 64, 64, 16)
    assert status == PGB_ERR_INVALID and k == -1


def test_noalloc_rejects_k_beyond_the_static_array():
    """n within the limit, but K (large splats on a large image) beyond what
    the rest of the static array holds: refused after phase one with K
    reported, the caller's id buffer untouched even though it is big enough."""
    uv, depth, rad, tiles, W, H = sort_inputs(1, 65536, 1024, 1024, 1024.0, 4.0,
                                              log_scale_shift=3.0)
    K = int(tiles[rad > 0].sum())
    assert K > 2_000_000          # well past the ~1.0M entries the array holds
    status, k, ids, rng = call_noalloc(uv, depth, rad, tiles, W, H, K)
    assert status == PGB_ERR_OVERFLOW and k == K
    assert bool((ids == -1).all())
    assert bool((rng == -7).all())
