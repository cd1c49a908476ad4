"""The continuous-batching server: every result is the same alone (the plain
one-request path) and in the mix (batched with other views of its scene,
overlapping other batches): tolerance 1e-5 abs -- the batched path shares
every list, order and blend arithmetic with the plain path, only the colour
is the fused SH kernel's; and admission by memory still serves every
request."""
import pytest
import torch

from pointrix_gb300 import serve

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes():
    return serve.serving_scenes(seed=3, count=3, n_min=20_000, n_max=120_000)


def test_results_identical_alone_and_in_the_mix(scenes):
    reqs = serve.random_requests(24, len(scenes), seed=1)
    alone = [serve.render_plain(scenes[r.scene], r).clone() for r in reqs]
    server = serve.RenderServer(scenes, slots=6)
    for r in serve.random_requests(24, len(scenes), seed=1):
        server.submit(r)
    done = {r.rid: r for r in server.close(timeout=120)}
    assert len(done) == 24
    for i, ref in enumerate(alone):
        img = done[i].image
        assert img.shape == ref.shape
        assert float((img - ref).abs().max()) <= 1e-5
    assert max(server.batches) > 1            # requests of one scene were batched
    assert sum(server.batches) == 24
    assert server.in_use == 0 and len(server.free_streams) == 6


def test_memory_budget_admission_serialises_but_serves_all(scenes):
    # a budget below one batch's working set: batches run one at a time
    server = serve.RenderServer(scenes, slots=4, memory_budget=1)
    reqs = serve.random_requests(8, len(scenes), seed=2)
    for r in reqs:
        server.submit(r)
    done = server.close(timeout=120)
    assert sorted(r.rid for r in done) == list(range(8))
    assert all(r.image is not None and torch.isfinite(r.image).all() for r in done)
    assert server.in_use == 0


def test_poisson_load_reports_latency(scenes):
    reqs = serve.random_requests(40, len(scenes), seed=3, rate=400.0)
    server = serve.RenderServer(scenes, slots=8)
    t0 = serve.drive(server, reqs)
    stats = serve.summarize(server.close(timeout=120), t0)
    assert stats["requests"] == 40
    assert 0 < stats["p50_ms"] <= stats["p99_ms"]
