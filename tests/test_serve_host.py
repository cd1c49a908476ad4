"""Host-side logic of the server (no GPU): request generation, Poisson
arrivals, statistics and memory accounting."""
import math

from pointrix_gb300 import serve


class _Req:
    def __init__(self, arrival, finished, pixels):
        self.arrival, self.finished, self.pixels = arrival, finished, pixels

    @property
    def latency(self):
        return self.finished - self.arrival


def test_summarize_percentiles_and_throughput():
    done = [_Req(0.0, 0.001 * (i + 1), 1000) for i in range(100)]
    s = serve.summarize(done, 0.0)
    assert s["requests"] == 100
    assert math.isclose(s["p50_ms"], 50.0) and math.isclose(s["p99_ms"], 99.0)
    assert math.isclose(s["mpix_per_s"], 100 * 1000 / 0.1 / 1e6)


def test_poisson_offsets_are_increasing_with_the_right_rate():
    reqs = serve.random_requests(2000, 8, seed=0, rate=500.0)
    t = [r.arrival for r in reqs]
    assert all(b > a for a, b in zip(t, t[1:]))
    assert 0.8 * 500 < len(t) / t[-1] < 1.2 * 500
    assert {(r.W, r.H) for r in reqs} == set(serve.SERVE_RES)
    assert all(0 <= r.scene < 8 for r in reqs)


def test_byte_estimates_grow_with_work():
    assert serve.n_bytes(2_000_000) > serve.n_bytes(200_000) > 0
    assert serve.k_bytes(10_000_000, 1920, 1080) > serve.k_bytes(10_000, 512, 512) > 0
