"""Host logic of the blend batch autotuner (no GPU: a fake timer)."""
from pointrix_gb300 import autotune


def test_choose_times_once_and_caches():
    autotune.reset()
    calls = []
    cost = {64: 3.0, 128: 1.0, 256: 2.0}

    def run(b):
        calls.append(b)

    def timer(fn):
        fn()
        return cost[calls[-1]]

    key = autotune.workload_class("blend_bwd", 7, 1600 * 1060, 16_600_000, 6700)
    assert autotune.choose(key, (64, 128, 256), run, timer=timer) == 128
    assert calls == [64, 128, 256]
    assert autotune.choose(key, (64, 128, 256), run, timer=timer) == 128
    assert calls == [64, 128, 256]          # cached: no more timing
    assert autotune.table()[key] == 128
    autotune.reset()


def test_classes_and_disable():
    k1 = autotune.workload_class("blend_fwd", 7, 1600 * 1060, 16_600_000, 6700)
    k2 = autotune.workload_class("blend_fwd", 7, 1600 * 1060, 1_000_000, 6700)
    assert k1 != k2                           # list length per tile moves the class
    autotune.set_enabled(False)
    try:
        assert autotune.choose(k1, (64, 128), lambda b: None, timer=lambda fn: 1.0) == 0
    finally:
        autotune.set_enabled(True)
        autotune.reset()


def test_cache_file_round_trip(tmp_path):
    path = tmp_path / "tune.json"
    autotune.reset()
    autotune.set_cache_file(path)
    try:
        key = autotune.workload_class("blend_fwd", 7, 1600 * 1060, 16_600_000, 6700)
        assert autotune.choose(key, (64, 128), lambda b: None,
                               timer=lambda fn: 1.0) == 64  # tie: the smaller
        autotune.reset()
        autotune.set_cache_file(path)      # a new process: choices come back untimed
        assert autotune.choose(key, (64, 128), lambda b: None,
                               timer=lambda fn: (_ for _ in ()).throw(AssertionError)) == 64
    finally:
        autotune.set_cache_file(None)
        autotune.reset()
