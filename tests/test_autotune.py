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


def test_unreadable_entries_and_stale_choices_are_timed_again(tmp_path):
    import json

    key = autotune.workload_class("blend_bwd", 7, 1600 * 1060, 16_600_000, 6700)
    path = tmp_path / "tune.json"
    # a foreign key, a non-integer choice, and this class holding a variant
    # that the current build does not offer
    path.write_text(json.dumps({"blend_fwd/x/1": 64, "blend_fwd/7/20/1": "big",
                                autotune._key_str(key): 999}))
    autotune.reset()
    autotune.set_cache_file(path)
    try:
        timed = []
        assert autotune.choose(key, (64, 4096 + 64), lambda b: timed.append(b),
                               timer=lambda fn: (fn(), 1.0)[1]) == 64
        assert timed == [64, 4096 + 64]
        assert json.loads(path.read_text())[autotune._key_str(key)] == 64
        # disabled timing with a stale entry: the library default
        autotune.reset()
        autotune.set_cache_file(None)
        autotune._cache[key] = 999
        autotune.set_enabled(False)
        assert autotune.choose(key, (64, 128), lambda b: None) == 0
    finally:
        autotune.set_enabled(True)
        autotune.set_cache_file(None)
        autotune.reset()


def test_unwritable_cache_file_warns_and_still_chooses(tmp_path):
    import pytest

    blocker = tmp_path / "not_a_dir"
    blocker.write_text("")
    autotune.reset()
    autotune.set_cache_file(blocker / "tune.json")  # its parent is a file
    try:
        key = autotune.workload_class("blend_fwd", 3, 640 * 480, 1_000_000, 1200)
        with pytest.warns(RuntimeWarning, match="not written"):
            assert autotune.choose(key, (64, 128), lambda b: None,
                                   timer=lambda fn: 1.0) == 64
        assert autotune.table()[key] == 64
        assert list(tmp_path.iterdir()) == [blocker]   # no temporary file left
    finally:
        autotune.set_cache_file(None)
        autotune.reset()


def test_pins_override_timing_and_cache():
    """PGB_BLEND_VARIANT-style pins take precedence over the cache and the
    timer; a pinned value the build does not compile is ignored."""
    from pointrix_gb300 import autotune as A
    A.reset()
    calls = []
    timer = lambda fn: (calls.append(1), fn())[1]  # noqa: E731
    try:
        A.set_pins("fwd=128,bwd=4160")
        kf = ("blend_fwd", 7, 20, 11)
        kb = ("blend_bwd", 7, 20, 11)
        assert A.choose(kf, [64, 128], lambda b: float(b), timer=timer) == 128
        assert A.choose(kb, [64, 128, 4160], lambda b: float(b), timer=timer) == 4160
        assert calls == []
        A.set_pins("bwd=999")
        assert A.choose(kb, [64, 128], lambda b: float(b), timer=timer) == 64   # timed instead
        assert calls
    finally:
        A.set_pins("")
        A.reset()


def test_timing_can_be_forbidden_in_one_thread():
    """A serving thread turns timing off for itself only: it gets the
    default for a class nobody has timed, other threads still time."""
    import threading
    from pointrix_gb300 import autotune as A
    A.reset()
    got = {}

    def server():
        A.timing_in_this_thread(False)
        got["server"] = A.choose(("blend_fwd", 3, 10, 4), [64, 128], lambda b: float(b),
                                 timer=lambda fn: fn())

    t = threading.Thread(target=server)
    t.start()
    t.join()
    try:
        assert got["server"] == 0
        assert A.choose(("blend_fwd", 3, 10, 4), [64, 128], lambda b: float(b),
                        timer=lambda fn: fn()) == 64
    finally:
        A.reset()
