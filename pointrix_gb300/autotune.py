"""Run-time choice of the blend kernels' variant (per-block splat batch,
and for the backward the pixels per thread).

The blend kernels stage a tile's depth-sorted splats into shared memory in
batches; the best batch size depends on the image, the channel count and how
many splats a tile's list holds (short lists waste a large batch's staging,
long lists pay a small batch's extra barriers).  The backward also comes
with two or four pixels per thread (four: half the per-splat warp reductions
per pixel, coarser culling boxes).  The library compiles a few variants
(``pgb_blend_batches``: forward 64/128 records per batch, backward 64/128/256
with two pixels per thread and 4096 + 64/128 with four); all give the same
images, and the backward the same gradients up to the order of its float
sums.  On the first call of a workload class this module times
every compiled batch on the live inputs (CUDA events, one warm-up and two
timed runs each) and keeps the fastest for the class; later calls -- and
calls while a CUDA graph is being captured -- use the kept choice (or the
default before any).  ``PGB_AUTOTUNE=0`` in the environment disables timing
(the default batch is used).  ``PGB_AUTOTUNE_CACHE=<file>`` keeps the
choices in a JSON file: read on first use, rewritten after every new choice,
so a later process (a profiler run, a restarted trainer) takes the same
variants without timing them again.  ``PGB_BLEND_VARIANT=fwd=<b>,bwd=<b>``
pins the variant of every class of that kernel (e.g. ``fwd=128,bwd=4160``:
forward 128-record batches, backward four pixels per thread with 64-record
batches), so that a run -- a profile, a comparison -- is reproducible
without any cache file; a pinned value the build does not compile is
ignored.

A class is (kernel, channel count, log2 of the pixel count, log2 of the
mean list length per tile): the quantities that move the optimum.
"""
from __future__ import annotations

import json
import math
import os
import threading
import warnings

import torch

__all__ = ["choose", "workload_class", "table", "timings", "reset", "set_enabled",
           "set_cache_file", "set_pins", "timing_in_this_thread"]

_lock = threading.Lock()
_cache: dict = {}
_times: dict = {}
_enabled = os.environ.get("PGB_AUTOTUNE", "1") != "0"
_cache_file = os.environ.get("PGB_AUTOTUNE_CACHE") or None
_loaded = False


def _parse_pins(text: str) -> dict:
    pins = {}
    for part in (text or "").split(","):
        name, _, val = part.partition("=")
        name = name.strip()
        if name in ("fwd", "bwd") and val.strip().lstrip("-").isdigit():
            pins["blend_" + name] = int(val)
    return pins


_pins = _parse_pins(os.environ.get("PGB_BLEND_VARIANT", ""))
_thread = threading.local()


def timing_in_this_thread(flag: bool) -> None:
    """Allow (True) or forbid (False) timing runs in the calling thread only:
    a thread that serves requests must not stall on a first-seen class (it
    then uses the kept choice of the class, or the default)."""
    _thread.enabled = bool(flag)


def _key_str(key) -> str:
    return "/".join(map(str, key))


def _load_locked() -> None:
    global _loaded
    if _loaded or not _cache_file:
        return
    _loaded = True
    try:
        with open(_cache_file) as f:
            saved = json.load(f)
    except (OSError, ValueError):
        return
    for k, b in (saved.items() if isinstance(saved, dict) else ()):
        try:
            kind, *rest = str(k).split("/")
            _cache.setdefault((kind, *map(int, rest)), int(b))
        except (TypeError, ValueError):
            continue  # an entry this version cannot read: that class is timed again


def _save_locked() -> None:
    # a temporary file of this process and thread, renamed over the cache, so
    # that processes sharing one cache file never see half a file
    if not _cache_file:
        return
    tmp = f"{_cache_file}.{os.getpid()}.{threading.get_ident()}.tmp"
    try:
        with open(tmp, "w") as f:
            json.dump({_key_str(k): b for k, b in _cache.items()}, f)
        os.replace(tmp, _cache_file)
    except OSError as e:
        # the file only spares later processes the timing runs
        warnings.warn(f"autotune cache {_cache_file} not written: {e}", RuntimeWarning)
        try:
            os.remove(tmp)
        except OSError:
            pass


def workload_class(kind: str, channels: int, pixels: int, entries: int, tiles: int) -> tuple:
    """The cache key of a blend call."""
    per_tile = entries / max(tiles, 1)
    return (kind, int(channels), int(math.log2(max(pixels, 1))), int(math.log2(per_tile + 1)))


def _cuda_timer(fn, device) -> float:
    stream = torch.cuda.current_stream(device)
    fn()  # warm-up
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / 2.0


def choose(key, candidates, run, device=None, timer=None) -> int:
    """The batch for ``key``: the cached choice, else (when enabled and not
    capturing) the fastest of ``candidates`` timed with ``run(batch)``, else
    0 (the library default).  A cached choice that is not among
    ``candidates`` (a cache file from a build with other variants) is not
    used."""
    pin = _pins.get(key[0]) if key else None
    if pin is not None and pin in candidates:
        return pin
    with _lock:
        _load_locked()
        hit = _cache.get(key)
    if hit is not None and hit in candidates:
        return hit
    capturing = torch.cuda.is_available() and torch.cuda.is_current_stream_capturing()
    if not getattr(_thread, "enabled", _enabled) or capturing or not candidates:
        return 0
    timer = timer or (lambda fn: _cuda_timer(fn, device))
    times = {b: timer(lambda b=b: run(b)) for b in candidates}
    best = min(times, key=lambda b: (times[b], b))
    with _lock:
        _times.setdefault(key, times)
        if _cache.get(key) not in candidates:  # keep a valid choice another thread made
            _cache[key] = best
        _save_locked()
        return _cache[key]


def table() -> dict:
    """The kept choices (class -> batch)."""
    with _lock:
        return dict(_cache)


def timings() -> dict:
    """The measured milliseconds per candidate of every timed class."""
    with _lock:
        return {k: dict(v) for k, v in _times.items()}


def reset() -> None:
    with _lock:
        _cache.clear()
        _times.clear()


def set_cache_file(path) -> None:
    """Keep the choices in ``path`` (None: in memory only); loads it now."""
    global _cache_file, _loaded
    with _lock:
        _cache_file = os.fspath(path) if path else None
        _loaded = False
        _load_locked()


def set_pins(text: str) -> None:
    """Pins as in ``PGB_BLEND_VARIANT`` ("" clears them)."""
    global _pins
    _pins = _parse_pins(text)


def set_enabled(flag: bool) -> None:
    global _enabled
    _enabled = bool(flag)
