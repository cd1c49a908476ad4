"""Continuous-batching render server over resident scenes.

The reference's only serving-like loop is the web viewer, which renders one
camera at a time and synchronises after each (``pointrix/webgui/gui.py:
162-211``).  This module keeps several scenes' Gaussians resident in HBM and
serves forward-only render requests of mixed sizes concurrently:

* requests waiting for the same scene are batched: up to ``max_batch`` of
  them (any mix of image sizes) become one job whose views are projected in
  one kernel, sorted in one view-batch sort (16 x 32 tiles) and blended in
  one launch (``pointrix_gb300.multiview``), each view's image then copied
  to pinned host memory;
* each job is a small state machine on its own CUDA stream -- stage A
  enqueues the colour, the projection and the depth phase of the sort and
  starts a non-blocking read-back of the entry count K; stage B (once K is on
  the host and the K-sized sort/blend buffers fit) enqueues the tile sort,
  the blend and the copies;
* one scheduler thread admits waiting requests as stream slots and device
  memory free up, advances every job whose previous stage has completed
  (event queries, never a blocking sync), and retires finished ones -- so
  requests that arrive while others are on the GPU join immediately, and
  their work overlaps on the device;
* admission is by the bytes actually free on the device (free device memory
  plus what the caching allocator holds unused), less a safety margin,
  optionally capped by ``memory_budget``: a job starts when its N-sized
  working set fits, and its K-sized sort and blend buffers must fit before
  stage B.

A view's image does not depend on the other views of its batch or on what
else is running (the batched kernels give each view exactly the lists,
order and arithmetic of rendering it alone), so a result is the same alone
and in the mix (``tests/test_gpu_serve.py``).
"""
from __future__ import annotations

import math
import queue
import statistics
import threading
import time
from dataclasses import dataclass

import torch

from . import autotune, ops

TILE = 16


def _indexed(device) -> torch.device:
    dev = torch.device(device)
    if dev.type == "cuda" and dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


# ---------------------------------------------------------------------------
# scenes and requests
# ---------------------------------------------------------------------------
class ResidentScene:
    """Activated Gaussian parameters kept on the device (forward only)."""

    def __init__(self, position, scaling, rotation, opacity, shs, device="cuda"):
        dev = torch.device(device)
        self.position = position.detach().to(dev).float().contiguous()
        self.scaling = scaling.detach().to(dev).float().contiguous()
        self.rotation = rotation.detach().to(dev).float().contiguous()
        self.opacity = opacity.detach().to(dev).float().reshape(-1, 1).contiguous()
        self.shs = shs.detach().to(dev).float().contiguous()        # [N,K,3]
        self.n = self.position.shape[0]

    @property
    def nbytes(self) -> int:
        return sum(t.numel() * 4 for t in (self.position, self.scaling, self.rotation,
                                            self.opacity, self.shs))

    def opacity_views(self, V: int) -> torch.Tensor:
        """The opacities repeated for a batch of V views [V*N] (kept: the
        scene is resident and read-only)."""
        cache = self.__dict__.setdefault("_op_views", {})
        t = cache.get(V)
        if t is None:
            t = cache[V] = self.opacity.reshape(1, self.n).expand(V, self.n).reshape(-1).contiguous()
        return t


@dataclass
class RenderRequest:
    """One view of one resident scene.  ``extr`` is world->camera [4,4] (or
    [3,4]), ``intr`` is (fx, fy, cx, cy)."""
    scene: int
    W: int
    H: int
    intr: torch.Tensor
    extr: torch.Tensor
    center: torch.Tensor
    bg: float = 0.0
    rid: int = -1
    arrival: float = 0.0           # host perf_counter time the request arrived
    started: float = 0.0           # admitted (stage A enqueued)
    stage_b: float = 0.0           # K known, stage B enqueued (server paths)
    finished: float = 0.0          # result on the host
    image: torch.Tensor | None = None   # [3,H,W] float32, pinned host memory
    error: str | None = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival

    @property
    def pixels(self) -> int:
        return self.W * self.H


def n_bytes(n: int) -> int:
    """Device bytes a request holds per resident Gaussian through stage A and
    the blend: directions and colour (24), uv/depth/cov3d/conic/radius/tiles
    (68), sort phase-one scratch (28), blend record (48 for 3 channels)."""
    return n * (24 + 68 + 28 + 48)


def k_bytes(k: int, W: int, H: int) -> int:
    """Device bytes of the K-sized sort buffers and the image of stage B."""
    T = ((W + TILE - 1) // TILE) * ((H + TILE - 1) // TILE)
    return k * (16 + 4) + 2 * 3 * k // 4096 * 1024 + T * 8 + W * H * (3 * 4 + 8)


# ---------------------------------------------------------------------------
# the plain pipeline (one request; msplat's operators, as render_iter chains
# them) and the batched pipeline of the server
# ---------------------------------------------------------------------------
def _stage_a(scene: ResidentScene, req: RenderRequest):
    """Per-Gaussian operators and the depth phase of the sort, on the
    current stream.  Returns the tensors stage B needs."""
    dev = scene.position.device
    intr = req.intr.to(dev, non_blocking=True).reshape(4)
    extr = req.extr.to(dev, non_blocking=True)[:3, :].contiguous()
    center = req.center.to(dev, non_blocking=True).reshape(1, 3)
    d = scene.position - center
    d = d / d.norm(dim=1, keepdim=True)
    rgb = (ops.compute_sh(scene.shs.permute(0, 2, 1), d) + 0.5).clamp(min=0.0)
    uv, depth = ops.project_point(scene.position, intr, extr, req.W, req.H)
    vis = depth != 0
    cov = ops.compute_cov3d(scene.scaling, scene.rotation, vis)
    conic, radius, tiles = ops.ewa_project(scene.position, cov, intr, extr, uv, req.W, req.H, vis)
    handle = ops.sort_gaussian_begin(uv, depth, req.W, req.H, radius, tiles)
    return {"uv": uv, "conic": conic, "rgb": rgb, "handle": handle}


def _stage_b(scene: ResidentScene, req: RenderRequest, st: dict, pinned=None) -> torch.Tensor:
    """Tile sort and blend, then the image to pinned host memory."""
    ids, rng = st["handle"].finish()
    img = ops.alpha_blending(st["uv"], st["conic"], scene.opacity, st["rgb"], ids, rng, req.bg,
                             req.W, req.H)
    host = pinned.take(tuple(img.shape)) if pinned is not None else \
        torch.empty(img.shape, dtype=torch.float32, pin_memory=True)
    host.copy_(img, non_blocking=True)
    return host


BATCH_TILE_HEIGHT = 32


def _batch_a(scene: ResidentScene, reqs):
    """Stage A of a batch of views of one scene (current stream): every
    view's colour in one pass over the SH coefficients, every view's
    projection in one kernel, the depth phase of the views' sort."""
    from . import fused, multiview

    dev = scene.position.device
    n, V = scene.n, len(reqs)
    sizes = [(r.W, r.H) for r in reqs]
    intrs = torch.stack([r.intr.to(dev, non_blocking=True).reshape(4) for r in reqs])
    extrs = torch.stack([r.extr.to(dev, non_blocking=True)[:3, :] for r in reqs])
    centres = torch.stack([r.center.to(dev, non_blocking=True).reshape(3) for r in reqs])
    if fused.sh_rgb_supported(scene.shs):
        rgb = fused.sh_rgb_views(scene.shs, scene.position, centres).reshape(V * n, 3)
    else:
        rgbs = []
        for c in centres:
            d = scene.position - c.reshape(1, 3)
            d = d / d.norm(dim=1, keepdim=True)
            rgbs.append((ops.compute_sh(scene.shs.permute(0, 2, 1), d) + 0.5).clamp(min=0.0))
        rgb = torch.cat(rgbs)
    uv, depth, conic, radius, tiles = fused.preprocess_views(scene.position, scene.scaling,
                                                             scene.rotation, intrs, extrs, sizes)
    handle = multiview.sort_views_begin(uv, depth, radius, tiles, sizes, n,
                                        tile_height=BATCH_TILE_HEIGHT)
    return {"uv": uv, "conic": conic, "rgb": rgb, "radius": radius, "handle": handle,
            "sizes": sizes}


def _batch_b(scene: ResidentScene, reqs, st: dict, pinned=None):
    """Stage B of a batch: the views' tile sort and one blend launch, then
    each view's image to pinned host memory (from ``pinned``, a
    :class:`PinnedPool`, when given)."""
    from . import multiview

    n, V = scene.n, len(reqs)
    ids, rng = st["handle"].finish()
    op_all = scene.opacity_views(V)
    imgs = multiview.blend_views(st["uv"], st["conic"], op_all, st["rgb"], ids, rng, reqs[0].bg,
                                 st["sizes"], n, tile_height=BATCH_TILE_HEIGHT,
                                 radius=st["radius"])
    hosts = []
    for img in imgs:
        host = pinned.take(tuple(img.shape)) if pinned is not None else \
            torch.empty(img.shape, dtype=torch.float32, pin_memory=True)
        host.copy_(img, non_blocking=True)
        hosts.append(host)
    return hosts


class PinnedPool:
    """Pinned host image buffers by shape, handed out for results and taken
    back when the client has released its image (page-locking new host
    memory takes milliseconds, so a server recycles its result buffers).
    Thread-safe; the servers share one pool per process, so buffers a server
    (or a warm-up) page-locked serve the next one."""

    def __init__(self):
        self.free: dict = {}
        self._lock = threading.Lock()

    def take(self, shape):
        with self._lock:
            lst = self.free.get(tuple(shape))
            if lst:
                return lst.pop()
        return torch.empty(shape, dtype=torch.float32, pin_memory=True)

    def give(self, t):
        with self._lock:
            self.free.setdefault(tuple(t.shape), []).append(t)


_SHARED_PINNED = PinnedPool()


@torch.no_grad()
def render_plain(scene: ResidentScene, req: RenderRequest, pinned=None) -> torch.Tensor:
    """One request, synchronously, on the current stream (the plain path)."""
    st = _stage_a(scene, req)
    host = _stage_b(scene, req, st, pinned)
    torch.cuda.current_stream(scene.position.device).synchronize()
    return host


class _Job:
    """A batch of requests (one scene) in flight: stream slot, stage,
    reserved bytes."""

    __slots__ = ("reqs", "scene", "stream", "stage", "st", "hosts", "event", "reserved")

    def __init__(self, reqs, scene, stream):
        self.reqs, self.scene, self.stream = reqs, scene, stream
        self.stage, self.st, self.hosts, self.event, self.reserved = "A", None, None, None, 0


def batch_k_bytes(k: int, sizes) -> int:
    """Device bytes of a batch's K-sized sort buffers and images (stage B)."""
    T = sum(((W + TILE - 1) // TILE) * ((H + 2 * TILE - 1) // (2 * TILE)) for W, H in sizes)
    return k * (16 + 4) + 2 * 3 * k // 4096 * 1024 + T * 8 + sum(W * H for W, H in sizes) * (3 * 4 + 8)


# The servers' job streams, one list per device, shared by every server on
# it: the caching allocator keeps freed device memory per stream, so a
# server (or a warm-up) that used these streams leaves their pools warm for
# the next; a fresh stream would allocate anew in the middle of its first
# burst of requests.
_JOB_STREAMS: dict = {}
_JOB_STREAMS_LOCK = threading.Lock()


def _job_streams(device: torch.device, slots: int) -> list:
    with _JOB_STREAMS_LOCK:
        lst = _JOB_STREAMS.setdefault(device, [])
        while len(lst) < slots:
            lst.append(torch.cuda.Stream(device))
        return lst[:slots]


class RenderServer:
    """Continuous-batching server: see the module docstring.

    ``slots`` bounds the jobs in flight (one CUDA stream each); a job
    beyond the first starts only when at least ``backlog`` requests are
    waiting -- overlapping jobs on the device slows each of them and adds
    allocations on a second stream, which pays only when requests queue up
    (measured at 100-500 req/s: a backlog of 2 put the p99 at 2-8x the
    one-at-a-time path's; 8 keeps it near that path's and still overlaps
    jobs under overload);
    ``max_batch`` the requests of one scene batched into a job;
    ``memory_budget`` (None: no cap beyond the free device memory) caps the
    bytes the jobs' working sets may hold; ``reserve`` bytes of free device
    memory are left untouched.  Submit requests with :meth:`submit`
    (thread-safe); completed requests come back through ``on_done`` (called
    on the scheduler thread) and from :meth:`close`."""

    def __init__(self, scenes, slots: int = 2, memory_budget: int | None = None, device="cuda",
                 on_done=None, max_batch: int = 16, reserve: int = 1 << 30, backlog: int = 8):
        self.scenes = scenes
        self.device = _indexed(device)
        self.streams = _job_streams(self.device, slots)
        self.free_streams = list(range(slots))
        self.budget = None if memory_budget is None else int(memory_budget)
        self.reserve = int(reserve)
        self.max_batch = max(1, int(max_batch))
        self.in_use = 0
        self.inbox: "queue.Queue[RenderRequest | None]" = queue.Queue()
        self.waiting: list[RenderRequest] = []
        self.active: list[_Job] = []
        self.done: list[RenderRequest] = []
        self.batches: list[int] = []        # size of every job started
        self.backlog = max(1, int(backlog))
        self.pinned = _SHARED_PINNED
        self.on_done = on_done
        self._closed = False
        self._thread = threading.Thread(target=self._loop, name="pgb-render-server", daemon=True)
        self._error: BaseException | None = None
        self._thread.start()

    # -- client side ------------------------------------------------------
    def submit(self, req: RenderRequest) -> None:
        if self._closed:
            raise RuntimeError("RenderServer is closed")
        if not (0 <= req.scene < len(self.scenes)):
            raise ValueError(f"no resident scene {req.scene}")
        if req.arrival == 0.0:
            req.arrival = time.perf_counter()
        self.inbox.put(req)

    def close(self, timeout: float | None = None) -> list[RenderRequest]:
        """Stop accepting requests, finish those in flight, return all done."""
        self._closed = True
        self.inbox.put(None)
        self._thread.join(timeout)
        if self._error is not None:
            raise RuntimeError("render server failed") from self._error
        return self.done

    # -- scheduler --------------------------------------------------------
    def _fits(self, need: int) -> bool:
        """Whether ``need`` more bytes fit: the device's free memory plus what
        the caching allocator holds unused, less the reserve, and the
        optional budget."""
        if self.budget is not None and self.in_use + need > self.budget:
            return False
        free, _ = torch.cuda.mem_get_info(self.device)
        cached = torch.cuda.memory_reserved(self.device) - torch.cuda.memory_allocated(self.device)
        return need <= free + cached - self.reserve

    def _admit(self):
        while self.waiting and self.free_streams:
            if self.active and len(self.waiting) < self.backlog:
                return                                 # no queue: no overlap
            first = self.waiting[0]
            group = [first] + [r for r in self.waiting[1:]
                               if r.scene == first.scene and r.bg == first.bg][:self.max_batch - 1]
            scene = self.scenes[first.scene]
            need = n_bytes(scene.n) * len(group)
            if self.active and not self._fits(need):
                return                                 # wait for memory to free up
            ids = {id(r) for r in group}
            self.waiting = [r for r in self.waiting if id(r) not in ids]
            job = _Job(group, scene, self.streams[self.free_streams.pop()])
            job.reserved = need
            self.in_use += need
            now = time.perf_counter()
            for r in group:
                r.started = now
            with torch.cuda.stream(job.stream):
                job.st = _batch_a(scene, group)
            self.active.append(job)
            self.batches.append(len(group))

    def _advance(self) -> bool:
        progressed = False
        still = []
        for job in self.active:
            if job.stage == "A" and job.st["handle"].ready():
                K = job.st["handle"].count()
                need = batch_k_bytes(K, job.st["sizes"])
                in_b = any(j.stage == "B" for j in self.active)
                if in_b and not self._fits(need):
                    still.append(job)                  # wait for a stage-B job to retire
                    continue
                job.reserved += need
                self.in_use += need
                now = time.perf_counter()
                for r in job.reqs:
                    r.stage_b = now
                with torch.cuda.stream(job.stream):
                    job.hosts = _batch_b(job.scene, job.reqs, job.st, self.pinned)
                    job.event = torch.cuda.Event()
                    job.event.record(job.stream)
                job.stage = "B"
                progressed = True
                still.append(job)
            elif job.stage == "B" and job.event.query():
                now = time.perf_counter()
                for req, host in zip(job.reqs, job.hosts):
                    req.image = host
                    req.finished = now
                    self.done.append(req)
                    if self.on_done is not None:
                        self.on_done(req)
                        if req.image is None:          # the client took it: recycle
                            self.pinned.give(host)
                job.st = None
                self.in_use -= job.reserved
                self.free_streams.append(self.streams.index(job.stream))
                ops._drain_pending(block=False)
                progressed = True
            else:
                still.append(job)
        self.active = still
        return progressed

    def _wait_first(self):
        job = self.active[0]
        ev = job.st["handle"].h.event if job.stage == "A" else job.event
        if ev is not None:
            ev.synchronize()

    def _loop(self):
        try:
            torch.cuda.set_device(self.device)
            # no autotuner timing runs on the serving thread: a first-seen
            # workload class would stall every request in flight
            autotune.timing_in_this_thread(False)
            closing = False
            with torch.no_grad():
                while True:
                    # take every request that has arrived; block briefly when idle
                    try:
                        item = self.inbox.get(timeout=0.0005 if not (self.active or self.waiting) else 0.0)
                        while True:
                            if item is None:
                                closing = True
                            else:
                                self.waiting.append(item)
                            item = self.inbox.get_nowait()
                    except queue.Empty:
                        pass
                    self._admit()
                    if not self._advance() and self.active:
                        if not self.waiting and self.inbox.empty():
                            # nothing to admit: wait for the first job's
                            # current stage on its event (the wait releases
                            # the GIL and wakes as soon as the stage ends)
                            self._wait_first()
                        else:
                            time.sleep(0)    # yield (the GIL too), then poll again
                    if closing and not self.active and not self.waiting:
                        break
        except BaseException as e:  # surfaced by close()
            self._error = e


class PlainServer:
    """One request at a time, synchronously, in arrival order: the viewer's
    loop (``pointrix/webgui/gui.py:162-211``) as a server."""

    def __init__(self, scenes, device="cuda", on_done=None):
        self.scenes = scenes
        self.device = _indexed(device)
        self.inbox: "queue.Queue[RenderRequest | None]" = queue.Queue()
        self.done: list[RenderRequest] = []
        self.on_done = on_done
        self.pinned = _SHARED_PINNED
        self._thread = threading.Thread(target=self._loop, name="pgb-plain-server", daemon=True)
        self._error: BaseException | None = None
        self._thread.start()

    def submit(self, req: RenderRequest) -> None:
        if req.arrival == 0.0:
            req.arrival = time.perf_counter()
        self.inbox.put(req)

    def close(self, timeout=None):
        self.inbox.put(None)
        self._thread.join(timeout)
        if self._error is not None:
            raise RuntimeError("plain server failed") from self._error
        return self.done

    def _loop(self):
        try:
            torch.cuda.set_device(self.device)
            autotune.timing_in_this_thread(False)    # as the continuous server
            while True:
                req = self.inbox.get()
                if req is None:
                    break
                req.started = time.perf_counter()
                host = render_plain(self.scenes[req.scene], req, self.pinned)
                req.image = host
                req.finished = time.perf_counter()
                self.done.append(req)
                if self.on_done is not None:
                    self.on_done(req)
                    if req.image is None:
                        self.pinned.give(host)
        except BaseException as e:
            self._error = e


# ---------------------------------------------------------------------------
# load generation and statistics
# ---------------------------------------------------------------------------
SERVE_RES = ((512, 512), (800, 800), (1280, 720), (1920, 1080))


def serving_scenes(seed: int = 5, count: int = 8, n_min: int = 200_000, n_max: int = 2_000_000,
                   device="cuda"):
    """``count`` resident SH-3 scenes, Gaussian counts log-uniform in
    [n_min, n_max], the distributions of the training workload."""
    from .workloads import scene_sh3

    g = torch.Generator().manual_seed(seed)
    out = []
    for i in range(count):
        u = float(torch.rand(1, generator=g))
        n = int(round(math.exp(math.log(n_min) + u * (math.log(n_max) - math.log(n_min)))))
        s = scene_sh3(seed * 100 + i, n)
        pos, sc, q, op, shs = s.activated()
        out.append(ResidentScene(pos, sc, q, op, shs, device))
    return out


def random_requests(count: int, n_scenes: int, seed: int = 0, rate: float | None = None):
    """Requests for a random scene, a camera at radius U[3,6] looking at the
    origin, a resolution from SERVE_RES (focal 0.8 W); with ``rate``, Poisson
    arrival offsets (seconds) in ``req.arrival``."""
    from .workloads import make_camera

    g = torch.Generator().manual_seed(seed)
    reqs, t = [], 0.0
    for i in range(count):
        scene = int(torch.randint(0, n_scenes, (1,), generator=g))
        W, H = SERVE_RES[int(torch.randint(0, len(SERVE_RES), (1,), generator=g))]
        radius = 3.0 + 3.0 * float(torch.rand(1, generator=g))
        cam = make_camera(g, W, H, 0.8 * W, radius)
        pin = (lambda t: t.pin_memory()) if torch.cuda.is_available() else (lambda t: t)
        r = RenderRequest(scene, W, H, pin(cam.intr.reshape(4)), pin(cam.extr), pin(cam.center),
                          rid=i)
        if rate:
            t += float(torch.empty(1).exponential_(rate, generator=g))
            r.arrival = t
        reqs.append(r)
    return reqs


def drive(server, requests) -> float:
    """Submits ``requests`` at their Poisson offsets (``req.arrival``,
    relative) from the calling thread; returns the start time."""
    offsets = [r.arrival for r in requests]
    t0 = time.perf_counter()
    for r, off in zip(requests, offsets):
        now = time.perf_counter() - t0
        if off > now:
            time.sleep(off - now)
        r.arrival = t0 + off
        server.submit(r)
    return t0


def summarize(done, t0: float) -> dict:
    lat = sorted(r.latency for r in done)
    if not lat:
        return {"requests": 0}
    span = max(r.finished for r in done) - t0
    q = lambda p: lat[min(len(lat) - 1, int(math.ceil(p * len(lat))) - 1)]
    return {
        "requests": len(done),
        "p50_ms": 1e3 * q(0.50),
        "p99_ms": 1e3 * q(0.99),
        "mean_ms": 1e3 * statistics.mean(lat),
        "mpix_per_s": sum(r.pixels for r in done) / span / 1e6,
        "req_per_s": len(done) / span,
    }
