"""Continuous-batching render server over resident scenes.

The reference's only serving-like loop is the web viewer, which renders one
camera at a time and synchronises after each (``pointrix/webgui/gui.py:
162-211``).  This module keeps several scenes' Gaussians resident in HBM and
serves forward-only render requests of mixed sizes concurrently:

* each request is a small state machine on its own CUDA stream -- stage A
  enqueues the per-Gaussian operators and the depth phase of the sort and
  starts a non-blocking read-back of the entry count K; stage B (once K is on
  the host and the K-sized sort/blend buffers fit the memory budget)
  enqueues the tile sort, the blend and the copy of the image to pinned host
  memory;
* one scheduler thread admits waiting requests as stream slots and memory
  free up, advances every request whose previous stage has completed (event
  queries, never a blocking sync), and retires finished ones -- so requests
  that arrive while others are on the GPU join immediately and their work
  overlaps on the device;
* admission is by bytes: a request is started when its N-sized working set
  fits the budget, and its K-sized sort and blend buffers are reserved
  before stage B.

Every request runs exactly the operators of the plain path on the same
inputs, and no kernel of the forward path depends on what else is running,
so a result is the same alone and in the mix (``tests/test_gpu_serve.py``).
"""
from __future__ import annotations

import math
import queue
import statistics
import threading
import time
from dataclasses import dataclass

import torch

from . import ops

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
# the per-request pipeline (same operators as the plain path)
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


def _stage_b(scene: ResidentScene, req: RenderRequest, st: dict) -> torch.Tensor:
    """Tile sort and blend, then the image to pinned host memory."""
    ids, rng = st["handle"].finish()
    img = ops.alpha_blending(st["uv"], st["conic"], scene.opacity, st["rgb"], ids, rng, req.bg,
                             req.W, req.H)
    host = torch.empty(img.shape, dtype=torch.float32, pin_memory=True)
    host.copy_(img, non_blocking=True)
    return host


@torch.no_grad()
def render_plain(scene: ResidentScene, req: RenderRequest) -> torch.Tensor:
    """One request, synchronously, on the current stream (the plain path)."""
    st = _stage_a(scene, req)
    host = _stage_b(scene, req, st)
    torch.cuda.current_stream(scene.position.device).synchronize()
    return host


class _Job:
    """A request in flight: stream slot, stage, reserved bytes."""

    __slots__ = ("req", "scene", "stream", "stage", "st", "host", "event", "reserved")

    def __init__(self, req, scene, stream):
        self.req, self.scene, self.stream = req, scene, stream
        self.stage, self.st, self.host, self.event, self.reserved = "A", None, None, None, 0


class RenderServer:
    """Continuous-batching server: see the module docstring.

    ``slots`` bounds the requests in flight (one CUDA stream each);
    ``memory_budget`` bounds the bytes their working sets may hold.
    Submit requests with :meth:`submit` (thread-safe); completed requests
    come back through ``on_done`` (called on the scheduler thread) and from
    :meth:`close`."""

    def __init__(self, scenes, slots: int = 8, memory_budget: int = 8 << 30, device="cuda",
                 on_done=None):
        self.scenes = scenes
        self.device = _indexed(device)
        self.streams = [torch.cuda.Stream(self.device) for _ in range(slots)]
        self.free_streams = list(range(slots))
        self.budget = int(memory_budget)
        self.in_use = 0
        self.inbox: "queue.Queue[RenderRequest | None]" = queue.Queue()
        self.waiting: list[RenderRequest] = []
        self.active: list[_Job] = []
        self.done: list[RenderRequest] = []
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
    def _admit(self):
        while self.waiting and self.free_streams:
            req = self.waiting[0]
            need = n_bytes(self.scenes[req.scene].n)
            if self.active and self.in_use + need > self.budget:
                return                                 # wait for memory to free up
            self.waiting.pop(0)
            job = _Job(req, self.scenes[req.scene], self.streams[self.free_streams.pop()])
            job.reserved = need
            self.in_use += need
            req.started = time.perf_counter()
            with torch.cuda.stream(job.stream):
                job.st = _stage_a(job.scene, req)
            self.active.append(job)

    def _advance(self) -> bool:
        progressed = False
        still = []
        for job in self.active:
            req = job.req
            if job.stage == "A" and job.st["handle"].ready():
                K = job.st["handle"].count()
                need = k_bytes(K, req.W, req.H)
                in_b = any(j.stage == "B" for j in self.active)
                if in_b and self.in_use + need > self.budget:
                    still.append(job)                  # wait for a stage-B job to retire
                    continue
                job.reserved += need
                self.in_use += need
                with torch.cuda.stream(job.stream):
                    job.host = _stage_b(job.scene, req, job.st)
                    job.event = torch.cuda.Event()
                    job.event.record(job.stream)
                job.stage = "B"
                progressed = True
                still.append(job)
            elif job.stage == "B" and job.event.query():
                req.image = job.host
                req.finished = time.perf_counter()
                job.st = None
                self.in_use -= job.reserved
                self.free_streams.append(self.streams.index(job.stream))
                self.done.append(req)
                ops._drain_pending(block=False)
                if self.on_done is not None:
                    self.on_done(req)
                progressed = True
            else:
                still.append(job)
        self.active = still
        return progressed

    def _loop(self):
        try:
            torch.cuda.set_device(self.device)
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
                        time.sleep(20e-6)
                    if closing and not self.active and not self.waiting:
                        break
        except BaseException as e:  # surfaced by close()
            self._error = e


class PlainServer:
    """One request at a time, synchronously, in arrival order: the viewer's
    loop (``pointrix/webgui/gui.py:162-211``) as a server."""

    def __init__(self, scenes, device="cuda"):
        self.scenes = scenes
        self.device = _indexed(device)
        self.inbox: "queue.Queue[RenderRequest | None]" = queue.Queue()
        self.done: list[RenderRequest] = []
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
            while True:
                req = self.inbox.get()
                if req is None:
                    break
                req.started = time.perf_counter()
                req.image = render_plain(self.scenes[req.scene], req)
                req.finished = time.perf_counter()
                self.done.append(req)
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
