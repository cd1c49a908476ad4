#!/usr/bin/env python
"""Benchmark of the msplat training step on GB300.

Workload (the headline configuration): one training step of a single view --
1,000,000 Gaussians with SH degree 3, one 1600x1060 camera (focal 1150 px,
radius 5), forward RGB + depth + normal (7 channels), loss L1 + 0.2 * L2
against a fixed random target, backward to every Gaussian parameter and to
the camera extrinsic (6-DoF quaternion + translation) and intrinsics.  Data
are seeded synthetic tensors with the stated distributions.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  ``value`` is training iterations per second with the
scene resident in HBM (device-timed with CUDA events) of the step captured
once as a CUDA graph and replayed (``pointrix_gb300.graph.GraphedStep``: the
sort keeps K on the device, Adam keeps its step counts there);
``eager_ms_per_step`` is the same step launched call by call, which also
gives the per-operator times.  ``e2e`` is the same metric through the same
calls with the per-step camera and target image copied in from pinned host
memory and the loss read back every step.  ``--impl reference`` times the CPU float64 rendition of the same step
(the oracle: the reference operator backend itself is absent) on a bounded
sample of tiles, on all host cores.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import torch  # noqa: E402

METRIC = "train iters/s & Mpix/s at 1M Gaussians SH3; serve p50/p99 ms vs plain path"
WORKLOAD = ("single-view training step: 1,000,000 Gaussians SH3, 1600x1060, RGB+depth+normal "
            "(7 ch), L1+0.2*L2, grads to all Gaussian params + camera extrinsic/intrinsics, Adam step")
PEAKS_FALLBACK = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000, help="Gaussians (workload default 1M)")
    ap.add_argument("--cpu-budget", type=float, default=150.0,
                    help="seconds of full CPU steps the reference arm may spend (at least one step)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving p50/p99 leg")
    ap.add_argument("--no-multiview", action="store_true",
                    help="skip the 16-view batched-vs-per-view leg")
    ap.add_argument("--no-recompute", action="store_true",
                    help="skip the 6M-Gaussian 4K stored-vs-recompute leg")
    ap.add_argument("--no-ssim", action="store_true",
                    help="skip the fused-vs-torch SSIM loss leg")
    return ap.parse_args()


# ----------------------------------------------------------------- dist ---
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_init(world, backend):
    if world > 1 and not torch.distributed.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.distributed.init_process_group(backend)


def barrier(world):
    if world > 1:
        torch.distributed.barrier()


def max_over_ranks(x, world, device):
    if world == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------- clocks ---
class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None
        self.marks = {}

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def mark(self, name):
        """Records the host time of an event (the timed region's start and end)."""
        self.marks[name] = time.time()

    def summary(self):
        """Median SM clock and the throttle reasons seen over the sampled
        window.  The caller keeps the GPU loaded for the whole window (the
        timed region is ~40 ms, shorter than nvidia-smi's start-up), and
        `in_region` counts the samples stamped between the marks."""
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                stamp = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((float(parts[2]), float(parts[3]), parts[6:10], stamp))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, flags, _ in rows for i, f in enumerate(flags) if f == "Active"})
        t0, t1 = self.marks.get("start"), self.marks.get("end")
        inside = [r for r in rows if t0 is not None and t1 is not None and t0 - 0.02 <= r[3] <= t1 + 0.02]
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "in_region": len(inside),
                "window_s": round(rows[-1][3] - rows[0][3], 3)}


def keep_busy(fn, device, seconds):
    """Replays `fn` for about `seconds` of wall time."""
    t_end = time.perf_counter() + seconds
    while time.perf_counter() < t_end:
        for _ in range(20):
            fn()
        torch.cuda.synchronize(device)


# ------------------------------------------------------------- workload ---
def quat_to_rot(q):
    from pointrix_gb300.workloads import rotation_from_unit_quat
    return rotation_from_unit_quat(q / q.norm())


def rot_to_quat(R):
    R = R.double()
    w = torch.sqrt(torch.clamp(1 + R[0, 0] + R[1, 1] + R[2, 2], min=1e-12)) / 2
    x = (R[2, 1] - R[1, 2]) / (4 * w)
    y = (R[0, 2] - R[2, 0]) / (4 * w)
    z = (R[1, 0] - R[0, 1]) / (4 * w)
    return torch.stack([w, x, y, z]).float()


class CameraParams:
    """Differentiable camera: wxyz quaternion + translation (6-DoF) and
    intrinsics, assembled into the world->camera matrix each step."""

    def __init__(self, cam, device, grad=True):
        self.W, self.H = cam.W, cam.H
        self.q = rot_to_quat(cam.extr[:3, :3]).to(device).requires_grad_(grad)
        self.t = cam.extr[:3, 3].clone().to(device).requires_grad_(grad)
        self.intr = cam.intr.clone().to(device).requires_grad_(grad)
        self.bottom = torch.tensor([[0.0, 0, 0, 1]], device=device)

    def pose(self, fused=True):
        """(world->camera [4,4], camera centre [3]) from the 6-DoF leaves: one
        library kernel each way (``fused.camera_pose``), or the torch
        composition with the same arithmetic."""
        if fused and self.q.is_cuda:
            from pointrix_gb300 import fused as FU
            return FU.camera_pose(self.q, self.t)
        R = quat_to_rot(self.q)
        E = torch.cat([torch.cat([R, self.t[:, None]], 1), self.bottom], 0)
        return E, -(R.T @ self.t)

    def leaves(self):
        return [self.q, self.t, self.intr]


def training_step(renderer, scene, camp, target, WL, optimizer=None, fused=True):
    """Gradients to None, forward, L1 + 0.2 L2 loss, backward, and (when
    given) the Adam step.  ``fused``: the parameter activations + normal and
    the loss each as one library kernel (same arithmetic as the torch
    composition, which ``fused=False`` runs)."""
    if optimizer is not None:
        optimizer.zero_grad(set_to_none=True)
    if fused:
        from pointrix_gb300 import fused as FU
        sc, q, op, normal = FU.gaussian_activations(scene.log_scale, scene.quat_raw,
                                                    scene.opacity_logit)
        pos, shs = scene.position, scene.shs
    else:
        pos, sc, q, op, shs = scene.activated()
        normal = WL.normals_from_scene(sc, q)
    E, center = camp.pose(fused)
    out = renderer.render_iter(camp.H, camp.W, E, camp.intr, center,
                               pos, op, sc, q, shs, extra_features={"normal": normal})
    if fused:
        loss = FU.l1_l2_loss(out["rendered_features"], target, 0.2)
    else:
        F = torch.nn.functional
        f = out["rendered_features_split"]
        img = torch.cat([f["rgb"], f["depth"], f["normal"]], 0)
        loss = F.l1_loss(img, target) + 0.2 * F.mse_loss(img, target)
    loss.backward()
    if optimizer is not None:
        optimizer.step()
    return loss


def make_optimizer(scene, camp, capturable=False):
    """Adam with 3DGS-style per-group learning rates over every Gaussian
    parameter and the camera pose/intrinsics (one kernel launch per step;
    two with device-side step counts for graph capture)."""
    groups = [
        {"params": [scene.position], "lr": 1.6e-4},
        {"params": [scene.log_scale], "lr": 5e-3},
        {"params": [scene.quat_raw], "lr": 1e-3},
        {"params": [scene.opacity_logit], "lr": 5e-2},
        {"params": [scene.shs], "lr": 2.5e-3},
        {"params": [camp.q, camp.t], "lr": 1e-4},
        {"params": [camp.intr], "lr": 1e-3},
    ]
    from pointrix_gb300.optim import Adam

    return Adam(groups, eps=1e-15, capturable=capturable)


def count_entries(scene, camp, W, H):
    """K: the (Gaussian, tile) entries of the current scene and camera."""
    from pointrix_gb300 import ops
    with torch.no_grad():
        pos, sc, q, op, shs = scene.activated()
        E = camp.pose()[0][:3]
        uv, depth = ops.project_point(pos, camp.intr, E, W, H)
        vis = depth != 0
        cov = ops.compute_cov3d(sc, q, vis)
        conic, radius, tiles = ops.ewa_project(pos, cov, camp.intr, E, uv, W, H, vis)
        return int(tiles[radius > 0].sum())


def zero_grads(tensors):
    for t in tensors:
        t.grad = None


# ----------------------------------------------- algorithmic bytes/unit ---
def blend_fwd_bytes(n, C, K, T, W, H):
    """Inputs and outputs of one alpha_blending forward, each once: per
    Gaussian uv 8 + conic 12 + opacity 4 + C features; per list entry a 4 B
    id; per tile an 8 B range; per pixel C outputs + final T + n_contrib."""
    return n * (24 + 4 * C) + 4 * K + 8 * T + W * H * (4 * C + 8)


def blend_bwd_bytes(n, C, K, T, W, H):
    """The forward's record (read) and the gradient outputs per Gaussian, ids,
    ranges, and per pixel dL/dout + final T + n_contrib."""
    rec = 4 * (16 if C <= 10 else 32)
    return n * (rec + 24 + 4 * C) + 4 * K + 8 * T + W * H * (4 * C + 8)


def sort_bytes(n, K, T):
    """Depth sort of N (key,value) pairs in four 8-bit passes, emission of K
    pairs, tile sort in ceil(log2 T / 8) passes, range pass."""
    passes = 1 if T <= 256 else 2
    return n * (12 + 4 * 16) + n * 28 + K * 8 + passes * K * 16 + K * 4 + T * 8


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    except Exception:
        return PEAKS_FALLBACK, "fallback"


# ------------------------------------------------------ CPU (the oracle) ---
CPU_LRS = (1.6e-4, 5e-3, 1e-3, 5e-2, 2.5e-3, 1e-4, 1e-4, 1e-3)   # as make_optimizer


class CpuStep:
    """The training step in float64 on the host cores with the oracle's
    operators: activations and normal, camera pose from its quaternion and
    translation, SH colour, projection, covariance, EWA, the sort, blending
    forward and backward over every tile, L1 + 0.2 L2 on all seven channels,
    the backward to every Gaussian parameter and the camera, and the Adam
    step (torch.optim.Adam, float64).  Nothing is sampled or scaled."""

    def __init__(self, scene, cam, target, threads):
        from pointrix_gb300 import workloads as WL

        self.WL = WL
        self.threads = threads
        torch.set_num_threads(threads)
        dt = torch.float64
        self.leaves = [t.detach().to(dt).clone().requires_grad_(True) for t in
                       (scene.position, scene.log_scale, scene.quat_raw, scene.opacity_logit,
                        scene.shs)]
        self.camq = rot_to_quat(cam.extr[:3, :3]).to(dt).requires_grad_(True)
        self.camt = cam.extr[:3, 3].to(dt).clone().requires_grad_(True)
        self.intr = cam.intr.to(dt).clone().requires_grad_(True)
        self.W, self.H = cam.W, cam.H
        self.target = target.to(dt)
        params = self.leaves + [self.camq, self.camt, self.intr]
        self.opt = torch.optim.Adam([{"params": [p], "lr": lr} for p, lr in zip(params, CPU_LRS)],
                                    eps=1e-15)
        # the blend's worker processes, started once (not part of a step);
        # list capacity from the entries of the initial parameters
        from oracle import msplat_cpu as O
        from oracle.blend_pool import BlendPool
        with torch.no_grad():
            pos = self.leaves[0]
            R = WL.rotation_from_unit_quat(self.camq / self.camq.norm())
            extr = torch.cat([R, self.camt[:, None]], 1)
            uv, depth = O.project_point(pos, self.intr, extr, cam.W, cam.H, nearest=0.2)
            sc = torch.exp(self.leaves[1])
            q = self.leaves[2] / self.leaves[2].norm(dim=1, keepdim=True)
            cov = O.compute_cov3d(sc, q, depth != 0)
            _, radius, nt = O.ewa_project(pos, cov, self.intr, extr, uv, cam.W, cam.H, depth != 0)
            K = int(nt[radius > 0].sum())
        self.pool = BlendPool(pos.shape[0], 7, int(1.3 * K) + 65536, cam.W, cam.H, self.target,
                              workers=threads, scale=1.0 / self.target.numel())

    def close(self):
        self.pool.close()

    def run(self):
        """One step; returns (seconds, details)."""
        from oracle import msplat_cpu as O

        WL = self.WL
        W, H = self.W, self.H
        t0 = time.perf_counter()
        self.opt.zero_grad(set_to_none=True)
        pos, logs, qr, opl, shs = self.leaves
        sc = torch.exp(logs)
        q = qr / qr.norm(dim=1, keepdim=True)
        op = torch.sigmoid(opl)
        R = WL.rotation_from_unit_quat(self.camq / self.camq.norm())
        extr = torch.cat([R, self.camt[:, None]], 1)
        center = -(R.T @ self.camt)
        d = pos - center[None]
        d = d / d.norm(dim=1, keepdim=True)
        rgb = (O.compute_sh(shs.permute(0, 2, 1), d) + 0.5).clamp(min=0)
        uv, depth = O.project_point(pos, self.intr, extr, W, H, nearest=0.2)
        vis = depth != 0
        cov = O.compute_cov3d(sc, q, vis)
        conic, radius, ntiles = O.ewa_project(pos, cov, self.intr, extr, uv, W, H, vis)
        normal = WL.normals_from_scene(sc, q)
        feat = torch.cat([rgb, depth, normal], 1)
        t1 = time.perf_counter()
        ids, rng = O.sort_gaussian(uv.detach(), depth.detach(), W, H, radius, ntiles)
        t2 = time.perf_counter()
        # blend forward and backward tile by tile (bounded memory), the
        # tiles spread over worker processes on the host cores; then the
        # chain's backward
        loss, gu, gc, go, gf = self.pool.run(uv, conic, op, feat, ids, rng)
        t3 = time.perf_counter()
        torch.autograd.backward([uv, conic, op, feat], [gu, gc, go, gf])
        t4 = time.perf_counter()
        self.opt.step()
        t5 = time.perf_counter()
        return t5 - t0, {"preprocess_fwd_s": t1 - t0, "sort_s": t2 - t1,
                         "blend_fwd_bwd_s": t3 - t2, "chain_backward_s": t4 - t3, "adam_s": t5 - t4, "K": int(ids.numel()),
                         "tiles": int(rng.shape[0]), "loss": float(loss)}


def cpu_timed_steps(args, budget_s):
    """Full float64 CPU steps of the workload: one warm-up step when
    ``args.warmup`` > 0, then timed steps until ``args.steps`` are done or
    the next would end past ``budget_s`` (at least one).  Returns (mean s per
    step, steps timed, warm-up steps run, threads, details of the last)."""
    from pointrix_gb300 import workloads as WL

    scene, cam = WL.scene_train_view(1, n=args.n)
    g = torch.Generator().manual_seed(7)
    target = torch.rand(7, cam.H, cam.W, generator=g)
    threads = len(os.sched_getaffinity(0))
    step = CpuStep(scene, cam, target, threads)
    try:
        t_start = time.perf_counter()
        warm = 0
        if args.warmup > 0:
            step.run()
            warm = 1
        times, det = [], {}
        while len(times) < max(1, args.steps):
            s, det = step.run()
            times.append(s)
            if time.perf_counter() - t_start + statistics.mean(times) > budget_s:
                break
    finally:
        step.close()
    return statistics.mean(times), len(times), warm, threads, det


def cpu_sample_string(n, steps, warm):
    return (f"float64 oracle training step on the host cores, all {n} Gaussians and all tiles "
            f"(nothing sampled or scaled): activations, camera pose, SH colour, projection, EWA, "
            f"sort, blend fwd+bwd over every tile, L1+0.2*L2, backward, Adam; "
            f"{steps} timed full step(s) after {warm} warm-up step(s)")


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    sec, steps, warm, threads, det = cpu_timed_steps(args, budget_s=args.cpu_budget)
    value = 1.0 / sec
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warm, "steps_requested": args.steps,
        "warmup_requested": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "gaussians": args.n, "width": 1600, "height": 1060,
                   "channels": 7, "sh_degree": 3, "parallelism": "cpu, host cores"},
        "cpu_baseline": {"value": value, "unit": "iters/s", "cores": threads, "kind": "port",
                         "sample": cpu_sample_string(args.n, steps, warm), "detail": det},
        "e2e": {"value": value, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# ------------------------------------------------------ batched multi-view ---
MULTIVIEW_WORKLOAD = ("batched multi-view: 3,000,000 Gaussians SH3, 16 views on a radius-5 sphere, "
                      "resolutions from 640x480/1280x720/1600x1060/1920x1080, RGB+depth, L1 loss, "
                      "forward+backward for all views")


def multiview_measure(device, n=3_000_000, views=16, steps=20):
    """Mpix/s of the batched forward+backward over all views -- one sort and
    one blend launch each way for the whole batch, the step captured once as
    a CUDA graph and replayed -- against the per-view loop of plain launches
    (MsplatRender.render_batch's order, a host read of K per view).  Both
    compute the same images (the largest difference is reported)."""
    from pointrix_gb300 import fused, multiview, ops
    from pointrix_gb300 import workloads as WL
    from pointrix_gb300.graph import GraphedStep
    from pointrix_gb300.renderer import MsplatRender

    scene = WL.scene_sh3(3, n).to(device).leaves()
    cams = [c.to(device) for c in WL.cameras_multiview(2, views)]
    g = torch.Generator().manual_seed(33)
    targets = [torch.rand(4, c.H, c.W, generator=g).to(device) for c in cams]
    pix = sum(c.W * c.H for c in cams)
    params = [scene.position, scene.log_scale, scene.quat_raw, scene.opacity_logit, scene.shs]
    r = MsplatRender(MsplatRender.Config(render_depth=True), device=device)
    r.sh_degree = 3
    F = torch.nn.functional
    last = {}

    def per_view():
        zero_grads(params)
        pos, sc, q, op, shs = scene.activated()
        loss, imgs = 0.0, []
        for cam, tgt in zip(cams, targets):
            out = r.render_iter(cam.H, cam.W, cam.extr, cam.intr, cam.center, pos, op, sc, q, shs)
            img = out["rendered_features"]
            imgs.append(img)
            loss = loss + F.l1_loss(img, tgt)
        loss.backward()
        last["per_view"] = [i.detach() for i in imgs]   # no autograd graph kept alive

    cap = {}

    def batched():
        zero_grads(params)
        pos, sc, q, op, shs = scene.activated()
        imgs, _, _ = multiview.render_views(pos, sc, q, op, shs, cams, capacity=cap.get("k"),
                                            tile_height=cap.get("th", 16))
        loss = fused.l1_l2_loss(imgs[0], targets[0], 0.0)
        for img, tgt in zip(imgs[1:], targets[1:]):
            loss = loss + fused.l1_l2_loss(img, tgt, 0.0)
        loss.backward()
        last["batched"] = [i.detach() for i in imgs]
        return loss

    def timed(fn):
        """Per-step latency of ``steps`` steps (each bracketed by
        synchronisations), after one untimed step."""
        fn()
        torch.cuda.synchronize(device)
        times = []
        for _ in range(steps):
            torch.cuda.synchronize(device)
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize(device)
            times.append(1e3 * (time.perf_counter() - t0))
        ms = statistics.mean(times)
        q = sorted(times)
        return {"ms_per_step": ms, "mpix_per_s": pix / (ms * 1e-3) / 1e6, "steps": steps,
                "p50_ms": statistics.median(q), "p99_ms": q[min(len(q) - 1, int(0.99 * len(q)))],
                "max_ms": q[-1]}

    res = {"per_view_loop": timed(per_view)}
    per_view_imgs = [t.detach().clone() for t in last["per_view"]]
    k_batch = multiview_k(scene, cams)
    # the tile shape is tuned by timing the whole batched step with each
    # (the per-block splat batches are tuned by the blend autotuner inside)
    shapes, diffs, ks = {}, {}, {}
    for th in multiview.TILE_HEIGHTS:
        ks[th] = multiview_k(scene, cams, th)
        cap["k"] = int(1.15 * ks[th]) + (1 << 20)
        cap["th"] = th
        graphed = GraphedStep(batched, warmup=1, device=device)
        shapes[f"16x{th}"] = timed(graphed)
        ops.check_device_status(device)
        diffs[f"16x{th}"] = max(float((a - b).abs().max())
                                for a, b in zip(per_view_imgs, last["batched"]))
        del graphed
        torch.cuda.empty_cache()
    best = min(shapes, key=lambda k: shapes[k]["ms_per_step"])
    res["batched_graph"] = shapes[best]
    res["speedup"] = res["per_view_loop"]["ms_per_step"] / res["batched_graph"]["ms_per_step"]
    return {"workload": MULTIVIEW_WORKLOAD, "pixels_per_step": pix, "K_entries": k_batch,
            "K_entries_by_tile": {f"16x{th}": k for th, k in ks.items()},
            "max_abs_image_diff": max(diffs.values()), "image_diff_by_tile": diffs,
            "tile_shape": best, "by_tile_shape": shapes, **res}


def multiview_k(scene, cams, tile_height=16):
    """Total (element, tile) entries of a batch of views for 16 x
    ``tile_height`` tiles."""
    from pointrix_gb300 import multiview, ops
    total = 0
    with torch.no_grad():
        pos, sc, q, op, shs = scene.activated()
        for cam in cams:
            E = cam.extr[:3]
            uv, depth = ops.project_point(pos, cam.intr, E, cam.W, cam.H)
            vis = depth != 0
            cov = ops.compute_cov3d(sc, q, vis)
            _, radius, tiles = ops.ewa_project(pos, cov, cam.intr, E, uv, cam.W, cam.H, vis)
            if tile_height != 16:
                tiles = multiview.tile_counts_views(uv, radius, [(cam.W, cam.H)], pos.shape[0],
                                                    tile_height)
            total += int(tiles[radius > 0].sum())
    return total


# --------------------------------------------------------------- SSIM loss ---
def ssim_measure(device, C=3, H=1060, W=1600, reps=10):
    """Fused SSIM forward+backward against the torch composition of
    pointrix/model/loss.py:ssim (conv2d with the 11x11 window), same image."""
    import math
    from pointrix_gb300 import fused
    F = torch.nn.functional
    g = torch.Generator(device=device).manual_seed(0)
    y = torch.rand(C, H, W, device=device, generator=g)
    x = (y + 0.1 * torch.randn(C, H, W, device=device, generator=g)).clamp(0, 1).requires_grad_(True)
    w1 = torch.tensor([math.exp(-(k - 5) ** 2 / (2 * 1.5 ** 2)) for k in range(11)], device=device)
    w1 = w1 / w1.sum()
    win = (w1[:, None] @ w1[None, :])[None, None].expand(C, 1, 11, 11).contiguous()

    def torch_ssim(a, b):
        conv = lambda t: F.conv2d(t[None], win, padding=5, groups=C)  # noqa: E731
        mu1, mu2 = conv(a), conv(b)
        s11, s22, s12 = conv(a * a) - mu1 ** 2, conv(b * b) - mu2 ** 2, conv(a * b) - mu1 * mu2
        m = ((2 * mu1 * mu2 + 1e-4) * (2 * s12 + 9e-4)) / ((mu1 ** 2 + mu2 ** 2 + 1e-4) * (s11 + s22 + 9e-4))
        return m.mean()

    res = {"workload": f"SSIM loss forward+backward, {C}x{H}x{W}"}
    vals = {}
    for name, fn in (("torch", torch_ssim), ("fused", fused.ssim)):
        for _ in range(3):
            x.grad = None
            fn(x, y).backward()
        torch.cuda.synchronize(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            x.grad = None
            v = fn(x, y)
            v.backward()
        e1.record()
        torch.cuda.synchronize(device)
        res[f"{name}_ms"] = e0.elapsed_time(e1) / reps
        vals[name] = (float(v.detach()), x.grad.detach().clone())
    res["value_abs_diff"] = abs(vals["fused"][0] - vals["torch"][0])
    gt = vals["torch"][1]
    res["grad_rel_max"] = float((vals["fused"][1] - gt).abs().max() / gt.abs().max())
    return res


# -------------------------------------------------------- recompute mode ---
RECOMPUTE_WORKLOAD = ("memory-bound differentiation: 6,000,000 Gaussians SH3, one 3840x2160 view, "
                      "focal 2800, radius 5, RGB+depth, L1 loss, backward to all Gaussian params")


def recompute_measure(device, n=6_000_000, steps=3):
    """Stored vs recompute-in-backward: step time, peak HBM, memory held from
    forward to backward, and gradient agreement between the two modes."""
    from pointrix_gb300 import workloads as WL
    from pointrix_gb300.renderer import MsplatRender

    scene = WL.scene_sh3(4, n).to(device).leaves()
    g = torch.Generator().manual_seed(44)
    cam = WL.make_camera(g, 3840, 2160, 2800.0, 5.0).to(device)
    target = torch.rand(4, cam.H, cam.W, generator=g).to(device)
    from pointrix_gb300 import ops
    res, grads = {}, {}
    K = count_entries_cam(scene, cam)
    modes = {"stored": (False, 0), "recompute": (True, 0), "recompute_4_bands": (True, 4)}
    for name, (mode, bands) in modes.items():
        r = MsplatRender(MsplatRender.Config(render_depth=True, recompute_backward=mode,
                                             recompute_bands=bands), device=device)
        r.sh_degree = 3
        params = [scene.position, scene.log_scale, scene.quat_raw, scene.opacity_logit, scene.shs]
        times, held = [], 0
        for it in range(steps + 1):
            zero_grads(params)
            torch.cuda.synchronize(device)
            torch.cuda.reset_peak_memory_stats(device)
            base = torch.cuda.memory_allocated(device)
            t0 = time.perf_counter()
            pos, sc, q, op, shs = scene.activated()
            out = r.render_iter(cam.H, cam.W, cam.extr, cam.intr, cam.center, pos, op, sc, q, shs)
            f = out["rendered_features_split"]
            loss = torch.nn.functional.l1_loss(torch.cat([f["rgb"], f["depth"]], 0), target)
            torch.cuda.synchronize(device)
            held = torch.cuda.memory_allocated(device) - base
            loss.backward()
            torch.cuda.synchronize(device)
            if it > 0:
                times.append(time.perf_counter() - t0)
        peak = torch.cuda.max_memory_allocated(device) - base
        grads[name] = [p.grad.detach().clone() for p in params]
        res[name] = {"ms_per_step": 1e3 * statistics.mean(times), "peak_gb": peak / 1e9,
                     "held_fwd_to_bwd_gb": held / 1e9}
        if mode:
            res[name]["bands"] = len(ops.last_band_plan)
            res[name]["max_band_entries"] = max(k for _, _, k in ops.last_band_plan)
    rel = {name: max(float((a - b).norm() / b.norm().clamp(min=1e-30))
                     for a, b in zip(grads[name], grads["stored"])) for name in modes if name != "stored"}
    return {"workload": RECOMPUTE_WORKLOAD, "K_entries": K, **res,
            "grad_rel_l2_max": max(rel.values()), "grad_rel_l2": rel}


def count_entries_cam(scene, cam):
    """K of a scene for a fixed camera (cam.extr [4,4], cam.intr)."""
    from pointrix_gb300 import ops
    with torch.no_grad():
        pos, sc, q, op, shs = scene.activated()
        E = cam.extr[:3]
        uv, depth = ops.project_point(pos, cam.intr, E, cam.W, cam.H)
        vis = depth != 0
        cov = ops.compute_cov3d(sc, q, vis)
        conic, radius, tiles = ops.ewa_project(pos, cov, cam.intr, E, uv, cam.W, cam.H, vis)
        return int(tiles[radius > 0].sum())


# --------------------------------------------------------------- serving ---
SERVE_WORKLOAD = ("serving: 8 resident SH3 scenes, N log-uniform in [200k, 2M], forward RGB, "
                  "Poisson arrivals, camera radius U[3,6], 512^2/800^2/1280x720/1920x1080")


def serve_measure(device, rates=(50, 100, 200, 500, 1000, 2000), duration=10.0):
    """p50/p99 latency and Mpix/s of the continuous-batching server against
    the one-request-at-a-time plain path, per Poisson arrival rate
    (``duration`` seconds of arrivals per rate and server; every request is
    served and counted, including the backlog after the arrivals stop)."""
    from pointrix_gb300 import serve

    scenes = serve.serving_scenes(device=device)
    # warm-up of both paths: a burst (the large batches of the high rates)
    # and two seconds of paced arrivals (the one- to three-view jobs of the
    # low rates), so no measured rate is the first to run a code path
    for cls in (serve.PlainServer, serve.RenderServer):
        srv = cls(scenes)
        for r in serve.random_requests(64, len(scenes), seed=99):
            srv.submit(r)
        srv.close()
        srv = cls(scenes, on_done=_drop_image)
        serve.drive(srv, serve.random_requests(200, len(scenes), seed=98, rate=100))
        srv.close()
    out = []
    for rate in rates:
        row = {"rate_req_per_s": rate}
        for name, cls in (("plain", serve.PlainServer), ("continuous", serve.RenderServer)):
            reqs = serve.random_requests(int(rate * duration), len(scenes), seed=rate, rate=rate)
            # the client takes each image as it arrives (the host buffers of
            # tens of thousands of results are not kept)
            srv = cls(scenes, on_done=_drop_image)
            t0 = serve.drive(srv, reqs)
            stats = serve.summarize(srv.close(), t0)
            if name == "continuous" and srv.batches:
                stats["mean_batch"] = statistics.mean(srv.batches)
                stats["max_batch"] = max(srv.batches)
            row[name] = {k: round(v, 3) if isinstance(v, float) else v for k, v in stats.items()}
        out.append(row)
    return {"workload": SERVE_WORKLOAD, "duration_s": duration, "rates": out}


def _drop_image(req):
    req.image = None


def serve_summary(serving):
    """Compact per-rate line for the end of the bench output: p50/p99 ms and
    Mpix/s of the plain path and the continuous-batching server."""
    if not serving:
        return None
    out = {}
    for row in serving["rates"]:
        p, c = row["plain"], row["continuous"]
        out[str(row["rate_req_per_s"])] = {
            "plain_p50_p99_ms": [p.get("p50_ms"), p.get("p99_ms")], "plain_mpix_s": p.get("mpix_per_s"),
            "cont_p50_p99_ms": [c.get("p50_ms"), c.get("p99_ms")], "cont_mpix_s": c.get("mpix_per_s"),
            "cont_mean_batch": c.get("mean_batch")}
    return out


# ------------------------------------------------------------ roofline ---
# FP32 operations per composited (pixel, splat) pair, C channels (an FMA
# counts two).  Forward: dy, the base-2 power (two FMAs), alpha = min(0.99,
# o 2^p), T (1 - alpha), alpha T, C feature FMAs: 9 + 2C.  Backward: dy,
# power, g0 and g1 (two FMAs), alpha, 1 - alpha, T / (1 - alpha), F = sum
# dout f (C FMAs), the feature gradients (C FMAs), dalpha, the SB update,
# dpow and the six moment FMAs: 35 + 4C.  The exponential is on the SFU and
# not counted.
def fwd_flop_per_pair(C):
    return 9 + 2 * C


def bwd_flop_per_pair(C):
    return 35 + 4 * C


def fp32_peak_tflops(sm_mhz):
    """152 SMs x 128 FP32 lanes x 2 (FMA) at the given SM clock."""
    return 152 * 128 * 2 * sm_mhz * 1e6 / 1e12


def issue_peak(sm_mhz):
    """Warp instructions per second: 152 SMs x 4 schedulers x 1 per cycle."""
    return 152 * 4 * sm_mhz * 1e6


def blend_census(scene, camp, W, H):
    """(evaluated, composited) (pixel, splat) pairs of the step's blend, on
    the device (``ops.blend_pair_census``), outside the timed region."""
    from pointrix_gb300 import ops
    with torch.no_grad():
        pos, sc, q, op, shs = scene.activated()
        E = camp.pose()[0][:3]
        uv, depth = ops.project_point(pos, camp.intr, E, W, H)
        vis = depth != 0
        cov = ops.compute_cov3d(sc, q, vis)
        conic, radius, tiles = ops.ewa_project(pos, cov, camp.intr, E, uv, W, H, vis)
        ids, rng = ops.sort_gaussian(uv, depth, W, H, radius, tiles)
        feat = torch.zeros(pos.shape[0], 7, device=pos.device)
        return ops.blend_pair_census(uv, conic, op, feat, ids, rng, W, H)


def hbm_bytes(n, K, T, W, H, params):
    """Algorithmic bytes per launch of the HBM-streaming kernels of the step
    (each input and output once; n Gaussians, K list entries, T tiles)."""
    pix = W * H
    passes = 1 if T <= 256 else 2
    return {
        "gaussian_activate_fwd": 76 * n, "gaussian_activate_bwd": 108 * n,
        "sh_rgb_fwd": 216 * n, "sh_rgb_bwd": 420 * n,
        "preprocess_fwd": 72 * n, "preprocess_bwd": 104 * n,
        "sort_begin": n * (12 + 8 + 4 * 16),
        "sort_finish": n * 28 + K * (8 + passes * 16 + 4) + T * 8,
        # the loss forward also writes the gradient for dL = 1, so its
        # backward (dL is 1 in the step) reads one scalar and returns
        "l1_l2_loss_fwd": 12 * 7 * pix,
        "adam_step": 28 * params,
    }


def blend_roofline(scene, camp, W, H, n, K, T, per_op, clk):
    """The dominant kernel's roofline.  The blend kernels are bound by
    instruction issue and the FP32 pipe, not by HBM (their DRAM traffic is a
    few percent of peak): ``achieved`` is FP32 work per second (composited
    pairs x FLOP per pair / live launch time) against the FP32 peak at the
    measured SM clock; ``issue`` is the warp-instruction rate (instructions
    per launch from the committed ncu capture / live launch time) against
    the issue peak.  ``hbm_kernels`` gives the HBM-streaming kernels against
    the copy bandwidth."""
    peaks, peak_kind = load_peaks()
    hbm_peak = float(peaks.get("hbm_gbs", PEAKS_FALLBACK["hbm_gbs"]))
    mhz = float(clk.get("sm_mhz") or 2070.0)
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
            prof = json.load(f)
    except Exception:
        prof = {}
    traffic = prof.get("bytes_per_launch", {})
    insts = prof.get("warp_instructions_per_launch", {})
    ev, comp = blend_census(scene, camp, W, H)
    fp32_peak = fp32_peak_tflops(mhz)
    kern = {}
    for name, flop in (("alpha_blending_fwd", fwd_flop_per_pair(7)),
                       ("alpha_blending_bwd", bwd_flop_per_pair(7))):
        if name not in per_op:
            continue
        t = per_op[name] * 1e-3
        ach = flop * comp / t / 1e12
        entry = {"launch_ms": per_op[name], "flop_per_composited_pair": flop,
                 "achieved_tflops": ach, "fp32_peak_tflops": fp32_peak, "fp32_frac": ach / fp32_peak,
                 "pairs_per_ns": comp / t * 1e-9, "dram_bytes_per_launch": traffic.get(name)}
        if insts.get(name):
            rate = insts[name] / t
            entry.update({"warp_instructions_per_launch": insts[name],
                          "issue_rate": rate, "issue_peak": issue_peak(mhz),
                          "issue_frac": rate / issue_peak(mhz)})
        kern[name] = entry
    params = sum(p.numel() for p in (scene.position, scene.log_scale, scene.quat_raw,
                                     scene.opacity_logit, scene.shs)) + 11
    hbm = []
    for name, b in hbm_bytes(n, K, T, W, H, params).items():
        if name in per_op:
            gbs = b / (per_op[name] * 1e-3) / 1e9
            hbm.append({"kernel": name, "launch_ms": round(per_op[name], 4), "bytes": b,
                        "achieved_gbs": round(gbs, 1), "frac": round(gbs / hbm_peak, 3)})
    dom = "alpha_blending_bwd" if "alpha_blending_bwd" in kern else next(iter(kern), None)
    d = kern.get(dom, {})
    return {"bound": "fp32/issue", "kernel": dom,
            "achieved": d.get("achieved_tflops"), "peak": fp32_peak, "unit": "TFLOP/s",
            "frac": d.get("fp32_frac"), "traffic": d.get("dram_bytes_per_launch"),
            "peak_source": f"derived: 152 SMs x 128 FP32 lanes x 2 at the measured {mhz:.0f} MHz",
            "issue_frac": d.get("issue_frac"),
            "pairs": {"evaluated": ev, "composited": comp},
            "blend": kern, "hbm_kernels": hbm, "hbm_peak_gbs": hbm_peak, "hbm_peak_source": peak_kind}


# ------------------------------------------------------------- GPU arm ---
class StepState:
    """A copy of everything a training step updates -- the Gaussian and
    camera parameters and Adam's moments and device step counts -- restored
    in place (the captured graph keeps its buffers) before each measured
    phase, so that the eager, graph-replay and end-to-end timings all start
    from the same scene: the scene drifts as it trains, and an unreset run
    would time a different workload in each phase."""

    def __init__(self, scene, camp, optimizer):
        self.tensors = [scene.position, scene.log_scale, scene.quat_raw, scene.opacity_logit,
                        scene.shs, *camp.leaves()]
        for p in list(self.tensors):
            st = optimizer.state.get(p, {})
            self.tensors += [st[k] for k in ("exp_avg", "exp_avg_sq") if k in st]
        for name in ("_count_all", "_steps_dev"):
            t = getattr(optimizer, name, None)
            if t is not None:
                self.tensors.append(t)
        with torch.no_grad():
            self.saved = [t.detach().clone() for t in self.tensors]

    def restore(self):
        with torch.no_grad():
            for t, v in zip(self.tensors, self.saved):
                t.copy_(v)


def run_gb300(args):
    world, rank, local = dist_env()
    dist_init(world, "nccl")
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    from pointrix_gb300 import autotune, ops
    from pointrix_gb300 import workloads as WL
    from pointrix_gb300.graph import GraphedStep
    from pointrix_gb300.renderer import MsplatRender

    scene_cpu, cam = WL.scene_train_view(1, n=args.n)
    scene = scene_cpu.to(device).leaves()
    camp = CameraParams(cam, device)
    g = torch.Generator().manual_seed(7)
    target_cpu = torch.rand(7, cam.H, cam.W, generator=g)
    target = target_cpu.to(device)
    renderer = MsplatRender(MsplatRender.Config(render_depth=True, max_sh_degree=3), device=device)
    renderer.sh_degree = 3
    optimizer = make_optimizer(scene, camp, capturable=True)
    W, H = cam.W, cam.H
    stream = torch.cuda.current_stream(device)

    def step():
        return training_step(renderer, scene, camp, target, WL, optimizer)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize(device)
    # the sort keeps K on the device from here on: lists sized for a capacity
    # above the K of this camera, so that no step synchronises with the host
    renderer.cfg.sort_capacity = int(1.25 * count_entries(scene, camp, W, H)) + 65536
    state = StepState(scene, camp, optimizer)

    # -- eager launches (same kernels as the graph): per-operator CUDA-event
    #    times for the roofline, and the launch count
    barrier(world)
    torch.cuda.synchronize(device)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    state.restore()
    with ops.kernel_timing() as kt:
        start.record(stream)
        for _ in range(args.steps):
            step()
        end.record(stream)
        torch.cuda.synchronize(device)
    eager_ms = max_over_ranks(start.elapsed_time(end) / args.steps, world, device)
    ops.check_device_status(device)

    # -- the step captured once as a CUDA graph and replayed (device-resident
    #    inputs): the headline
    graphed = GraphedStep(step, warmup=2, device=device)
    for _ in range(max(3, args.warmup)):
        graphed()
    state.restore()
    torch.cuda.synchronize(device)
    with ClockSampler(device.index) as clocks:
        # keep the GPU busy while nvidia-smi starts, so that the samples
        # around the short timed region are taken under load
        keep_busy(graphed, device, 0.5)
        state.restore()
        barrier(world)
        torch.cuda.synchronize(device)
        clocks.mark("start")
        start.record(stream)
        for _ in range(args.steps):
            graphed()
        end.record(stream)
        torch.cuda.synchronize(device)
        clocks.mark("end")
        barrier(world)
        keep_busy(graphed, device, 0.25)
    ms = max_over_ranks(start.elapsed_time(end) / args.steps, world, device)
    value = world / (ms / 1e3)
    ops.check_device_status(device)

    # -- end to end through the same public calls, host buffers: each step
    #    copies its camera and target in from pinned memory, replays the step
    #    and reads its loss back.  The copies of step i + 1 run on a copy
    #    stream while step i computes (two staging buffers, event-ordered);
    #    the host reads each step's loss one step later, as a training loop
    #    that logs asynchronously does.  Every copy is inside the timed region.
    state.restore()       # the camera copied in each step is the starting camera
    target_host = target_cpu.pin_memory()
    cam_host = [t.detach().cpu().pin_memory() for t in camp.leaves()]
    h2d = target_host.numel() * 4 + sum(t.numel() * 4 for t in cam_host)
    copy_stream = torch.cuda.Stream(device)
    stage_t = [torch.empty_like(target) for _ in range(2)]
    stage_c = [[torch.empty_like(t) for t in camp.leaves()] for _ in range(2)]
    ready = [torch.cuda.Event() for _ in range(2)]
    free = [torch.cuda.Event() for _ in range(2)]
    loss_host = [torch.empty((), dtype=torch.float32).pin_memory() for _ in range(2)]
    loss_ev = [torch.cuda.Event() for _ in range(2)]
    for b in range(2):
        free[b].record(stream)

    def copy_in(i):
        b = i % 2
        copy_stream.wait_event(free[b])  # step i - 2 has consumed this buffer
        with torch.cuda.stream(copy_stream):
            stage_t[b].copy_(target_host, non_blocking=True)
            for dst, src in zip(stage_c[b], cam_host):
                dst.copy_(src, non_blocking=True)
            ready[b].record(copy_stream)

    state.restore()
    barrier(world)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    copy_in(0)
    for i in range(args.steps):
        b = i % 2
        if i + 1 < args.steps:
            copy_in(i + 1)  # overlaps with step i
        stream.wait_event(ready[b])
        with torch.no_grad():
            target.copy_(stage_t[b], non_blocking=True)
            for dst, src in zip(camp.leaves(), stage_c[b]):
                dst.copy_(src, non_blocking=True)
        free[b].record(stream)
        loss = graphed()
        loss_host[b].copy_(loss.detach(), non_blocking=True)
        loss_ev[b].record(stream)
        if i >= 1:
            loss_ev[(i - 1) % 2].synchronize()  # step i - 1's loss is on the host
    loss_ev[(args.steps - 1) % 2].synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(e2e_s, world, device)
    barrier(world)
    ops.check_device_status(device)

    # -- dominant kernel and its roofline (live CUDA-event durations)
    per_op = {name: statistics.mean(kt.ms(name)) for name in kt.names()}
    state.restore()       # the roofline's counts are taken on the starting scene
    K = count_entries(scene, camp, W, H)
    T = ((W + 15) // 16) * ((H + 15) // 16)
    n = args.n
    clk = clocks.summary()
    roofline = blend_roofline(scene, camp, W, H, n, K, T, per_op, clk)

    serving = recompute = None
    if rank == 0 and not args.no_serve:
        serving = serve_measure(device)
    if rank == 0 and not args.no_recompute:
        recompute = recompute_measure(device)
    multi = None
    if rank == 0 and not args.no_multiview:
        multi = multiview_measure(device)
    loss_ssim = ssim_measure(device) if rank == 0 and not args.no_ssim else None
    if rank == 0:
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            # one full, unsampled float64 step
            cargs = argparse.Namespace(n=n, steps=1, warmup=0)
            sec, steps_c, warm_c, threads, det = cpu_timed_steps(cargs, budget_s=0.0)
            cpu = {"value": 1.0 / sec, "unit": "iters/s", "cores": threads, "kind": "port",
                   "sample": cpu_sample_string(n, steps_c, warm_c), "detail": det}
        line = {
            "metric": METRIC, "value": value, "unit": "iters/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "eager_ms_per_step": eager_ms,
            "config": {"workload": WORKLOAD, "gaussians": n, "width": W, "height": H, "channels": 7,
                       "sh_degree": 3, "K_duplicates": K, "tiles": T,
                       "l2": "inputs larger than L2 (0.31 GB of Gaussian parameters + 47 MB target per step)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "mpix_per_s": value * W * H / 1e6,
            "e2e": {"value": world / e2e_s, "unit": "iters/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": 4,
                    "note": "next step's inputs copied on a copy stream during the current step; "
                            "each loss read back one step later"},
            "roofline": roofline,
            "per_op_ms": {k: round(v, 4) for k, v in per_op.items()},
            "gpu_launches": kt.total_launches(),
            "clocks": clk,
            "cpu_baseline": cpu,
            "serve": serving,
            "recompute": recompute,
            "multiview": multi,
            "ssim": loss_ssim,
            "blend_batch": {"/".join(map(str, k)): b for k, b in autotune.table().items()},
            "blend_batch_ms": {"/".join(map(str, k)): {str(b): round(t, 4) for b, t in v.items()}
                               for k, v in autotune.timings().items()},
            # compact summaries last, where a truncated log still shows them
            "multiview_summary": None if not multi else {
                "tile_shape": multi["tile_shape"], "speedup_vs_per_view_loop": multi["speedup"],
                "batched_p50_p99_ms": [multi["batched_graph"]["p50_ms"], multi["batched_graph"]["p99_ms"]],
                "loop_p50_p99_ms": [multi["per_view_loop"]["p50_ms"], multi["per_view_loop"]["p99_ms"]],
                "max_abs_image_diff": multi["max_abs_image_diff"]},
            "recompute_summary": None if not recompute else {
                k: {"ms": round(v["ms_per_step"], 2), "peak_gb": round(v["peak_gb"], 2)}
                for k, v in recompute.items() if isinstance(v, dict) and "peak_gb" in v},
            "serve_summary": serve_summary(serving),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
