"""The multi-process path of bench.py on CPU: two ranks over gloo on
127.0.0.1 (torch's launcher, as the GPU runs use it with NCCL).  Covers the
rendezvous, the barrier and the max-over-ranks step time that every rank
prints nothing but rank 0 reports, and the reference arm under the launcher:
rank 0 alone runs the oracle and prints the one JSON line."""
import json
import os
import re
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _launch(args, timeout=600):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}"] + args
    env = dict(os.environ, PYTHONPATH=str(ROOT), OMP_NUM_THREADS="2")
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)


def test_two_gloo_ranks_barrier_and_max(tmp_path):
    script = tmp_path / "ranks.py"
    script.write_text(
        "import torch\n"
        "import bench\n"
        "world, rank, local = bench.dist_env()\n"
        "assert world == 2\n"
        "bench.dist_init(world, 'gloo')\n"
        "bench.barrier(world)\n"
        "v = bench.max_over_ranks(float(rank + 1), world, torch.device('cpu'))\n"
        "bench.barrier(world)\n"
        "print(f'rank {rank} max {v}', flush=True)\n"
        "torch.distributed.destroy_process_group()\n")
    r = _launch([str(script)])
    assert r.returncode == 0, r.stderr[-2000:]
    # the two ranks share the launcher's stdout: their lines may interleave
    found = sorted(re.findall(r"rank (\d) max ([0-9.]+)", r.stdout))
    assert found == [("0", "2.0"), ("1", "2.0")], r.stdout


def test_reference_arm_prints_once_under_the_launcher(tmp_path):
    # bench's options go through a wrapper: the launcher's own parser would
    # take "--n" for an abbreviation of its options
    script = tmp_path / "ref.py"
    script.write_text(
        "import runpy, sys\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--gpus', '2', '--n', '3000',\n"
        "            '--steps', '1', '--warmup', '0']\n"
        f"runpy.run_path({str(ROOT / 'bench.py')!r}, run_name='__main__')\n")
    r = _launch([str(script)])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
