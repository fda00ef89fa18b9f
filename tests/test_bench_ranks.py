"""bench.py's reference arm launched with two ranks (torchrun, CPU only).

The path runs replicas only: under torchrun rank 0 alone times the CPU
restatement of the reference shaders and prints the one JSON line; the
other ranks exit 0 without work.  torchrun sets OMP_NUM_THREADS=1 for every
rank, so rank 0 must take the host's cores itself."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_two_ranks_one_line():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), str(ROOT / "bench.py"),
           "--impl", "reference", "--workload", "plain_small_8x4x8_r128_sdf64", "--steps", "1", "--warmup", "0",
           "--frames-per-step", "8"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["gpu_launches"] == 0
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["cores"] == (os.cpu_count() or 1)
    assert line["config"]["workload"] == "plain_small_8x4x8_r128_sdf64"
