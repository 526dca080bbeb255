"""Multi-GPU path: replicas only (one independent case per rank, no data exchange).  The
rank logic of bench.py — max over ranks of the timings, whole-job MLUPS, rank 0 alone
printing — is exercised here with world-size-2 gloo process groups on the CPU."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.reduce_max([1.0 + rank, 10.0 - rank, 0.5])
        out.put((rank, got, bench.replica_value(1000, 10, got[0], world)))
    finally:
        dist.destroy_process_group()


def test_reduce_max_and_whole_job_value_with_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, value in res:
        assert got == [2.0, 10.0, 0.5], (rank, got)  # slowest rank's timing, on every rank
        assert value == pytest.approx(2 * 1000 * 10 / 2.0 / 1e6)


def test_reference_arm_prints_once_under_torchrun(built):
    """`bench.py --impl reference` launched like the multi-GPU bench: rank 0 alone measures
    and prints one JSON line; the other rank exits 0 without work."""
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "1", "--size", "32", "--ref-budget", "10"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600,
                       env={**os.environ, "OMP_NUM_THREADS": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["unit"] == "MLUPS"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"


def test_shedding_statistics_of_a_known_signal():
    """bench.shedding_stats on synthetic forces: constant drag plus a sinusoidal lift of known
    amplitude and frequency gives back Cd, rms Cl and St (the C5 workload's statistics); the
    zero-crossing frequency also holds for a window that is not a whole number of periods."""
    import math
    import numpy as np
    sys.path.insert(0, str(ROOT))
    import bench
    d, u, nz, n = 64.0, 0.05, 256, 38400  # second half: exactly 3 shedding periods
    q = 0.5 * u * u * d * nz
    t = np.arange(n)
    st_true = 0.2
    f = st_true * u / d  # shedding frequency per step
    fx = 1.25 * q + 0.0 * t
    fy = 0.3 * q * np.sin(2 * math.pi * f * t)
    cd, cl_rms, st = bench.shedding_stats(fx, fy, d, u, nz)
    assert abs(cd - 1.25) < 1e-12
    assert abs(cl_rms - 0.3 / math.sqrt(2)) < 1e-9
    assert abs(st - st_true) < 1e-9
    assert all(math.isnan(v) for v in bench.shedding_stats(fx[:3], fy[:3], d, u, nz))
    from mrlbm_3d_cuda_gb300.statistics import shedding
    st2 = 0.1835  # the shipped case's shedding: about 9.2 periods in its 8,001-step window
    t2 = np.arange(48000, 56001)
    d2, u2, nz2 = 16.0, 0.1, 48
    q2 = 0.5 * u2 * u2 * d2 * nz2
    s = shedding(t2, 1.6 * q2 + 0 * t2, 0.28 * q2 * np.sin(2 * math.pi * st2 * u2 / d2 * t2 + 0.7), d2, u2, nz2)
    assert abs(s.st / st2 - 1) < 1e-4 and s.periods == 8
