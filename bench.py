"""Benchmark: MR-LBM D3Q27 throughput (MLUPS) and HBM roofline on the 256^3 Taylor-Green
vortex (periodic, u0 = 0.05, Re = 1600), the workload the headline metric is quoted on.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--storage f32|f16|bf16] [--impl ours|reference]

One step = one full time step of the solver (stream + collide, one fused kernel) over the
256^3 grid.  `value` is device-timed with inputs resident in HBM; `e2e` goes through the C
ABI with host buffers: the initial moment field is uploaded from pinned memory, every step
reads back its FP64 mass / energy sample, and the final field is read back, all inside the
timed region.  The reference arm (--impl reference) times the CPU restatement of the
reference algorithm (the reference has no CPU path) on a bounded slab of the same workload.
Multi-GPU: no z-slab exchange between GPUs is implemented, so N > 1 runs N independent
replicas (weak scaling), one per rank.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

B_ALG = {"f32": 152.0, "f16": 76.0, "bf16": 76.0, "f16u32": 92.0}   # algorithmic bytes per lattice update (f16u32: 2 x 28 B moments + FP16 face populations)
B_MIN = {"f32": 80.0, "f16": 40.0, "bf16": 40.0, "f16u32": 56.0}    # moments in + out only
STORAGE = {"f32": 0, "f16": 1, "bf16": 2, "f16u32": 3}


def measured_traffic(storage: str):
    """DRAM bytes per node of the step kernel from the committed ncu summary, or None."""
    p = ROOT / "profiles" / "dram_traffic.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 3 and not line.startswith("#") and parts[0] == "step_kernel" and parts[1] == storage:
            return float(parts[2])
    return None


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.rows = []
        self._first = threading.Event()
        self._proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, FileNotFoundError):
            self._proc = None
        # nvidia-smi needs a moment before its first sample: start timing only once it samples
        t0 = time.time()
        while self._proc and not self._first.is_set() and time.time() - t0 < 5.0:
            self._first.wait(0.05)
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)
                self._first.set()

    def __exit__(self, *exc):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[3 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_max(values):
    """Element-wise max over all ranks (identity without a process group): every rank's
    timings are replaced by the slowest rank's."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def replica_value(n_nodes: int, steps: int, seconds: float, world: int) -> float:
    """Whole-job MLUPS of `world` replicas, each advancing n_nodes for `steps` steps, timed by
    the slowest one."""
    return world * n_nodes * steps / seconds / 1e6


def cpu_baseline(n: int, steps: int, bits: int = 64, budget_s: float = 20.0):
    """The oracle (CPU restatement of the reference step; the reference has no CPU path) on the
    full n^3 Taylor-Green grid of the workload, all host threads: one untimed step, then up to
    `steps` timed steps, fewer if they would take longer than about `budget_s`.  The
    descriptor is built without the solver library (oracle.periodic_box_desc)."""
    import oracle
    desc = oracle.periodic_box_desc(n, 0.05, 1600.0)
    o = oracle.Oracle(desc, bits)
    o.init(2, (float(np.float32(0.05)), n / (2 * math.pi)))  # INIT_TAYLOR_GREEN
    t0 = time.perf_counter()
    o.step(1)
    first = time.perf_counter() - t0
    k = max(1, min(steps, int(budget_s / max(first, 1e-3))))
    t0 = time.perf_counter()
    o.step(k)
    dt = time.perf_counter() - t0
    o.close()
    cores = os.cpu_count() or 1
    return {"value": n ** 3 * k / dt / 1e6, "unit": "MLUPS", "cores": cores, "kind": "port",
            "sample": f"{k} time steps of the full {n}^3 Taylor-Green grid after one untimed step, "
                      f"FP{bits} restatement of the reference step, OpenMP {cores} threads"}


# The reference's own GPU build on the same workload and GPU model (stock time loop timed with
# CUDA events in a staged copy of its sources): recorded in profiles/reference_build_loops.md.
_REF_SRC = {"kind": "reference build, stock loop", "source": "profiles/reference_build_loops.md"}
REFERENCE_GPU = {"tgv256": {"value": 9451.0, "unit": "MLUPS", "ms_per_step": 1.7752, "steps": 196, **_REF_SRC},
                 "cylinder16": {"value": 6872.0, "unit": "MLUPS", "ms_per_step": 0.33797, "steps": 55996, **_REF_SRC},
                 "annulus": {"value": 7173.0, "unit": "MLUPS", "ms_per_step": 0.6601, "steps": 996, **_REF_SRC}}


def watchdog_steps(first: int, k: int, every: int = 64) -> int:
    """Steps it in [first, first + k) on which the divergence watchdog runs ((it + 1) % every == 0)."""
    return (first + k) // every - first // every


def metric_name(n: int) -> str:
    return f"MLUPS (D3Q27 MR-LBM, {n}^3 Taylor-Green)"


def run_reference(args):
    """The reference's algorithm on the host cores: the FP32 oracle (the reference has no CPU
    path) on the full n^3 Taylor-Green grid of the workload, all host threads.  Each timed
    step is one full time step; the number of timed steps is K or fewer, so that the timed
    steps take about --ref-budget seconds at most (the line says how many ran).  Only rank 0
    runs; the descriptor is built without the solver library."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    import oracle
    n = args.n
    desc = oracle.periodic_box_desc(n, 0.05, 1600.0)
    o = oracle.Oracle(desc, 32)
    o.init(2, (float(np.float32(0.05)), n / (2 * math.pi)))  # INIT_TAYLOR_GREEN
    t0 = time.perf_counter()
    for _ in range(max(1, min(args.warmup, 3))):
        o.step(1)
    per = (time.perf_counter() - t0) / max(1, min(args.warmup, 3))
    k = max(1, min(args.steps, int(args.ref_budget / max(per, 1e-3))))
    times = []
    for _ in range(k):
        t0 = time.perf_counter()
        o.step(1)
        times.append(time.perf_counter() - t0)
    o.close()
    total = sum(times)
    value = n ** 3 * len(times) / total / 1e6 if total > 0 else 0.0
    cores = os.cpu_count() or 1
    sample = (f"{len(times)} full time steps of the {n}^3 Taylor-Green grid (of the {args.steps} asked, bounded "
              f"to about {args.ref_budget:.0f} s) after {max(1, min(args.warmup, 3))} untimed ones, FP32 "
              f"restatement of the reference step, OpenMP {cores} threads")
    line = {
        "impl": "reference", "metric": metric_name(n), "value": value, "unit": "MLUPS",
        "n_gpus": world, "steps": args.steps, "steps_timed": len(times), "warmup": args.warmup,
        "ms_per_step": 1e3 * total / max(1, len(times)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"taylor-green {n}^3 D3Q27, u0=0.05, Re=1600, full grid", "storage": "f32"},
        "cpu_baseline": {"value": value, "unit": "MLUPS", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_batch(args):
    """C4: independent cylinder cases of uneven size, batched (one persistent launch per kernel
    per step, CUDA-graph replay, autotuned tiles) against plain per-case launches."""
    import torch
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from mrlbm_3d_cuda_gb300 import Batch, cases
    from mrlbm_3d_cuda_gb300 import native as N
    storage = args.storage
    descs = cases.c4_batch(args.batch_cases, 1234, STORAGE[storage])
    for d in descs:
        d.watchdog_every = -1  # cases that diverge are reported from their final fields below
    t0 = time.perf_counter()
    b = Batch(descs)
    for c in b.cases:
        c.init(N.INIT_REST)
    setup_s = time.perf_counter() - t0
    tile = b.autotune(3) if not args.no_autotune else None
    n_nodes = b.n_nodes

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def timed(fn):
        fn(args.warmup)
        b.sync()
        barrier()
        t = time.perf_counter()
        fn(args.steps)
        b.sync()
        barrier()
        return time.perf_counter() - t

    with ClockSampler(local) as clk:
        t_batch = timed(b.step)
    # C4's draw includes cases near tau = 0.5 (D = 8, Re = 300: tau 0.504) where the scheme
    # diverges within thousands of steps; the throughput is the same either way
    diverged = []
    for i, (c, d) in enumerate(zip(b.cases, descs)):
        if not np.isfinite(c.moments(["rho", "ux"])).all():
            diverged.append({"case": i, "D": float(d.d_wall[0]), "Re": round(float(d.re), 2),
                             "tau": round(1.0 / float(d.omega), 5)})
    for c in b.cases:
        c.init(N.INIT_REST)
    t_seq = timed(b.step_sequential)
    t_batch, t_seq = reduce_max([t_batch, t_seq])
    value = replica_value(n_nodes, args.steps, t_batch, world)
    seq_value = replica_value(n_nodes, args.steps, t_seq, world)

    # end to end: upload every case's field from pinned memory, step with force sampling,
    # read back every case's force history and final field
    hosts = [torch.empty((10, c.n), dtype=torch.float32, pin_memory=True) for c in b.cases]
    for c, hb in zip(b.cases, hosts):
        c.moments(out=hb.numpy())
    b.set_sampling(1)
    barrier()
    t = time.perf_counter()
    for c, hb in zip(b.cases, hosts):
        c.set_moments(hb.numpy())
    b.step(args.steps)
    for c, hb in zip(b.cases, hosts):
        c.force_history(args.steps)
        c.moments(out=hb.numpy())
    b.sync()
    barrier()
    e2e_s = reduce_max([time.perf_counter() - t])[0]
    in_bytes = sum(hb.numel() * 4 for hb in hosts)
    peak, peak_kind = measured_peaks()
    line = {
        "metric": f"MLUPS (D3Q27 MR-LBM, batch of {len(descs)} cylinder cases)",
        "value": value, "unit": "MLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_batch / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": storage, "data": "synthetic",
        "config": {"workload": f"{len(descs)} cylinder-in-channel cases (cases.c4_batch, seed 1234), "
                               f"{n_nodes / 1e6:.1f} M nodes in all, {storage} moment storage",
                   "tile": list(tile) if tile else None, "setup_s": setup_s,
                   "sequential_value": seq_value, "batch_over_sequential": value / seq_value,
                   "diverged_cases": diverged,
                   "timing": "host wall clock around K batched steps, synchronised",
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "achieved": n_nodes * B_ALG[storage] * args.steps / t_batch / 1e9,
                     "peak": peak, "unit": "GB/s",
                     "frac": n_nodes * B_ALG[storage] * args.steps / t_batch / 1e9 / peak, "peak_kind": peak_kind,
                     "bytes_per_lup": B_ALG[storage], "traffic": None},
        "e2e": {"value": replica_value(n_nodes, args.steps, e2e_s, world), "unit": "MLUPS",
                "h2d_bytes_per_step": in_bytes / args.steps, "d2h_bytes_per_step": (in_bytes + 80 * len(descs) * args.steps) / args.steps},
        "gpu_launches": 3 * args.steps,
        "clocks": clk.summary(),
    }
    b.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def shedding_stats(fx, fy, d, u, nz, rho0=1.0):
    """Cd (mean), rms Cl and Strouhal number (lift zero crossings) from per-step wall forces,
    over the second half of the run."""
    from mrlbm_3d_cuda_gb300.statistics import shedding
    if len(fx) < 4:
        return float("nan"), float("nan"), float("nan")
    half = len(fx) // 2
    s = shedding(np.arange(len(fx) - half), fx[half:], fy[half:], d, u, nz, rho0)
    return s.cd, s.cl_rms, s.st


def run_c5(args):
    """C5: 1024 x 512 x 256 cylinder, D = 64, Re = 3900, u = 0.05 (1 + 1 % noise): FP16 moment
    storage (FP32 collision, FP64 force sums) against an FP32-storage run of the same case;
    MLUPS of the FP16 run, Cd / rms Cl / St of both."""
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    stats, value, ms_step, clocks = {}, None, None, None
    runs = args.c5_runs.split(",")
    workload = ""  # described by the FP16 run
    sr = bool(args.stochastic_rounding)
    for st in runs:
        desc = cases.c5_turbulent_cylinder(STORAGE[st], re=args.re)
        desc.stochastic_rounding = int(sr and st != "f32")
        sim = Simulation(desc, init=False)
        sim.set_stream(stream.cuda_stream)
        if args.c5_init == "noisy":
            sim.init(N.INIT_NOISY_UNIFORM, (0.05, 0.0, 0.0, 0.01, 1234))
        else:
            sim.init(N.INIT_REST)
        sim.set_sampling(1, 1000)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        done, diverged, ms = 0, None, 0.0
        with ClockSampler(local) as clk:
            while done < args.steps:  # chunks of 1000 steps, each checked for a non-finite state
                k = min(1000, args.steps - done)
                ev0.record(stream)
                sim.step(k)
                ev1.record(stream)
                torch.cuda.synchronize()
                ms += ev0.elapsed_time(ev1)
                done += k
                if not np.isfinite(sim.diagnostics()[1]).all():
                    diverged = done
                    break
        _, f = sim.force_history(done)
        good = np.isfinite(f[:, 0, :2]).all(axis=1)
        n_ok = int(np.argmin(good)) if not good.all() else len(good)
        stats[st] = shedding_stats(f[:n_ok, 0, 0], f[:n_ok, 0, 1], desc.d_wall[0], desc.u_max, desc.nz)
        stats[st] += (diverged,)
        ms_done = done
        if st == "f16":
            n_nodes = desc.nx * desc.ny * desc.nz
            value, ms_step, clocks = replica_value(n_nodes, ms_done, ms * 1e-3, 1), ms / ms_done, clk.summary()
            workload = (f"cylinder {desc.nx}x{desc.ny}x{desc.nz}, D={desc.d_wall[0]:.0f}, Re={args.re:g}, u=0.05, "
                        f"start: {'uniform +1% noise' if args.c5_init == 'noisy' else 'rest'}, tau={1 / desc.omega:.5f}"
                        + (", FP16 stochastic rounding" if sr else ""))
        sim.close()
    nan4 = (float("nan"),) * 3 + (None,)
    (cd16, cl16, st16, div16), (cd32, cl32, st32, div32) = stats.get("f16", nan4), stats.get("f32", nan4)
    line = {
        "metric": "MLUPS (D3Q27 MR-LBM, 1024x512x256 cylinder, FP16 storage)", "value": value,
        "unit": "MLUPS", "n_gpus": 1, "steps": args.steps, "warmup": 0, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f16", "data": "synthetic",
        "config": {"workload": workload, "storage": "f16 vs f32",
                   "f16": {"cd": cd16, "cl_rms": cl16, "st": st16, "diverged_at_step": div16},
                   "f32": {"cd": cd32, "cl_rms": cl32, "st": st32, "diverged_at_step": div32},
                   "cd_rel_err": cd16 / cd32 - 1, "cl_rms_rel_err": cl16 / cl32 - 1, "st_rel_err": st16 / st32 - 1,
                   "statistics": "second half of the run; St from the Cl spectrum peak"},
        "gpu_launches": (3 + sr) * args.steps, "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# Storage-precision errors measured on a GB300 against the FP64 oracle
# (tests/test_storage_precision.py): C1 cylinder mean Cd, and max |E / E64 - 1| of the 64^3
# Taylor-Green vortex over 1000 steps.
STATED_ERRORS = {"f32": {"c1_cd_rel_err": 1.0e-5, "tgv64_energy_rel_err": 1.1e-6},
                 "f16": {"c1_cd_rel_err": 1.0e-3, "tgv64_energy_rel_err": 7.3e-4},
                 "f16_sr": {"c1_cd_rel_err": 1.0e-4, "tgv64_energy_rel_err": 4.5e-5},
                 "f16u32": {"c1_cd_rel_err": 8.3e-4, "tgv64_energy_rel_err": 5.9e-6},
                 "f16u32_sr": {"c1_cd_rel_err": 4.4e-5, "tgv64_energy_rel_err": 3.2e-7}}


def storage_comparison(args, stream, n, world):
    """The same Taylor-Green step with FP16 storage and with the hybrid storage (FP32
    velocity, FP16 density deviation and second moments), each rounding to nearest and
    stochastically: device-resident MLUPS over min(steps, 1000) timed steps, beside the stated
    errors."""
    import torch
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    out = {}
    k = max(1, min(args.steps, 1000))
    for name, st, sr in (("f16", "f16", 0), ("f16_sr", "f16", 1), ("f16u32", "f16u32", 0),
                         ("f16u32_sr", "f16u32", 1)):
        desc = cases.c2_taylor_green(n, STORAGE[st])
        desc.stochastic_rounding = sr
        sim = Simulation(desc, init=False)
        sim.set_stream(stream.cuda_stream)
        sim.init(N.INIT_TAYLOR_GREEN, cases.tgv_params(desc))
        sim.step(max(3, args.warmup))
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        sim.step(k)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = reduce_max([ev0.elapsed_time(ev1)])[0]
        nodes = desc.nx * desc.ny * desc.nz
        value = replica_value(nodes, k, ms * 1e-3, world)
        peak, _ = measured_peaks()
        out[name] = {"value": value, "unit": "MLUPS", "steps": k,
                     "frac_vs_min_traffic": nodes * B_MIN[st] / (ms / k * 1e-3) / 1e9 / peak,
                     **STATED_ERRORS.get(name, {})}
        sim.close()
    out["f32"] = dict(STATED_ERRORS["f32"])
    out["errors_from"] = "tests/test_storage_precision.py: GB300 runs against the FP64 oracle"
    return out


def run_ours(args):
    import torch
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N

    storage = args.storage
    cyl = args.workload in ("cylinder", "annulus")  # cases with walls: reference initial state
    ref_gpu = None
    if args.workload == "cylinder":
        desc = cases.reference_cylinder(STORAGE[storage], args.diameter)
        workload = (f"reference cylinder case scaled to D={args.diameter}: {desc.nx}x{desc.ny}x{desc.nz} D3Q27, "
                    f"Re=100, U=0.1, convective outlet, periodic y/z, {storage} moment storage")
        metric = f"MLUPS (D3Q27 MR-LBM, cylinder D={args.diameter} {desc.nx}x{desc.ny}x{desc.nz})"
        ref_gpu = REFERENCE_GPU["cylinder16"] if args.diameter == 16 else None
    elif args.workload == "annulus":
        desc = cases.reference_annulus(STORAGE[storage])
        workload = (f"reference annulus case: {desc.nx}x{desc.ny}x{desc.nz} D3Q27, r = 32 / 64, inner wall 0.03, "
                    f"Re=70, periodic z, {storage} moment storage")
        metric = f"MLUPS (D3Q27 MR-LBM, annulus {desc.nx}x{desc.ny}x{desc.nz})"
        ref_gpu = REFERENCE_GPU["annulus"]
    else:
        desc = cases.c2_taylor_green(args.n, STORAGE[storage])
        workload = f"taylor-green {args.n}^3 D3Q27, u0=0.05, Re=1600, {storage} moment storage"
        metric = metric_name(args.n)
    sr = bool(args.stochastic_rounding) and storage != "f32"
    if sr:
        desc.stochastic_rounding = 1
        workload += ", stochastic rounding"
    n_nodes = desc.nx * desc.ny * desc.nz
    stream = torch.cuda.Stream()  # a real stream handle: the library launches on it, events time it
    torch.cuda.set_stream(stream)
    sim = Simulation(desc, init=False)
    sim.set_stream(stream.cuda_stream)
    if cyl:
        sim.init(N.INIT_REFERENCE_NOISE)
    else:
        sim.init(N.INIT_TAYLOR_GREEN, cases.tgv_params(desc))
    info = sim.get_info()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident timing --------------------------------------------------------
    sim.step(args.warmup)
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(stream)
        sim.step(args.steps)
        ev1.record(stream)
        barrier()
    ms = reduce_max([ev0.elapsed_time(ev1)])[0]
    ms_step = ms / args.steps
    value = replica_value(n_nodes, args.steps, ms * 1e-3, world)
    kernel_ms = ms_step  # one step-kernel launch per step, back to back on one stream

    # ---- end-to-end through the C ABI with host buffers -----------------------------------
    host = torch.empty((10, n_nodes), dtype=torch.float32, pin_memory=True)
    hv = host.numpy()
    sim.moments(out=hv)  # current state as the e2e input
    sim.set_sampling(0, 1)
    e2e_steps = max(1, args.steps)
    barrier()
    t0 = time.perf_counter()
    sim.set_moments(hv)
    sim.step(e2e_steps)
    _, diag = sim.diagnostics(e2e_steps)
    sim.moments(out=hv)
    torch.cuda.synchronize()
    e2e_s = reduce_max([time.perf_counter() - t0])[0]
    e2e_value = replica_value(n_nodes, e2e_steps, e2e_s, world)
    sim.set_sampling(0, 0)
    assert np.isfinite(diag).all()

    peak, peak_kind = measured_peaks()
    achieved = n_nodes * B_ALG[storage] / (kernel_ms * 1e-3) / 1e9
    line = {
        "metric": metric,
        "value": value, "unit": "MLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": storage, "data": "synthetic",
        "config": {"workload": workload,
                   "storage": storage, "stochastic_rounding": sr, "tile": list(info.tile),
                   "ctas": int(info.reserved[0]),
                   "l2": f"inputs larger than L2 ({n_nodes * 10 * (4 if storage == 'f32' else 2) / 1e6:.0f} MB "
                         f"per moment buffer vs 129 MB L2)",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "bytes_per_lup": B_ALG[storage],
                     "frac_vs_min_traffic": n_nodes * B_MIN[storage] / (kernel_ms * 1e-3) / 1e9 / peak,
                     "traffic": (measured_traffic(storage) * n_nodes if measured_traffic(storage) else None),
                     "traffic_source": "ncu dram__bytes_read+write per node (profiles/dram_traffic.txt) x nodes"},
        "e2e": {"value": e2e_value, "unit": "MLUPS", "h2d_bytes_per_step": hv.nbytes / e2e_steps,
                "d2h_bytes_per_step": 16 + hv.nbytes / e2e_steps},
        # per step: the step kernel; the cylinder adds the boundary-tile step kernel, the
        # node-list kernel and the wall kernel; stochastic rounding adds its counter tick; every
        # 64th step (the divergence watchdog) adds the FP64 sum kernel
        "gpu_launches": args.steps * ((4 if cyl else 1) + sr) + watchdog_steps(args.warmup, args.steps),
        "clocks": clk.summary(),
    }
    if not cyl and storage == "f32" and not args.no_storage_comparison:
        line["storage_comparison"] = storage_comparison(args, stream, args.n, world)
        line["storage_comparison"]["f32"]["value"] = value
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.n, args.cpu_steps, bits=64)
    if not cyl and args.n == 256:
        ref_gpu = REFERENCE_GPU["tgv256"]
    if ref_gpu:
        line["reference_gpu"] = dict(ref_gpu, speedup=value / world / ref_gpu["value"])
    sim.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--storage", default="f32", choices=list(STORAGE))
    ap.add_argument("--stochastic-rounding", action="store_true",
                    help="16-bit storage: round the time-step stores stochastically (cvt.rs)")
    ap.add_argument("--size", dest="n", type=int, default=256, help="TGV grid edge (n^3)")
    ap.add_argument("--workload", default="tgv", choices=["tgv", "cylinder", "annulus", "batch", "c5"])
    ap.add_argument("--batch-cases", type=int, default=64)
    ap.add_argument("--re", type=float, default=3900.0, help="Reynolds number of the c5 workload")
    ap.add_argument("--c5-init", default="noisy", choices=["noisy", "rest"])
    ap.add_argument("--c5-runs", default="f16,f32", help="storage runs of the c5 workload (f16 first: its speed is the value)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--diameter", type=int, default=16)
    ap.add_argument("--ref-budget", type=float, default=60.0,
                    help="--impl reference: seconds of timed full-grid CPU steps at most")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-storage-comparison", action="store_true",
                    help="skip the FP16 runs that the default FP32 Taylor-Green line reports beside it")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "c5":
        run_c5(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
