"""Golden vectors from runs of the reference's own GPU build (sakthi-lbm/MRLBM_3D_CUDA).

The reference ships no test data, so the time step is pinned against its own solver run on
a GB300: `oracle/ref_gpu.py` stages, builds and runs it, and this script reduces the run's
output to a fixture small enough to commit.  The reference writes

  * restart.bin (MRLBM_3D/src/restart/restart_io.cu:3-52): int iteration, then rho - rho0,
    ux, uy, uz, mxx, myy, mzz, mxy, mxz, myz, each NX*NY*NZ floats in the tiled IDX_BLOCK
    order (core/index.cuh:11-28), then the six face-population arrays (X_WEST, X_EAST,
    Y_SOUTH, Y_NORTH, Z_BACK, Z_FRONT, core/index.cuh:42-79);
  * forces.dat (statistics/stat_header.cuh:16-33): `iter Fx Fy Fz` per step of the statistics
    window;
  * pressure.dat (cases/cylinder/cylinder_kernels.cu:238-283): `theta z Cp`;
  * `REF_LOOP_MS <ms> REF_LOOP_STEPS <n>` on stdout (the staged copy's loop timer).

Kinds (the staged case, from baseline/_ref/<tag>/config.json):

  cylinder  the shipped cylinder case (336 x 144 x 48, D = 16, Re = 100, U = 0.1, periodic y
            and z, convective outlet) after N + 1 steps: every node that is not plain bulk
            fluid plus 40,000 random nodes, all 10 moments; with z walls the plain z-face
            nodes are sampled (8,000) except inside the classification window, kept whole on
            the two outer planes at each end; per-field max |m|, sum m, sum m^2 (FP64); the
            forces.dat rows; 5,000 positions of each face-population array.
  shedding  the shipped cylinder case run as shipped (56,000 steps, forces.dat over
            iterations 48,000..56,000), one or more runs of the same build: every run's
            forces.dat rows, pressure.dat and loop time.
  annulus   the shipped annulus (136 x 136 x 256, r = 32 / 64, inner wall 0.03, Re = 70)
            after N + 1 steps: every non-bulk node (both walls, BCFLUID) of the planes
            z = 0, 1, 2, 128, 253, 254, 255, 20,000 further random non-bulk nodes and 40,000
            random nodes, all 10 moments; field statistics as above.
  tgv       the Taylor-Green vortex on the n^3 periodic grid after N + 1 steps: 40,000 random
            nodes and the whole y = 0 plane, all 10 moments; field statistics; loop time.

Run on the GPU machine from the repository root (after oracle/ref_gpu.py build/run):
    python tests/golden/make_ref_run_golden.py <tag> <out.npz>
then, for the annulus and Taylor-Green fixtures, add the oracle's FP32 rounding floor (e32):
    python tests/golden/make_ref_run_golden.py e32 <fixture.npz> annulus|tgv
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

N_RANDOM = 40000


def read_restart(path: Path, n: int):
    raw = path.read_bytes()
    it = int(np.frombuffer(raw[:4], dtype=np.int32)[0])
    m = np.frombuffer(raw[4:4 + 40 * n], dtype=np.float32).reshape(10, n)
    halo = np.frombuffer(raw[4 + 40 * n:], dtype=np.float32)
    return it, m, halo


def tiled_to_lex(idx: np.ndarray, nx: int, ny: int, nz: int) -> np.ndarray:
    """Reference tiled IDX_BLOCK index (8 x 8 x 4 blocks) -> x + nx (y + ny z)."""
    idx = idx.astype(np.int64)
    gx, gy = nx // 8, ny // 8
    block, thread = idx // 256, idx % 256
    bx, by, bz = block % gx, (block // gx) % gy, block // (gx * gy)
    x, y, z = bx * 8 + thread % 8, by * 8 + (thread // 8) % 8, bz * 4 + thread // 64
    return x + nx * (y + ny * z)


def lex_to_tiled(lex: np.ndarray, nx: int, ny: int) -> np.ndarray:
    lex = lex.astype(np.int64)
    x, y, z = lex % nx, (lex // nx) % ny, lex // (nx * ny)
    gx, gy = nx // 8, ny // 8
    block = (x // 8) + gx * ((y // 8) + gy * (z // 4))
    return block * 256 + (x % 8) + 8 * (y % 8) + 64 * (z % 4)


def field_stats(m: np.ndarray) -> dict:
    m64 = m.astype(np.float64)
    return {"field_max": np.abs(m64).max(axis=1), "field_sum": m64.sum(axis=1),
            "field_sumsq": (m64 * m64).sum(axis=1)}


def loop_time(run_dir: Path) -> np.ndarray:
    p = run_dir / "loop_time.json"
    if not p.exists():
        return np.array([np.nan, 0.0])
    t = json.loads(p.read_text())
    return np.array([t["ms"], float(t["steps"])])


def node_classes(desc, layout_tiled: bool = True) -> np.ndarray:
    from mrlbm_3d_cuda_gb300 import Simulation
    from mrlbm_3d_cuda_gb300 import native as N
    sim = Simulation(desc, host_only=True)
    types = sim.node_types(layout=N.LAYOUT_REF_TILED if layout_tiled else N.LAYOUT_LEXICOGRAPHIC)
    sim.close()
    return types >> 20


def reduce_cylinder(d: Path, cfg: dict, out: str):
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    if cfg["diameter"] != 16:
        raise SystemExit("fixtures are made for the shipped D = 16 case only")
    z_walls = bool(cfg.get("z_walls", False))
    desc = cases.reference_cylinder(periodic_z=not z_walls)
    n = desc.nx * desc.ny * desc.nz
    restart = next((d / "run").rglob("restart.bin"))
    forces = np.loadtxt(next((d / "run").rglob("forces.dat")), ndmin=2)
    it, m, halo = read_restart(restart, n)
    nbk = (desc.nx // 8) * (desc.ny // 8) * (desc.nz // 4)
    face_len = [32 * nbk * 9] * 4 + [64 * nbk * 9] * 2
    assert halo.size == sum(face_len), (halo.size, face_len)
    hrng = np.random.default_rng(7)
    halo_pos, halo_val, off = [], [], 0
    for ln in face_len:
        pos = np.sort(hrng.choice(ln, 5000, replace=False))
        halo_pos.append(pos)
        halo_val.append(halo[off + pos])
        off += ln
    assert it == cfg["steps"] + 1, (it, cfg)
    cls = node_classes(desc)
    rng = np.random.default_rng(20261203)
    if z_walls:
        lex = tiled_to_lex(np.arange(n), desc.nx, desc.ny, desc.nz)
        x, y, z = lex % desc.nx, (lex // desc.nx) % desc.ny, lex // (desc.nx * desc.ny)
        b = desc.scan_box
        window = (x >= b[0]) & (x < b[1]) & (y >= b[2]) & (y < b[3]) & ((z <= 1) | (z >= desc.nz - 2))
        plain_face = np.isin(cls, (N.NODE_BACK, N.NODE_FRONT))
        face_pick = rng.choice(np.flatnonzero(plain_face & ~window), 8000, replace=False)
        special = np.union1d(np.flatnonzero((cls != 0) & ~plain_face), np.flatnonzero(window))
        special = np.union1d(special, face_pick)
    else:
        special = np.flatnonzero(cls != 0)
    idx = np.union1d(special, rng.choice(n, N_RANDOM, replace=False)).astype(np.int64)
    np.savez_compressed(
        out, steps=np.int64(it), idx=idx.astype(np.int32), moments=m[:, idx], **field_stats(m),
        forces=forces, nxyz=np.array([desc.nx, desc.ny, desc.nz], dtype=np.int32), z_walls=np.int32(z_walls),
        halo_pos=np.stack(halo_pos).astype(np.int64), halo_val=np.stack(halo_val))
    print(f"{out}: {it} steps, {idx.size} sampled nodes, {forces.shape[0]} force rows")


def reduce_shedding(d: Path, cfg: dict, out: str):
    runs = sorted(p for p in d.iterdir() if p.is_dir() and p.name.startswith("run"))
    forces, times, pressure = [], [], None
    for rd in runs:
        forces.append(np.loadtxt(next(rd.rglob("forces.dat")), ndmin=2))
        times.append(loop_time(rd))
        if pressure is None:
            pp = list(rd.rglob("pressure.dat"))
            if pp:
                pressure = np.loadtxt(pp[0], skiprows=1, ndmin=2)
    if not forces:
        raise SystemExit(f"no runs under {d}")
    np.savez_compressed(out, forces=np.stack(forces), loop_time=np.stack(times),
                        pressure=pressure if pressure is not None else np.zeros((0, 3)),
                        steps=np.int64(cfg["steps"]))
    print(f"{out}: {len(forces)} runs, {forces[0].shape[0]} force rows each")


def reduce_annulus(d: Path, cfg: dict, out: str):
    from mrlbm_3d_cuda_gb300 import cases
    desc = cases.reference_annulus(periodic_z=not cfg.get("z_walls", False))
    nx, ny, nz = desc.nx, desc.ny, desc.nz
    n = nx * ny * nz
    it, m, _ = read_restart(next((d / "run").rglob("restart.bin")), n)
    assert it == cfg["steps"] + 1, (it, cfg)
    cls = node_classes(desc)
    lex = tiled_to_lex(np.arange(n), nx, ny, nz)
    z = lex // (nx * ny)
    planes = np.isin(z, (0, 1, 2, nz // 2, nz - 3, nz - 2, nz - 1))
    special = cls != 0
    rng = np.random.default_rng(20261204)
    keep = np.flatnonzero(special & planes)
    rest = np.flatnonzero(special & ~planes)
    idx = np.union1d(keep, rng.choice(rest, min(20000, rest.size), replace=False))
    idx = np.union1d(idx, rng.choice(n, N_RANDOM, replace=False)).astype(np.int64)
    np.savez_compressed(out, steps=np.int64(it), idx=idx.astype(np.int32), moments=m[:, idx], **field_stats(m),
                        nxyz=np.array([nx, ny, nz], dtype=np.int32), z_walls=np.int32(cfg.get("z_walls", False)),
                        loop_time=loop_time(d / "run"))
    print(f"{out}: {it} steps, {idx.size} sampled nodes ({keep.size} wall-region nodes on whole planes)")


def reduce_tgv(d: Path, cfg: dict, out: str):
    nn = int(cfg["n"])
    n = nn ** 3
    it, m, _ = read_restart(next((d / "run").rglob("restart.bin")), n)
    assert it == cfg["steps"] + 1, (it, cfg)
    rng = np.random.default_rng(20261205)
    x, z = np.meshgrid(np.arange(nn), np.arange(nn), indexing="ij")
    plane = lex_to_tiled((x + nn * nn * z).ravel(), nn, nn)  # the whole y = 0 plane
    idx = np.union1d(rng.choice(n, 60000, replace=False)[:40000], plane).astype(np.int64)
    np.savez_compressed(out, steps=np.int64(it), idx=idx.astype(np.int32), moments=m[:, idx], **field_stats(m),
                        nxyz=np.array([nn, nn, nn], dtype=np.int32), loop_time=loop_time(d / "run"),
                        u0=np.float64(cfg["u0"]), re=np.float64(cfg["re"]))
    print(f"{out}: {it} steps, {idx.size} sampled nodes, loop {loop_time(d / 'run')}")


def add_e32(path: str, kind: str):
    """Add the FP32 rounding floor of the reference algorithm to a fixture: the distance of the
    FP32 oracle from the FP64 oracle after the fixture's step count, on its sampled nodes
    (per field: scaled max, plain max and L2 relative, as tests/conftest.field_errors), and the
    FP32 oracle's own distance from the reference build.  Run where the oracle is built (the
    annulus at 1,001 steps takes a few minutes on 16 cores)."""
    import oracle
    from mrlbm_3d_cuda_gb300 import cases
    sys.path.insert(0, str(ROOT / "tests"))
    from conftest import field_errors
    g = dict(np.load(path))
    steps, idx = int(g["steps"]), g["idx"].astype(np.int64)
    nx, ny, nz = (int(v) for v in g["nxyz"])
    if kind == "annulus":
        desc, init, params, u_ref = cases.reference_annulus(), 0, (), 0.03  # INIT_REFERENCE_NOISE
    elif kind == "tgv":
        desc, init, params, u_ref = oracle.periodic_box_desc(nx, 0.05, 1600.0), 2, (
            float(np.float32(0.05)), nx / (2 * np.pi)), 0.05
    else:
        desc, init, params, u_ref = cases.reference_cylinder(), 0, (), 0.1
    lex = tiled_to_lex(idx, nx, ny, nz)
    got = {}
    for bits in (32, 64):
        o = oracle.Oracle(desc, bits)
        o.init(init, params)
        o.step(steps)
        got[bits] = o.moments().reshape(10, -1)[:, lex]
        o.close()
    e = field_errors(got[32], got[64], u_ref)
    g["e32"], g["e32_plain"], g["e32_l2"] = e[:, 0], e[:, 1], e[:, 2]
    g["o32_vs_ref"] = field_errors(got[32], g["moments"], u_ref)
    np.savez_compressed(path, **g)
    print(f"{path}: e32 {np.array2string(e[:, 0], precision=2)}", flush=True)


def main(tag: str, out: str, kind: str | None = None):
    if tag == "e32":  # add the FP32 rounding floor to an existing fixture: e32 <fixture> <kind>
        return add_e32(out, kind)
    d = ROOT / "baseline" / "_ref" / tag
    cfg = json.loads((d / "config.json").read_text())
    kind = kind or ("shedding" if cfg.get("shipped_run") else cfg.get("case", "cylinder"))
    {"cylinder": reduce_cylinder, "shedding": reduce_shedding, "annulus": reduce_annulus,
     "tgv": reduce_tgv}[kind](d, cfg, out)


if __name__ == "__main__":
    main(*sys.argv[1:])
