"""Golden vectors from a run of the reference's own GPU build (sakthi-lbm/MRLBM_3D_CUDA).

The reference ships no test data, so the time step is pinned against its own solver run on
a GB300: `oracle/ref_gpu.py` stages, builds and runs the shipped cylinder case
(cases/cylinder/constants.cuh: 336 x 144 x 48, D = 16, Re = 100, U = 0.1, periodic y and z,
convective outlet) for MAX_ITER = N, i.e. iterations 0..N = N + 1 steps from the reference
initial state.  Its checkpoint (restart.bin, MRLBM_3D/src/restart/restart_io.cu:3-52:
int iteration, then rho - rho0, ux, uy, uz, mxx, myy, mzz, mxy, mxz, myz, each NX*NY*NZ
floats in the tiled IDX_BLOCK order) and forces.dat (stat_header.cuh:16-33: `iter Fx Fy Fz`
per step) are reduced here to a fixture small enough to commit:
  * every node that is not plain bulk fluid (walls, BCFLUID, inlet / outlet faces) plus a
    seeded random sample of 40,000 nodes, all 10 moments, by tiled index; with z walls
    (stage --z-walls, Z_PERIODIC 0) the plain z-face nodes are sampled (8,000 of them)
    except inside the classification window, which is kept whole on the two outer planes
    at each end (BCSOLID nodes and their neighbours);
  * per-field max |m|, sum m and sum m^2 over the whole grid (FP64);
  * the forces.dat rows;
  * 5,000 seeded positions of each of the six face-population arrays that follow the moments
    in restart.bin (X_WEST, X_EAST, Y_SOUTH, Y_NORTH, Z_BACK, Z_FRONT, core/index.cuh:42-79),
    with their values.

Run on the GPU machine from the repository root:
    python oracle/ref_gpu.py stage cyl_n10 --steps 10          (where the reference tree is)
    python oracle/ref_gpu.py check && python oracle/ref_gpu.py build cyl_n10 && python oracle/ref_gpu.py run cyl_n10
    python tests/golden/make_ref_run_golden.py cyl_n10 tests/golden/ref_cylinder_run_n10.npz
(z walls: stage cylz_n10 --steps 10 --z-walls, output ref_cylinder_zwall_run_n10.npz).
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


def main(tag: str, out: str):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    d = ROOT / "baseline" / "_ref" / tag
    cfg = json.loads((d / "config.json").read_text())
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
    sim = Simulation(desc, host_only=True)
    types = sim.node_types(layout=N.LAYOUT_REF_TILED)
    sim.close()
    cls = types >> 20
    rng = np.random.default_rng(20261203)
    if z_walls:
        from tests.golden.make_golden import tiled_to_lex
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
    m64 = m.astype(np.float64)
    np.savez_compressed(
        out, steps=np.int64(it), idx=idx.astype(np.int32), moments=m[:, idx],
        field_max=np.abs(m64).max(axis=1), field_sum=m64.sum(axis=1), field_sumsq=(m64 * m64).sum(axis=1),
        forces=forces, nxyz=np.array([desc.nx, desc.ny, desc.nz], dtype=np.int32), z_walls=np.int32(z_walls),
        halo_pos=np.stack(halo_pos).astype(np.int64), halo_val=np.stack(halo_val))
    print(f"{out}: {it} steps, {idx.size} sampled nodes, {forces.shape[0]} force rows")


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
