"""Generate the golden fixtures under tests/golden/ from the reference's own code.

ref_cylinder_geometry.npz — output of the reference's host node classification for its
shipped cylinder case (336 x 144 x 48, D = 16, Re = 100, periodic y and z), produced by
oracle/_ref/ref_geometry (oracle/ref_harness/ref_geometry.cu compiled from the reference
sources by oracle/build_ref.py).  Index arrays are converted from the reference's tiled
IDX_BLOCK order to lexicographic x + NX (y + NY z); the full node-type array is stored
lexicographic too.

ref_cylinder_staircase_geometry.npz — the same case with the staircase classification
(triangular = false, oracle/_ref/ref_geometry_staircase).

ref_cylinder_zwall_geometry.npz — the same for that case with z walls (Z_PERIODIC 0,
oracle/_ref/ref_geometry_zwall): adds the BCSOLID nodes on the z = 0 and z = NZ - 1 faces
(cases/cylinder/nodeClass.cuh:254-287) and their list.

ref_annulus_geometry.npz — the reference's classification of its shipped annulus case
(136 x 136 x 256, r 32 / 64) for both walls (oracle/_ref/ref_geometry_annulus): node types of
the z = 0 and z = 255 planes plus a SHA-256 of the whole array, per-wall lists, normals, wall
distances and masks, and the per-tag BCFLUID masks.  ref_annulus_zwall_geometry.npz: the same
for that case built with Z_PERIODIC 0, with both walls' BCSOLID lists.

ref_geometry_files.json — SHA-256 and size of each grid_layout/*.dat file the reference's own
write_geometry_files (cases/cylinder/cylinder_helpers.cuh:388-470) writes for both builds.

Run from the repository root where the reference tree is mounted:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.build_ref import (build_ref_geometry, build_ref_geometry_annulus,  # noqa: E402
                              build_ref_geometry_annulus_zwall, build_ref_geometry_staircase,
                              build_ref_geometry_zwall)


def tiled_to_lex(idx: np.ndarray, nx: int, ny: int, nz: int) -> np.ndarray:
    """Inverse of the reference IDX_BLOCK (core/index.cuh:11-28, GlobalIndexToXYZ :86-111)."""
    idx = idx.astype(np.int64)
    gx, gy = nx // 8, ny // 8
    block, thread = idx // 256, idx % 256
    bx, by, bz = block % gx, (block // gx) % gy, block // (gx * gy)
    tx, ty, tz = thread % 8, (thread // 8) % 8, thread // 64
    x, y, z = bx * 8 + tx, by * 8 + ty, bz * 4 + tz
    return x + nx * (y + ny * z)


def make_geometry(out: Path, zwall: bool = False, staircase: bool = False):
    exe = build_ref_geometry_zwall() if zwall else (build_ref_geometry_staircase() if staircase else build_ref_geometry())
    if exe is None:
        raise SystemExit("reference tree not present: cannot regenerate")
    with tempfile.TemporaryDirectory() as td:
        subprocess.run([str(exe), td], check=True, capture_output=True)
        d = Path(td)
        rd = lambda name, dt: np.fromfile(d / name, dtype=dt)  # noqa: E731
        meta = rd("meta.i32", np.int32)
        fmeta = rd("meta.f32", np.float32)
        nx, ny, nz, nb, nbf, nbs = (int(v) for v in meta[:6])
        types_tiled = rd("node_type_tiled.u32", np.uint32)
        lex = tiled_to_lex(np.arange(nx * ny * nz), nx, ny, nz)
        types = np.empty_like(types_tiled)
        types[lex] = types_tiled
        np.savez_compressed(
            out,
            shape=np.array([nx, ny, nz], dtype=np.int32),
            nb=np.int32(nb), nb_fluid=np.int32(nbf), nb_solid=np.int32(nbs), z_periodic=np.int32(meta[6]),
            xc=fmeta[0], yc=fmeta[1], d_wall=fmeta[2], omega=fmeta[3],
            node_types=types,
            boundary_list=tiled_to_lex(rd("boundary_list_tiled.u64", np.uint64), nx, ny, nz),
            unit_nx=rd("unit_nx.f32", np.float32), unit_ny=rd("unit_ny.f32", np.float32),
            delta=rd("delta_w.f32", np.float32),
            in_mask=rd("in_mask.u32", np.uint32), out_mask=rd("out_mask.u32", np.uint32),
            fluid_list=tiled_to_lex(rd("bcfluid_list_tiled.u64", np.uint64), nx, ny, nz),
            tag_in_mask=rd("tag_in_mask.u32", np.uint32), tag_out_mask=rd("tag_out_mask.u32", np.uint32),
            solid_list=tiled_to_lex(rd("bcsolid_list_tiled.u64", np.uint64), nx, ny, nz),
        )


def make_annulus(out: Path, zwall: bool = False):
    exe = build_ref_geometry_annulus_zwall() if zwall else build_ref_geometry_annulus()
    if exe is None:
        raise SystemExit("reference tree not present: cannot regenerate")
    with tempfile.TemporaryDirectory() as td:
        subprocess.run([str(exe), td], check=True, capture_output=True)
        d = Path(td)
        rd = lambda name, dt: np.fromfile(d / name, dtype=dt)  # noqa: E731
        meta = rd("meta.i32", np.int32)
        nx, ny, nz = (int(v) for v in meta[:3])
        tiled = rd("node_type_tiled.u32", np.uint32)
        lex = tiled_to_lex(np.arange(nx * ny * nz), nx, ny, nz)
        types = np.empty_like(tiled)
        types[lex] = tiled
        plane = nx * ny
        arrays = dict(shape=np.array([nx, ny, nz], dtype=np.int32),
                      nb=meta[[3, 5]].astype(np.int32), nb_fluid=meta[[4, 6]].astype(np.int32),
                      nb_solid=meta[[7, 8]].astype(np.int32), z_periodic=np.int32(meta[9]),
                      types_first_plane=types[:plane], types_last_plane=types[-plane:],
                      types_sha256=np.frombuffer(hashlib.sha256(types.tobytes()).digest(), dtype=np.uint8),
                      tag_in_mask=rd("tag_in_mask.u32", np.uint32), tag_out_mask=rd("tag_out_mask.u32", np.uint32))
        for w in ("inner", "outer"):
            arrays[f"{w}_boundary_list"] = tiled_to_lex(rd(f"{w}_boundary_list_tiled.u64", np.uint64), nx, ny, nz)
            arrays[f"{w}_unit_nx"] = rd(f"{w}_unit_nx.f32", np.float32)
            arrays[f"{w}_unit_ny"] = rd(f"{w}_unit_ny.f32", np.float32)
            arrays[f"{w}_delta"] = rd(f"{w}_delta_w.f32", np.float32)
            arrays[f"{w}_in_mask"] = rd(f"{w}_in_mask.u32", np.uint32)
            arrays[f"{w}_out_mask"] = rd(f"{w}_out_mask.u32", np.uint32)
            arrays[f"{w}_fluid_list"] = tiled_to_lex(rd(f"{w}_bcfluid_list_tiled.u64", np.uint64), nx, ny, nz)
            arrays[f"{w}_solid_list"] = tiled_to_lex(rd(f"{w}_bcsolid_list_tiled.u64", np.uint64), nx, ny, nz)
        np.savez_compressed(out, **arrays)


def make_geometry_files(out: Path):
    res = {}
    for variant, build in (("periodic_z", build_ref_geometry), ("z_walls", build_ref_geometry_zwall)):
        exe = build()
        if exe is None:
            raise SystemExit("reference tree not present: cannot regenerate")
        with tempfile.TemporaryDirectory() as td:
            subprocess.run([str(exe), td, "files"], check=True, capture_output=True)
            d = next(Path(td).rglob("grid_layout"))
            res[variant] = {f.name: {"sha256": hashlib.sha256(f.read_bytes()).hexdigest(), "bytes": f.stat().st_size}
                            for f in sorted(d.glob("*.dat"))}
    out.write_text(json.dumps(res, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    here = Path(__file__).resolve().parent
    for name, zwall, stair in (("ref_cylinder_geometry.npz", False, False),
                               ("ref_cylinder_zwall_geometry.npz", True, False),
                               ("ref_cylinder_staircase_geometry.npz", False, True)):
        make_geometry(here / name, zwall, stair)
        print("wrote", here / name)
    make_geometry_files(here / "ref_geometry_files.json")
    print("wrote", here / "ref_geometry_files.json")
    for name, zwall in (("ref_annulus_geometry.npz", False), ("ref_annulus_zwall_geometry.npz", True)):
        make_annulus(here / name, zwall)
        print("wrote", here / name)
