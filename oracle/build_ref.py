"""Recipe that compiles pieces of the reference (sakthi-lbm/MRLBM_3D_CUDA) from its own
sources, where they lie, into oracle/_ref/ — test infrastructure only.

* ``ref_geometry``: a host-only program (no GPU) that runs the reference's own node
  classification for its shipped cylinder case and dumps the result (see
  ref_harness/ref_geometry.cu).  Built when the reference tree is present (this
  container); the GPU machine has no reference tree and uses nothing from here.
* ``ref_geometry_zwall``: the same harness for the shipped case with z walls.  The reference
  selects that at compile time (``#define Z_PERIODIC`` in cases/cylinder/constants.cuh:10),
  so its src/ tree is copied to a temporary directory, that one line is set to 0, the
  harness is compiled against the copy and the copy is deleted.

The reference's own build script (compile.sh) is not used: nvcc is called on the one
harness translation unit with the reference's src/ directory on the include path.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
REF_ROOT = Path(os.environ.get("MRLBM_REFERENCE", "/root/reference"))
REF_SRC = REF_ROOT / "MRLBM_3D" / "src"


def reference_present() -> bool:
    return (REF_SRC / "main.cu").exists()


def _nvcc() -> str:
    for cand in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        p = Path(cand) / "bin" / "nvcc"
        if cand and p.exists():
            return str(p)
    return shutil.which("nvcc") or "nvcc"


def build_ref_geometry(force: bool = False) -> Path | None:
    if not reference_present():
        return None
    exe = OUT / "ref_geometry"
    src = HERE / "ref_harness" / "ref_geometry.cu"
    if not force and exe.exists() and exe.stat().st_mtime > src.stat().st_mtime:
        return exe
    OUT.mkdir(exist_ok=True)
    cmd = [_nvcc(), "-std=c++17", "-O2", "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a",
           "-I", str(REF_SRC), "-I", str(REF_SRC.parent), '-DID_SIM="000"', "-w", str(src), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference geometry harness failed to build:\n{' '.join(cmd)}\n{r.stderr}")
    return exe


def build_ref_geometry_zwall(force: bool = False) -> Path | None:
    if not reference_present():
        return None
    exe = OUT / "ref_geometry_zwall"
    src = HERE / "ref_harness" / "ref_geometry.cu"
    if not force and exe.exists() and exe.stat().st_mtime > src.stat().st_mtime:
        return exe
    OUT.mkdir(exist_ok=True)
    with tempfile.TemporaryDirectory() as td:
        tree = Path(td) / "src"
        shutil.copytree(REF_SRC, tree, ignore=shutil.ignore_patterns("*.o"))
        consts = tree / "cases" / "cylinder" / "constants.cuh"
        lines = consts.read_text().split("\n")
        hits = [i for i, ln in enumerate(lines) if ln.strip().startswith("#define Z_PERIODIC 1")]
        if len(hits) != 1:
            raise RuntimeError("cannot find the Z_PERIODIC switch in cases/cylinder/constants.cuh")
        lines[hits[0]] = "#define Z_PERIODIC 0"
        consts.write_text("\n".join(lines))
        cmd = [_nvcc(), "-std=c++17", "-O2", "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a",
               "-I", str(tree), "-I", str(REF_SRC.parent), '-DID_SIM="000"', "-w", str(src), "-o", str(exe)]
        r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference z-wall geometry harness failed to build:\n{' '.join(cmd)}\n{r.stderr}")
    return exe


def build(force: bool = False) -> dict:
    return {"ref_geometry": build_ref_geometry(force), "ref_geometry_zwall": build_ref_geometry_zwall(force)}


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
