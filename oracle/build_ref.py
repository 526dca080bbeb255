"""Recipe that compiles pieces of the reference (sakthi-lbm/MRLBM_3D_CUDA) from its own
sources, where they lie, into oracle/_ref/ — test infrastructure only.

* ``ref_geometry``: a host-only program (no GPU) that runs the reference's own node
  classification for its shipped cylinder case and dumps the result (see
  ref_harness/ref_geometry.cu).  Built when MRLBM_REFERENCE names the reference checkout
  (the directory that holds MRLBM_3D/); where it is unset nothing here is built or used.
* ``ref_geometry_annulus``: the annulus case's classification for both walls
  (ref_harness/ref_geometry_annulus.cu).  The reference selects the case at compile time
  (``#define CASE_ID`` in config.h:8), and its annulus case does not compile as shipped:
  statistics/stat_header.cuh reads ``h_rho_inlet`` / ``h_rho_inlet_average``, which only the
  cylinder's constants define.  The staged copy sets CASE_ID to CASE_ANNULUS and adds those
  two host globals to cases/annulus/constants.cuh; nothing else changes.
* ``ref_geometry_staircase``: the cylinder harness with ``triangular = false``
  (cases/cylinder/constants.cuh:15): the staircase classification.
* ``ref_geometry_annulus_zwall``: the same with ``#define Z_PERIODIC 0`` in the annulus
  constants (BCSOLID nodes on both walls).
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


def _ref_src() -> Path | None:
    """The reference's MRLBM_3D/src, from the MRLBM_REFERENCE environment variable (the
    directory holding MRLBM_3D/); None when it is unset."""
    loc = os.environ.get("MRLBM_REFERENCE")
    return Path(loc) / "MRLBM_3D" / "src" if loc else None


def reference_present() -> bool:
    src = _ref_src()
    return src is not None and (src / "main.cu").exists()


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
           "-I", str(_ref_src()), "-I", str(_ref_src().parent), '-DID_SIM="000"', "-w", str(src), "-o", str(exe)]
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
        shutil.copytree(_ref_src(), tree, ignore=shutil.ignore_patterns("*.o"))
        consts = tree / "cases" / "cylinder" / "constants.cuh"
        lines = consts.read_text().split("\n")
        hits = [i for i, ln in enumerate(lines) if ln.strip().startswith("#define Z_PERIODIC 1")]
        if len(hits) != 1:
            raise RuntimeError("cannot find the Z_PERIODIC switch in cases/cylinder/constants.cuh")
        lines[hits[0]] = "#define Z_PERIODIC 0"
        consts.write_text("\n".join(lines))
        cmd = [_nvcc(), "-std=c++17", "-O2", "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a",
               "-I", str(tree), "-I", str(_ref_src().parent), '-DID_SIM="000"', "-w", str(src), "-o", str(exe)]
        r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference z-wall geometry harness failed to build:\n{' '.join(cmd)}\n{r.stderr}")
    return exe


def _staged_build(name: str, harness: str, edits, force: bool) -> Path | None:
    """Compile `harness` against a temporary copy of the reference's src/ with `edits`
    (relative path, old line start, new line or None to append) applied."""
    if not reference_present():
        return None
    exe = OUT / name
    src = HERE / "ref_harness" / harness
    if not force and exe.exists() and exe.stat().st_mtime > src.stat().st_mtime:
        return exe
    OUT.mkdir(exist_ok=True)
    with tempfile.TemporaryDirectory() as td:
        tree = Path(td) / "src"
        shutil.copytree(_ref_src(), tree, ignore=shutil.ignore_patterns("*.o"))
        for rel, old, new in edits:
            f = tree / rel
            lines = f.read_text().split("\n")
            if old is None:
                lines.append(new)
            else:
                hits = [i for i, ln in enumerate(lines) if ln.strip().startswith(old)]
                if len(hits) != 1:
                    raise RuntimeError(f"cannot find '{old}' in {rel}")
                lines[hits[0]] = new
            f.write_text("\n".join(lines))
        cmd = [_nvcc(), "-std=c++17", "-O2", "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a",
               "-I", str(tree), "-I", str(_ref_src().parent), '-DID_SIM="000"', "-w", str(src), "-o", str(exe)]
        r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference harness {name} failed to build:\n{' '.join(cmd)}\n{r.stderr}")
    return exe


def build_ref_geometry_annulus(force: bool = False) -> Path | None:
    return _staged_build("ref_geometry_annulus", "ref_geometry_annulus.cu", [
        ("config.h", "#define CASE_ID CASE_CYLINDER", "#define CASE_ID CASE_ANNULUS"),
        ("cases/annulus/constants.cuh", None, "inline real h_rho_inlet = 1.0, h_rho_inlet_average = 0.0;"),
    ], force)


def build_ref_geometry_annulus_zwall(force: bool = False) -> Path | None:
    return _staged_build("ref_geometry_annulus_zwall", "ref_geometry_annulus.cu", [
        ("config.h", "#define CASE_ID CASE_CYLINDER", "#define CASE_ID CASE_ANNULUS"),
        ("cases/annulus/constants.cuh", None, "inline real h_rho_inlet = 1.0, h_rho_inlet_average = 0.0;"),
        ("cases/annulus/constants.cuh", "#define Z_PERIODIC 1", "#define Z_PERIODIC 0"),
    ], force)


def build_ref_geometry_staircase(force: bool = False) -> Path | None:
    return _staged_build("ref_geometry_staircase", "ref_geometry.cu", [
        ("cases/cylinder/constants.cuh", "constexpr bool triangular = true;", "constexpr bool triangular = false;"),
    ], force)


def build(force: bool = False) -> dict:
    """Every harness variant, compiled concurrently (one nvcc each)."""
    from concurrent.futures import ThreadPoolExecutor
    jobs = {"ref_geometry": build_ref_geometry, "ref_geometry_zwall": build_ref_geometry_zwall,
            "ref_geometry_staircase": build_ref_geometry_staircase,
            "ref_geometry_annulus": build_ref_geometry_annulus,
            "ref_geometry_annulus_zwall": build_ref_geometry_annulus_zwall}
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        futures = {name: ex.submit(fn, force) for name, fn in jobs.items()}
        return {name: f.result() for name, f in futures.items()}


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
