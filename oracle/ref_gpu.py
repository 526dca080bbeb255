"""Build and run the reference's own GPU solver (sakthi-lbm/MRLBM_3D_CUDA) as a parity and
timing baseline.  Test infrastructure only: nothing in the product imports this.

The reference has no tests or golden data, so parity of the time step is pinned by running
its own build on the GPU machine and comparing its checkpoint (restart.bin: iteration + the 10
moment arrays in its tiled IDX_BLOCK order, MRLBM_3D/src/restart/restart_io.cu:3-52) and
its forces.dat (MRLBM_3D/src/statistics/stat_header.cuh:16-33) with this solver's output
for the same case and step count.

Steps:
  stage  (here, where the reference tree is)  copy MRLBM_3D into baseline/_ref/<tag>/ and set
         the run length and output cadence in the copy's cases/cylinder/outputs.cuh (and, in
         constants.cuh, the diameter for the larger timing case or Z_PERIODIC 0 for the
         z-wall case); nothing else is changed.
  check  (on the GPU machine)  the reference kernels dereference host-allocated case structs
         (cases/cylinder/cylinder_kernels.cu:7-44 passes `new`-allocated structs to kernels),
         which is only valid where the GPU can access pageable host memory; refuse to run
         otherwise.
  build  (on the GPU machine)  one nvcc command over the copy's .cu files, as its compile.sh does
         (MRLBM_3D/compile.sh:43-54), for sm_103a.
  run    (on the GPU machine)  run the binary in baseline/_ref/<tag>/run/.

baseline/_ref/ is git-ignored and travels to the GPU machine with the working tree.
"""
from __future__ import annotations

import argparse
import json
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
REF_TREE = Path("/root/reference/MRLBM_3D")
STAGE = ROOT / "baseline" / "_ref"

ATS_CHECK = r"""
#include <cstdio>
#include <cuda_runtime.h>
int main() {
    int pageable = 0, host_tables = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, 0) != cudaSuccess) return 2;
    if (cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, 0) != cudaSuccess)
        return 2;
    std::printf("pageableMemoryAccess=%d usesHostPageTables=%d\n", pageable, host_tables);
    return pageable ? 0 : 1;
}
"""


def _replace_once(path: Path, old: str, new: str):
    """Replace the one uncommented line that starts with `old`."""
    lines = path.read_text().split("\n")
    hits = [i for i, ln in enumerate(lines) if ln.strip().startswith(old)]
    if len(hits) != 1:
        raise SystemExit(f"{path}: expected exactly one line '{old}'")
    lines[hits[0]] = lines[hits[0]].replace(old, new)
    path.write_text("\n".join(lines))


def stage(tag: str, steps: int, stats: bool, checkpoint: bool, diameter: int | None, z_walls: bool = False):
    if not REF_TREE.is_dir():
        raise SystemExit("the reference tree is not available here; stage where it is")
    dst = STAGE / tag
    if dst.exists():
        shutil.rmtree(dst)
    shutil.copytree(REF_TREE, dst / "MRLBM_3D", ignore=shutil.ignore_patterns("*.o", "OUTPUT"))
    src = dst / "MRLBM_3D" / "src"
    out = src / "cases" / "cylinder" / "outputs.cuh"
    big = 1 << 30
    _replace_once(out, "constexpr int MACR_SAVE = 5000;", f"constexpr int MACR_SAVE = {big};")
    _replace_once(out, "constexpr int MAX_ITER = (TSTAR + STAT_PERIOD) * SCALE;", f"constexpr int MAX_ITER = {steps};")
    _replace_once(out, "constexpr int STAT_START = TSTAR * SCALE;",
                  f"constexpr int STAT_START = {0 if stats else big};")
    _replace_once(out, "constexpr int CHECKPOINT_SAVE = MACR_SAVE;",
                  f"constexpr int CHECKPOINT_SAVE = {steps if checkpoint else big};")
    if diameter is not None:
        _replace_once(src / "cases" / "cylinder" / "constants.cuh", "constexpr int D = 16;",
                      f"constexpr int D = {diameter};")
    if z_walls:
        _replace_once(src / "cases" / "cylinder" / "constants.cuh", "#define Z_PERIODIC 1", "#define Z_PERIODIC 0")
    cfg = {"tag": tag, "steps": steps, "stats": stats, "checkpoint": checkpoint, "diameter": diameter or 16,
           "z_walls": z_walls}
    (dst / "config.json").write_text(json.dumps(cfg))
    print(f"staged {dst}")


def check():
    STAGE.mkdir(parents=True, exist_ok=True)
    cu = STAGE / "ats_check.cu"
    cu.write_text(ATS_CHECK)
    exe = STAGE / "ats_check"
    subprocess.run(["nvcc", "-o", str(exe), str(cu)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    print(r.stdout.strip())
    if r.returncode != 0:
        raise SystemExit("GPU cannot access pageable host memory: the reference build would fault here")


def build(tag: str, arch: str = "103a"):
    base = STAGE / tag / "MRLBM_3D"
    srcs = sorted(str(p.relative_to(base)) for p in (base / "src").rglob("*.cu"))
    cmd = ["nvcc", "-std=c++17", f"-gencode=arch=compute_{arch},code=sm_{arch}", "-rdc=true", "-O3", "--restrict",
           "-I.", "-Iinclude", "-Isrc", "-Isolver", f'-DID_SIM="{tag}"', *srcs, "-lcudadevrt",
           "-o", str(STAGE / tag / "refsim")]
    subprocess.run(cmd, cwd=base, check=True, stdout=subprocess.DEVNULL)
    print(f"built {STAGE / tag / 'refsim'}")


def run(tag: str) -> Path:
    d = STAGE / tag
    rd = d / "run"
    if rd.exists():
        shutil.rmtree(rd)
    rd.mkdir()
    with open(rd / "log.txt", "w") as log:
        subprocess.run([str(d / "refsim")], cwd=rd, check=True, stdout=log, stderr=subprocess.STDOUT)
    print((rd / "log.txt").read_text()[-2000:])
    return rd


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    s = sub.add_parser("stage")
    s.add_argument("tag")
    s.add_argument("--steps", type=int, required=True)
    s.add_argument("--no-stats", action="store_true")
    s.add_argument("--no-checkpoint", action="store_true")
    s.add_argument("--diameter", type=int)
    s.add_argument("--z-walls", action="store_true", help="build with Z_PERIODIC 0 (BCSOLID nodes)")
    sub.add_parser("check")
    b = sub.add_parser("build")
    b.add_argument("tag")
    r = sub.add_parser("run")
    r.add_argument("tag")
    a = ap.parse_args()
    if a.cmd == "stage":
        stage(a.tag, a.steps, not a.no_stats, not a.no_checkpoint, a.diameter, a.z_walls)
    elif a.cmd == "check":
        check()
    elif a.cmd == "build":
        build(a.tag)
    else:
        run(a.tag)


if __name__ == "__main__":
    sys.exit(main())
