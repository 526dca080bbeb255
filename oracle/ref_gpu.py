"""Build and run the reference's own GPU solver (sakthi-lbm/MRLBM_3D_CUDA) as a parity and
timing baseline.  Test infrastructure only: nothing in the product imports this.

The reference has no tests or golden data, so parity of the time step is pinned by running
its own build on the GPU machine and comparing its checkpoint (restart.bin: iteration + the 10
moment arrays in its tiled IDX_BLOCK order, MRLBM_3D/src/restart/restart_io.cu:3-52) and
its forces.dat (MRLBM_3D/src/statistics/stat_header.cuh:16-33) with this solver's output
for the same case and step count.

Steps:
  stage  (where the reference tree is; its location comes from --reference or the
         MRLBM_REFERENCE environment variable: the directory that holds MRLBM_3D/)
         copy MRLBM_3D into baseline/_ref/<tag>/ and edit the copy for one of these runs:
           cylinder   the shipped case (cases/cylinder/*); only the run length and output
                      cadence in outputs.cuh change, plus optionally D or Z_PERIODIC 0 in
                      constants.cuh.  --shipped-run keeps the shipped MAX_ITER and statistics
                      window ((TSTAR + STAT_PERIOD) * SCALE = 56,000 steps, forces.dat over
                      48,000..56,000) and only moves the vti / checkpoint cadence out of the
                      run (they do not touch the state).
           annulus    the shipped annulus (cases/annulus/*) with the build fix it needs
                      (CASE_ID = CASE_ANNULUS; the h_rho_inlet globals and the
                      NEUMANN_CURRENT_UPDATE flag that shared headers read but only the
                      cylinder's constants define; saveData.cuh included by annulus_structs.h;
                      write_vti_annulus -> write_vti_3d_annulus), RESTART = 0 and the run
                      length / checkpoint cadence.
           tgv        the 3-D Taylor-Green vortex on an all-periodic n^3 grid, u0 = 0.05,
                      Re = 1600, L = n / 2 pi.  The reference has no such case: the cylinder
                      module is staged with every axis periodic, no outlet, no body (its
                      hooks replaced by no-ops, so every node stays NODE_BULK and the solver
                      kernels run their plain bulk path) and the initializer
                      (solver/initializeLBM.cu:51-58) writing the Taylor-Green field with
                      m_ab = u_a u_b.
         Every staged copy times its own stock loop: CUDA events (default stream) from the
         start of iteration start+5 to the end of the last iteration's collision, printed as
         `REF_LOOP_MS <ms> REF_LOOP_STEPS <n>`; the checkpoint and output calls that follow a
         step are outside that interval only for the last iteration.
  check  (on the GPU machine)  the reference kernels dereference host-allocated case structs
         (cases/cylinder/cylinder_kernels.cu:7-44 passes `new`-allocated structs to kernels),
         which is only valid where the GPU can access pageable host memory; refuse to run
         otherwise.
  build  (on the GPU machine)  one nvcc command over the copy's .cu files, as its compile.sh does
         (MRLBM_3D/compile.sh:43-54), for sm_103a; several tags build concurrently.
  run    (on the GPU machine)  run the binary in baseline/_ref/<tag>/run[<k>]/.

baseline/_ref/ is git-ignored and travels to the GPU machine with the working tree.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
STAGE = ROOT / "baseline" / "_ref"
BIG = 1 << 30

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


def reference_tree(arg: str | None) -> Path:
    loc = arg or os.environ.get("MRLBM_REFERENCE")
    if not loc:
        raise SystemExit("give the reference checkout (the directory holding MRLBM_3D/) with --reference "
                         "or the MRLBM_REFERENCE environment variable")
    tree = Path(loc) / "MRLBM_3D"
    if not (tree / "src" / "main.cu").is_file():
        raise SystemExit(f"{tree} is not the reference's MRLBM_3D tree")
    return tree


def _edit(path: Path, old: str, new: str):
    """Replace the one line whose stripped text starts with `old` by `new`."""
    lines = path.read_text().split("\n")
    hits = [i for i, ln in enumerate(lines) if ln.strip().startswith(old)]
    if len(hits) != 1:
        raise SystemExit(f"{path}: expected exactly one line starting with '{old}', found {len(hits)}")
    lines[hits[0]] = new
    path.write_text("\n".join(lines))


def _append(path: Path, text: str):
    path.write_text(path.read_text() + "\n" + text + "\n")


def _loop_timer(src: Path):
    """CUDA events around the stock loop of main.cu (src/main.cu:21-35)."""
    main = src / "main.cu"
    _edit(main, "restart_simulation(sim);",
          "    restart_simulation(sim);\n"
          "    cudaEvent_t ref_t0, ref_t1;\n"
          "    cudaEventCreate(&ref_t0);\n"
          "    cudaEventCreate(&ref_t1);")
    _edit(main, "streaming(sim, iter);",
          "        if (iter == sim.start_iter + 5) cudaEventRecord(ref_t0);\n"
          "        streaming(sim, iter);")
    _edit(main, "post_step_pipeline(sim, iter);",
          "        if (iter == MAX_ITER) cudaEventRecord(ref_t1);\n"
          "        post_step_pipeline(sim, iter);")
    _edit(main, "finalize_simulation(sim);",
          "    cudaEventSynchronize(ref_t1);\n"
          "    {\n"
          "        float ref_ms = 0.f;\n"
          "        cudaEventElapsedTime(&ref_ms, ref_t0, ref_t1);\n"
          "        printf(\"REF_LOOP_MS %.6f REF_LOOP_STEPS %d\\n\", ref_ms, MAX_ITER - sim.start_iter - 4);\n"
          "    }\n"
          "    finalize_simulation(sim);")


def _stage_cylinder(src: Path, a) -> dict:
    out = src / "cases" / "cylinder" / "outputs.cuh"
    _edit(out, "constexpr int MACR_SAVE = 5000;", f"constexpr int MACR_SAVE = {BIG};")
    if a.shipped_run:
        _edit(out, "constexpr int CHECKPOINT_SAVE = MACR_SAVE;", f"constexpr int CHECKPOINT_SAVE = {BIG};")
    else:
        _edit(out, "constexpr int MAX_ITER = (TSTAR + STAT_PERIOD) * SCALE;", f"constexpr int MAX_ITER = {a.steps};")
        _edit(out, "constexpr int STAT_START = TSTAR * SCALE;",
              f"constexpr int STAT_START = {BIG if a.no_stats else 0};")
        _edit(out, "constexpr int CHECKPOINT_SAVE = MACR_SAVE;",
              f"constexpr int CHECKPOINT_SAVE = {BIG if a.no_checkpoint else a.steps};")
    consts = src / "cases" / "cylinder" / "constants.cuh"
    if a.diameter is not None:
        _edit(consts, "constexpr int D = 16;", f"constexpr int D = {a.diameter};")
    if a.z_walls:
        _edit(consts, "#define Z_PERIODIC 1", "#define Z_PERIODIC 0")
    return {"diameter": a.diameter or 16, "z_walls": bool(a.z_walls), "shipped_run": bool(a.shipped_run),
            "steps": 56000 if a.shipped_run else a.steps}


def _stage_annulus(src: Path, a) -> dict:
    _edit(src / "config.h", "#define CASE_ID CASE_CYLINDER", "#define CASE_ID CASE_ANNULUS")
    ann = src / "cases" / "annulus"
    _append(ann / "constants.cuh", "inline real h_rho_inlet = 1.0, h_rho_inlet_average = 0.0;\n"
                                   "constexpr bool NEUMANN_CURRENT_UPDATE = false;")
    _edit(ann / "annulus_structs.h", '#include "../../boundary/curvedLBM.cuh"',
          '#include "../../boundary/curvedLBM.cuh"\n#include "../../output/saveData.cuh"')
    _edit(ann / "annulus_kernels.cu", "write_vti_annulus(sim.h_fMom, iter);",
          "    write_vti_3d_annulus(sim.h_fMom, iter);")
    out = ann / "outputs.cuh"
    _edit(out, "constexpr bool RESTART = 1;", "constexpr bool RESTART = 0;")
    _edit(out, "constexpr int MAX_ITER = num_cycle", f"constexpr int MAX_ITER = {a.steps};")
    _edit(out, "constexpr int MACR_SAVE = MAX_ITER / 50;", f"constexpr int MACR_SAVE = {BIG};")
    _edit(out, "constexpr int STAT_START = MAX_ITER - STAT_PERIOD;", f"constexpr int STAT_START = {BIG};")
    _edit(out, "constexpr int CHECKPOINT_SAVE = MACR_SAVE;",
          f"constexpr int CHECKPOINT_SAVE = {BIG if a.no_checkpoint else a.steps};")
    if a.z_walls:
        _edit(ann / "constants.cuh", "#define Z_PERIODIC 1", "#define Z_PERIODIC 0")
    return {"z_walls": bool(a.z_walls), "steps": a.steps}


def _stage_tgv(src: Path, a) -> dict:
    n = a.n
    cyl = src / "cases" / "cylinder"
    c = cyl / "constants.cuh"
    _edit(c, "#define X_PERIODIC 0", "#define X_PERIODIC 1")
    _edit(c, "#define CONVECTIVE_OUTLET 1", "#define CONVECTIVE_OUTLET 0")
    for ax in ("NX", "NY", "NZ"):
        _edit(c, f"constexpr int {ax} =", f"constexpr int {ax} = {n};")
    _edit(c, "constexpr real RE = 100;", "constexpr real RE = 1600;")
    _edit(c, "constexpr real U_MAX = 0.1;", "constexpr real U_MAX = 0.05;")
    _edit(c, "constexpr real VISC = U_MAX * D_WALL / RE;",
          "constexpr real VISC = U_MAX * (toReal(NX) / (toReal(2.0) * toReal(3.14159265358979323846))) / RE;")
    case = cyl / "cylinder_case.cu"
    _edit(case, "case_module.initialize = cylinder_initialize;", "    case_module.initialize = [](Simulation &) {};")
    for hook in ("apply_boundary", "post_streaming", "post_collision", "post_process_step", "write_output",
                 "free_case"):
        _edit(case, f"case_module.{hook} =", f"    case_module.{hook} = nullptr;")
    init = src / "solver" / "initializeLBM.cu"
    _edit(init, "real rho = RHO_0;",
          "    const double tgv_L = (double)NX / (2.0 * 3.14159265358979323846);\n"
          "    const double tgv_u0 = (double)U_MAX;\n"
          "    const double tgv_X = x / tgv_L, tgv_Y = y / tgv_L, tgv_Z = z / tgv_L;\n"
          "    const double tgv_u = tgv_u0 * sin(tgv_X) * cos(tgv_Y) * cos(tgv_Z);\n"
          "    const double tgv_v = -tgv_u0 * cos(tgv_X) * sin(tgv_Y) * cos(tgv_Z);\n"
          "    const double tgv_p = (double)RHO_0 * tgv_u0 * tgv_u0 / 16.0 * (cos(2.0 * tgv_X) + cos(2.0 * tgv_Y)) *"
          " (cos(2.0 * tgv_Z) + 2.0);\n"
          "    real rho = (real)((double)RHO_0 + 3.0 * tgv_p);")
    _edit(init, "real ux = toReal(0.0);", "    real ux = (real)tgv_u;")
    _edit(init, "real uy = toReal(0.0);", "    real uy = (real)tgv_v;")
    _edit(init, "real uz = 1e-4 * U_MAX * sin(", "    real uz = toReal(0.0);")
    _edit(init, "get_noise(idx + 67890, noise_scale);", "")
    _edit(init, "myz *= inv_rho;",
          "    myz *= inv_rho;\n"
          "    mxx = (real)(tgv_u * tgv_u);\n"
          "    myy = (real)(tgv_v * tgv_v);\n"
          "    mzz = toReal(0.0);\n"
          "    mxy = (real)(tgv_u * tgv_v);\n"
          "    mxz = toReal(0.0);\n"
          "    myz = toReal(0.0);")
    out = cyl / "outputs.cuh"
    _edit(out, "constexpr int MACR_SAVE = 5000;", f"constexpr int MACR_SAVE = {BIG};")
    _edit(out, "constexpr int MAX_ITER = (TSTAR + STAT_PERIOD) * SCALE;", f"constexpr int MAX_ITER = {a.steps};")
    _edit(out, "constexpr int STAT_START = TSTAR * SCALE;", f"constexpr int STAT_START = {BIG};")
    _edit(out, "constexpr int CHECKPOINT_SAVE = MACR_SAVE;",
          f"constexpr int CHECKPOINT_SAVE = {BIG if a.no_checkpoint else a.steps};")
    return {"n": n, "steps": a.steps, "u0": 0.05, "re": 1600.0}


def stage(a):
    tree = reference_tree(a.reference)
    dst = STAGE / a.tag
    if dst.exists():
        shutil.rmtree(dst)
    shutil.copytree(tree, dst / "MRLBM_3D", ignore=shutil.ignore_patterns("*.o", "OUTPUT"))
    src = dst / "MRLBM_3D" / "src"
    cfg = {"cylinder": _stage_cylinder, "annulus": _stage_annulus, "tgv": _stage_tgv}[a.case](src, a)
    _loop_timer(src)
    cfg.update({"tag": a.tag, "case": a.case})
    (dst / "config.json").write_text(json.dumps(cfg))
    print(f"staged {dst}: {cfg}")


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


def _build_one(tag: str, arch: str) -> str:
    base = STAGE / tag / "MRLBM_3D"
    srcs = sorted(str(p.relative_to(base)) for p in (base / "src").rglob("*.cu"))
    cmd = ["nvcc", "-std=c++17", f"-gencode=arch=compute_{arch},code=sm_{arch}", "-rdc=true", "-O3", "--restrict",
           "-I.", "-Iinclude", "-Isrc", "-Isolver", f'-DID_SIM="{tag}"', "-w", *srcs, "-lcudadevrt",
           "-o", str(STAGE / tag / "refsim")]
    r = subprocess.run(cmd, cwd=base, capture_output=True, text=True)
    if r.returncode != 0:
        raise SystemExit(f"reference build {tag} failed:\n{r.stderr[-4000:]}")
    return f"built {STAGE / tag / 'refsim'}"


def build(tags: list[str], arch: str = "103a"):
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=max(1, len(tags))) as ex:
        for msg in ex.map(lambda t: _build_one(t, arch), tags):
            print(msg)


def run(tag: str, k: int = 0) -> Path:
    d = STAGE / tag
    rd = d / ("run" if k == 0 else f"run{k}")
    if rd.exists():
        shutil.rmtree(rd)
    rd.mkdir()
    with open(rd / "log.txt", "w") as log:
        subprocess.run([str(d / "refsim")], cwd=rd, check=True, stdout=log, stderr=subprocess.STDOUT)
    text = (rd / "log.txt").read_text()
    m = re.search(r"REF_LOOP_MS ([0-9.]+) REF_LOOP_STEPS ([0-9]+)", text)
    if m:
        (rd / "loop_time.json").write_text(json.dumps({"ms": float(m.group(1)), "steps": int(m.group(2))}))
    print(text[-1500:])
    return rd


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    s = sub.add_parser("stage")
    s.add_argument("tag")
    s.add_argument("--case", choices=("cylinder", "annulus", "tgv"), default="cylinder")
    s.add_argument("--reference", help="directory holding the reference's MRLBM_3D/ (else $MRLBM_REFERENCE)")
    s.add_argument("--steps", type=int, default=0, help="MAX_ITER: iterations 0..steps are run")
    s.add_argument("--shipped-run", action="store_true",
                   help="cylinder: keep the shipped MAX_ITER and statistics window")
    s.add_argument("--no-stats", action="store_true")
    s.add_argument("--no-checkpoint", action="store_true")
    s.add_argument("--diameter", type=int)
    s.add_argument("--z-walls", action="store_true", help="build with Z_PERIODIC 0 (BCSOLID nodes)")
    s.add_argument("--n", type=int, default=256, help="tgv: grid edge")
    sub.add_parser("check")
    b = sub.add_parser("build")
    b.add_argument("tags", nargs="+")
    r = sub.add_parser("run")
    r.add_argument("tag")
    r.add_argument("--repeat", type=int, default=0, help="run index (run/, run1/, ...)")
    a = ap.parse_args()
    if a.cmd == "stage":
        if not a.shipped_run and a.steps <= 0:
            raise SystemExit("--steps is required")
        stage(a)
    elif a.cmd == "check":
        check()
    elif a.cmd == "build":
        build(a.tags)
    else:
        run(a.tag, a.repeat)


if __name__ == "__main__":
    sys.exit(main())
