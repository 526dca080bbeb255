"""Parity against the reference's own solver build, run on a GB300.

Fixtures (tests/golden/ref_cylinder_run_n*.npz, made by tests/golden/make_ref_run_golden.py
from runs of the reference build staged by oracle/ref_gpu.py) hold the reference's state
after N + 1 steps of its shipped cylinder case (336 x 144 x 48, D = 16, Re = 100, U = 0.1,
periodic y and z, convective outlet) from its own initial state: all 10 moments at every
non-bulk node plus 40,000 random nodes, whole-grid field statistics, and its forces.dat.
ref_cylinder_zwall_run_n160.npz is the same case built with Z_PERIODIC 0: no-slip z faces
and the BCSOLID nodes where they meet the cylinder (boundaries.cuh:1039-1214).

Criteria (per field, metric of conftest.field_errors; s_f = 1 for rho, U for u, cs2 for m):
  * 11 steps: <= 1e-5 against the reference build;
  * 161 steps (the inlet pressure wave has reached the cylinder): within max(1e-5, 2 e32)
    of the reference build, e32 being the FP32 oracle's distance from the FP64 oracle on the
    same nodes (FP32 rounding of the reference's own arithmetic);
  * forces.dat: Fx within 0.5 % (the stated Cd tolerance) once the drag is developed, Fy
    within 0.5 % of |Fx| (Cl on the drag scale);
  * whole-grid max |m| and sum m^2 of the fields that carry the flow (rho, ux, uy, mxx, myy,
    mxy) within 1e-4 relative; uz, mzz, mxz, myz only hold the 1e-5 U seed noise of this
    2-D flow, whose whole-grid statistics are FP32-rounding dominated."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, field_errors

pytestmark = pytest.mark.gpu
U = 0.1
SIGNAL = [0, 1, 2, 4, 5, 7]


def tiled_to_lex(idx: np.ndarray, nx: int, ny: int, nz: int) -> np.ndarray:
    """Reference tiled IDX_BLOCK index (core/index.cuh:11-28, 8 x 8 x 4 blocks) -> x + nx (y + ny z)."""
    idx = idx.astype(np.int64)
    gx, gy = nx // 8, ny // 8
    block, thread = idx // 256, idx % 256
    bx, by, bz = block % gx, (block // gx) % gy, block // (gx * gy)
    x, y, z = bx * 8 + thread % 8, by * 8 + (thread // 8) % 8, bz * 4 + thread // 64
    return x + nx * (y + ny * z)


def run_ours(steps: int, periodic_z: bool = True):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    sim = Simulation(cases.reference_cylinder(periodic_z=periodic_z), init=False)
    sim.init(N.INIT_REFERENCE_NOISE)
    sim.set_sampling(1, 0)
    sim.step(steps)
    sim.sync()
    m = sim.moments(layout=N.LAYOUT_REF_TILED)
    st, f = sim.force_history()
    sim.close()
    return m, st, f


def check_common(g, m, st, f):
    m64 = m.astype(np.float64)
    for k in SIGNAL:
        assert abs(np.abs(m64[k]).max() / g["field_max"][k] - 1) < 1e-4, k
        assert abs((m64[k] ** 2).sum() / g["field_sumsq"][k] - 1) < 1e-4, k
    ref = g["forces"]
    assert list(st) == list(ref[:, 0].astype(np.int64))
    fx, fy = f[:, 0, 0], f[:, 0, 1]
    developed = np.abs(ref[:, 1]) > 1.0
    if developed.any():
        assert np.all(np.abs(fx - ref[:, 1])[developed] <= 5e-3 * np.abs(ref[developed, 1]))
        assert np.all(np.abs(fy - ref[:, 2])[developed] <= 5e-3 * np.abs(ref[developed, 1]))


def test_eleven_steps_match_reference_build(cuda_device):
    g = np.load(GOLDEN / "ref_cylinder_run_n10.npz")
    m, st, f = run_ours(int(g["steps"]))
    err = field_errors(m[:, g["idx"]], g["moments"], U)[:, 0]
    assert err.max() <= 1e-5, np.array2string(err, precision=3)
    check_common(g, m, st, f)


@pytest.mark.parametrize("fixture", ["ref_cylinder_run_n160.npz", "ref_cylinder_zwall_run_n160.npz"])
def test_161_steps_match_reference_build(cuda_device, fixture):
    import oracle
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    g = np.load(GOLDEN / fixture)
    steps = int(g["steps"])
    periodic_z = not int(g.get("z_walls", 0))
    m, st, f = run_ours(steps, periodic_z)
    idx = g["idx"]
    orc = {}
    for bits in (32, 64):
        o = oracle.Oracle(cases.reference_cylinder(periodic_z=periodic_z), bits)
        o.init(N.INIT_REFERENCE_NOISE)
        o.step(steps)
        orc[bits] = o.moments().reshape(10, -1)[:, tiled_to_lex(idx, *g["nxyz"])]
        o.close()
    e32 = field_errors(orc[32], orc[64], U)[:, 0]
    err = field_errors(m[:, idx], g["moments"], U)[:, 0]
    table = "\n gpu-ref " + np.array2string(err, precision=2) + "\n o32-o64 " + np.array2string(e32, precision=2)
    assert (err <= np.maximum(1e-5, 2.0 * e32)).all(), table
    check_common(g, m, st, f)
