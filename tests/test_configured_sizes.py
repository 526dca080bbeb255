"""Oracle parity at the configured sizes of the cylinder (C1) and annulus (C3) workloads.

C1 as configured: 128 x 64 x 32 cylinder, D = 16 at (32, 32), U = 0.05, Re = 100, velocity
inlet, zero-gradient outlet, no-slip y walls, periodic z, rho = 1 and u = 0 at start,
2000 steps, forces every step.  C3 as configured: annulus 160 x 160 x 128, r = 32 / 64
about (79.5, 79.5), inner wall 0.05, outer fixed, Re = 400 on the gap; 300 steps (the CPU
oracle's share of a test), torque on both walls every step.

Criteria: every field within max(1e-5, 2 e32) of the FP32 oracle in the scaled metric of
conftest.field_errors, e32 being the FP32 oracle's own distance from the FP64 oracle (the
reference algorithm's FP32 rounding); the plain ||a - b||inf / ||b||inf within max(1e-5,
2 e32_plain).  Forces (FP64 sums here, FP32 in the oracle's reference order): per step within
0.5% of the drag (C1) or of the inner-wall torque (C3), and the C1 drag and lift coefficient
means over the last 500 steps within 0.5% of the FP32 oracle's."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import field_errors, record_parity

pytestmark = pytest.mark.gpu


def _oracle_run(desc, steps, bits, kind):
    import oracle
    o = oracle.Oracle(desc, bits)
    o.init(kind)
    f = np.zeros((steps, 2, 5))
    for s in range(steps):
        o.step(1, forces=True)
        f[s] = o.forces()
    m = o.moments().reshape(10, -1)
    o.close()
    return m, f


def _gpu_run(desc, steps, kind):
    from mrlbm_3d_cuda_gb300 import Simulation
    sim = Simulation(desc, init=False)
    sim.init(kind)
    sim.set_sampling(1, 0)
    sim.step(steps)
    sim.sync()
    m = sim.moments().reshape(10, -1)
    st, f = sim.force_history()
    sim.close()
    assert list(st) == list(range(steps))
    return m, f


def _fields(name, m, o32, o64, u):
    errs = field_errors(m, o32, u)
    e = field_errors(o32, o64, u)
    record_parity(name, errs, e32=e[:, 0], e32_plain=e[:, 1])
    table = ("\n gpu-o32 " + np.array2string(errs[:, 0], precision=2) + "\n e32     " +
             np.array2string(e[:, 0], precision=2) + "\n plain   " + np.array2string(errs[:, 1], precision=2) +
             "\n e32pl   " + np.array2string(e[:, 1], precision=2))
    assert (errs[:, 0] <= np.maximum(1e-5, 2.0 * e[:, 0])).all(), table
    assert (errs[:, 1] <= np.maximum(1e-5, 2.0 * e[:, 1])).all(), table


def test_c1_as_configured_matches_oracle(cuda_device):
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.c1_cylinder()
    steps = 2000
    m, f = _gpu_run(desc, steps, N.INIT_REST)
    o32, f32 = _oracle_run(desc, steps, 32, N.INIT_REST)
    o64, _ = _oracle_run(desc, steps, 64, N.INIT_REST)
    _fields("c1_2000_vs_fp32_oracle", m, o32, o64, 0.05)
    fx, fy = f[:, 0, 0], f[:, 0, 1]
    gx, gy = f32[:, 0, 0], f32[:, 0, 1]
    developed = np.abs(gx) > 0.2 * np.abs(gx).max()
    assert np.all(np.abs(fx - gx)[developed] <= 5e-3 * np.abs(gx[developed]))
    assert np.all(np.abs(fy - gy)[developed] <= 5e-3 * np.abs(gx[developed]))
    q = 0.5 * 0.05 ** 2 * 16 * 32
    cd, cd32 = fx[-500:].mean() / q, gx[-500:].mean() / q
    cl, cl32 = fy[-500:] / q, gy[-500:] / q
    assert abs(cd / cd32 - 1) <= 5e-3, (cd, cd32)
    assert abs(cl.mean() - cl32.mean()) <= 5e-3 * abs(cd32), (cl.mean(), cl32.mean())


def test_c3_as_configured_matches_oracle(cuda_device):
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.c3_annulus()
    steps = 300
    m, f = _gpu_run(desc, steps, N.INIT_REST)
    o32, f32 = _oracle_run(desc, steps, 32, N.INIT_REST)
    o64, _ = _oracle_run(desc, steps, 64, N.INIT_REST)
    _fields("c3_300_vs_fp32_oracle", m, o32, o64, 0.05)
    t, t32 = f[:, :, 4], f32[:, :, 4]  # torque_z of both walls
    developed = np.abs(t32[:, 0]) > 0.2 * np.abs(t32[:, 0]).max()
    for w in (0, 1):
        assert np.all(np.abs(t[:, w] - t32[:, w])[developed] <= 5e-3 * np.abs(t32[developed, 0])), w
