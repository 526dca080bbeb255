"""Full-size checks through size-independent properties: the oracle cannot follow a 256^3 or
1024 x 512 x 256 grid in a test's time, so these runs are checked against what any correct
step must satisfy at every size.

* Shift invariance, bit for bit: on an all-periodic box the step commutes with a periodic
  shift of the field.  The shift moves nodes between tiles, between owner and rim columns
  and across the x-blocks of the storage layout, so every one of those paths must round
  identically.
* Conservation: total mass (FP64 diagnostics over all nodes) changes only by FP32 rounding.
* Taylor-Green decay (256^3): the kinetic energy decays at 2 nu k^2, k^2 = 3 / L^2, like the
  oracle's own known-answer test at 32^3: within 3% with FP32 storage.  With FP16 storage the
  rate comes out 13.5% low (measured on a GB300).  The likely cause: at this grid size the
  viscous stress is about 1% of the stored m_ab ~ u_a u_b, so FP16's 2^-11 relative rounding
  of m is a few percent of the stress, and on a smooth field the rounding errors are spatially
  correlated rather than averaging out.  The FP16 bound is 20%.  With stochastic rounding the
  rounding errors are independent and FP16 decays like FP32 (measured +0.19%, FP32 +0.23%):
  bound 3%.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHIFT = (3, 37, 45)  # (z, y, x): not a multiple of the 32-node x-block or the 16-row tile


def shifted_pair(desc, init, params, steps):
    from mrlbm_3d_cuda_gb300 import Simulation
    a = Simulation(desc, init=False)
    a.init(init, params)
    m0 = a.moments()
    a.set_moments(m0)  # both runs start from values that went through the same encoding
    b = Simulation(desc, init=False)
    b.init(init, params)
    b.set_moments(np.roll(m0, SHIFT, axis=(1, 2, 3)))
    del m0
    a.set_sampling(0, 1)
    a.step(steps)
    b.step(steps)
    ma = a.moments()
    same = np.array_equal(np.roll(ma, SHIFT, axis=(1, 2, 3)), b.moments())
    _, diag = a.diagnostics()
    a.close()
    b.close()
    return same, diag


@pytest.mark.parametrize("storage", ["f32", "f16", "f16sr"])
def test_taylor_green_256_shift_invariance_conservation_decay(cuda_device, storage):
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    st = N.STORAGE_F32 if storage == "f32" else N.STORAGE_F16
    desc = cases.periodic_box(256, u0=0.05, re=100.0, storage=st)
    desc.stochastic_rounding = int(storage == "f16sr")
    steps = 250
    same, diag = shifted_pair(desc, N.INIT_TAYLOR_GREEN, cases.tgv_params(desc), steps)
    # stochastic rounding keys its random bits on the absolute node index: no shift symmetry
    assert same or storage == "f16sr", "the step does not commute with a periodic shift"
    n = 256 ** 3
    mass, energy = diag[:, 0], diag[:, 1]
    # FP32 weights sum to 1 within a few ulp: the mean density may drift ~3e-7 per step
    assert abs(mass[-1] - mass[0]) / n < 1e-6 * steps
    nu = (1.0 / desc.omega - 0.5) / 3.0
    want = 2.0 * nu * 3.0 / desc.length ** 2
    rate = -math.log(energy[-1] / energy[50]) / (len(energy) - 1 - 50)
    assert abs(rate - want) / want < (0.20 if storage == "f16" else 0.03), (rate, want)


def test_largest_single_gpu_grid_shift_invariance(cuda_device):
    """The largest benchmark grid (1024 x 512 x 256, 134 M nodes) with FP16 storage."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.periodic_box(1024, 512, 256, u0=0.05, re=3900.0, storage=N.STORAGE_F16)
    steps = 12
    same, diag = shifted_pair(desc, N.INIT_NOISY_UNIFORM, (0.05, 0.0, 0.0, 0.01, 1234), steps)
    assert same, "the step does not commute with a periodic shift"
    assert np.isfinite(diag).all()
    assert abs(diag[-1, 0] - diag[0, 0]) / (1024 * 512 * 256) < 1e-6 * steps


C2_STORAGE = {"f32": (0, 0), "f16": (1, 0), "f16sr": (1, 1), "bf16": (2, 0), "bf16sr": (2, 1), "f16u32": (3, 0),
              "f16u32sr": (3, 1)}
# max over t of |E/E64 - 1| and of |eps - eps64| / max eps64 (eps = -dE/dt over 50 steps),
# about three times the GB300 measurement: FP32 4.7e-6 / 3.8e-5, FP16 6.4e-3 / 0.144, FP16 sr
# 3.2e-4 / 2.2e-3, BF16 0.198 / 3.08 (its decay goes wrong: bounded only against breakage),
# BF16 sr 2.0e-4 / 1.2e-2, hybrid (FP32 u, FP16 rho and m) 7.0e-6 / 1.3e-4, hybrid sr
# 1.4e-6 / 2.3e-5 (a single stochastic draw: ten times)
C2_BOUND = {"f32": (1.5e-5, 1.2e-4), "f16": (2e-2, 0.45), "f16sr": (1e-3, 7e-3), "bf16": (0.6, 10.0),
            "bf16sr": (6e-4, 4e-2), "f16u32": (2.5e-5, 4e-4), "f16u32sr": (1.5e-5, 2.5e-4)}


@pytest.mark.parametrize("storage", list(C2_STORAGE))
def test_c2_energy_and_dissipation_against_fp64(cuda_device, storage):
    """C2 as configured: Taylor-Green 256^3, u0 = 0.05, Re = 1600, 5000 steps, E(t) =
    sum |u|^2 / 2 and its decay rate eps(t) every 50 steps against the FP64 oracle run of the
    same field (tests/golden/tgv256_fp64_energy.npz, made by make_tgv_energy_golden.py)."""
    from conftest import GOLDEN, _PARITY_LOG
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    path = GOLDEN / "tgv256_fp64_energy.npz"
    if not path.exists():
        pytest.skip("FP64 energy fixture not generated")
    g = np.load(path)
    steps, e64 = g["steps"], g["energy"]
    every = int(steps[1] - steps[0])
    st, sr = C2_STORAGE[storage]
    desc = cases.c2_taylor_green(256, st)
    desc.stochastic_rounding = sr
    sim = Simulation(desc, init=False)
    sim.init(N.INIT_TAYLOR_GREEN, cases.tgv_params(desc))
    m0 = sim.moments().reshape(10, -1).astype(np.float64)
    e = [0.5 * float((m0[1] ** 2 + m0[2] ** 2 + m0[3] ** 2).sum())]
    del m0
    for _ in steps[1:]:
        sim.set_sampling(0, 0)
        sim.step(every - 1)
        sim.set_sampling(0, 1)
        sim.step(1)  # its sample is the state after these steps
    sim.sync()
    _, diag = sim.diagnostics()
    sim.close()
    e = np.array(e + list(diag[-(len(steps) - 1):, 1]))
    eps, eps64 = -np.diff(e) / every, -np.diff(e64) / every
    e_err = float(np.abs(e / e64 - 1).max())
    eps_err = float((np.abs(eps - eps64) / np.abs(eps64).max()).max())
    _PARITY_LOG[f"c2_energy_{storage}"] = {"max_rel_E": e_err, "max_rel_eps": eps_err,
                                           "E_end_rel": float(e[-1] / e64[-1] - 1)}
    assert e_err < C2_BOUND[storage][0] and eps_err < C2_BOUND[storage][1], (storage, e_err, eps_err)
