"""GPU parity: the CUDA solver (through the C ABI) against the oracle on the same inputs.

Tolerance: per field, max |gpu - oracle| / max(|oracle|_inf, s_f) <= 1e-5 after N steps,
with s_f the magnitude of the quantity as the FP32 algorithm computes it (rho: 1, u: U,
m_ab: cs2 = 1/3); see conftest.field_errors.  Forces: relative 5e-3 of |F| (the stated
Cd / Cl tolerance), in practice far tighter."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import field_errors

pytestmark = pytest.mark.gpu
TOL = 1e-5


def run_pair(desc, steps, init_kind, params=(), forces=False, bits=32):
    import oracle
    from mrlbm_3d_cuda_gb300 import Simulation
    sim = Simulation(desc, init=False)
    sim.init(init_kind, params)
    if forces:
        sim.set_sampling(1, 0)
    o = oracle.Oracle(desc, bits)
    o.init(init_kind, params)
    # initial states agree exactly (same initialiser arithmetic)
    g0 = sim.moments()
    o0 = o.moments()
    if bits == 32:
        assert np.array_equal(g0.astype(np.float64), o0), "initial state differs"
    for s in range(steps):
        sim.step(1)
        o.step(1, forces=forces and s == steps - 1)
    sim.sync()
    res = {"gpu": sim.moments(), "oracle": o.moments(), "types": sim.node_types()}
    if forces:
        res["gpu_f"] = sim.forces()
        res["oracle_f"] = o.forces()
    sim.close()
    o.close()
    return res


def assert_fields(res, u_ref, tol=TOL):
    err = field_errors(res["gpu"], res["oracle"], u_ref)
    assert np.isfinite(res["gpu"]).all()
    assert err[:, 0].max() < tol, "\n" + np.array2string(err, precision=3)
    return err


def test_reference_noise_initialiser_is_bitwise(cuda_device):
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    res = run_pair(cases.reference_cylinder(), 0, N.INIT_REFERENCE_NOISE)
    assert np.array_equal(res["gpu"].astype(np.float64), res["oracle"])


def test_taylor_green_periodic(cuda_device):
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.periodic_box(32, u0=0.05, re=400.0)
    res = run_pair(desc, 30, N.INIT_TAYLOR_GREEN, cases.tgv_params(desc))
    assert_fields(res, 0.05)


def test_non_multiple_of_tile_grid(cuda_device):
    """nx not a multiple of the 32-wide tile, ny not of the tile height: ragged tiles."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.periodic_box(40, 24, 12, u0=0.04, re=100.0)
    res = run_pair(desc, 12, N.INIT_NOISY_UNIFORM, (0.03, 0.01, -0.02, 0.3, 11))
    assert_fields(res, 0.05)


def test_channel_with_cylinder_walls_and_edges(cuda_device):
    """Inlet / outlet / no-slip faces and edges, BCFLUID nodes, curved wall, forces."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0)
    res = run_pair(desc, 40, N.INIT_REST, forces=True)
    assert_fields(res, 0.05)
    fg, fo = res["gpu_f"][0], res["oracle_f"][0]
    assert np.abs(fg[:3] - fo[:3]).max() <= 5e-3 * np.abs(fo[:3]).max()
    assert abs(fg[4] - fo[4]) <= 5e-3 * max(abs(fo[4]), 1e-3 * np.abs(fo[:2]).max())


def test_reference_cylinder_case(cuda_device):
    """The reference's shipped case (convective outlet, periodic y) from its own initial
    state, 8 steps."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    res = run_pair(cases.reference_cylinder(), 8, N.INIT_REFERENCE_NOISE, forces=True)
    assert_fields(res, 0.1)
    fg, fo = res["gpu_f"][0], res["oracle_f"][0]
    assert np.abs(fg[:2] - fo[:2]).max() <= 5e-3 * np.abs(fo[:2]).max()


def test_annulus_two_walls(cuda_device):
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.annulus(48, 48, 8, 8.0, 20.0, 0.05, 50.0)
    res = run_pair(desc, 30, N.INIT_REST, forces=True)
    assert_fields(res, 0.05)
    fg, fo = res["gpu_f"], res["oracle_f"]
    for w in range(2):
        assert abs(fg[w, 4] - fo[w, 4]) <= 5e-3 * abs(fo[w, 4]) + 1e-9


def test_staircase_classification(cuda_device):
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 32, 8, 8, 20.0, 15.5, 0.05, 40.0, triangular=False)
    res = run_pair(desc, 25, N.INIT_REST)
    assert_fields(res, 0.05)


@pytest.mark.parametrize("ty,lz", [(4, 3), (8, 5), (16, 64)])
def test_tile_shape_does_not_change_results(cuda_device, ty, lz, monkeypatch):
    """Every (tile height, z-segment) choice of the step kernel gives bit-identical fields."""
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0)
    outs = []
    for env in ({}, {"MRLBM_TILE_Y": str(ty), "MRLBM_LZ": str(lz)}):
        for k in ("MRLBM_TILE_Y", "MRLBM_LZ"):
            monkeypatch.delenv(k, raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        sim = Simulation(desc, init=False)
        sim.init(N.INIT_REST)
        sim.step(15)
        outs.append(sim.moments())
        sim.close()
    assert np.array_equal(outs[0], outs[1])


def test_layouts_round_trip(cuda_device):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.periodic_box(32, 16, 8)
    sim = Simulation(desc, init=False)
    rng = np.random.default_rng(3)
    vals = (rng.standard_normal((10, sim.n)) * 1e-2).astype(np.float32)
    sim.set_moments(vals, layout=N.LAYOUT_REF_TILED)
    assert np.array_equal(sim.moments(layout=N.LAYOUT_REF_TILED), vals)
    lex = sim.moments().reshape(10, -1)
    sim.set_moments(lex)
    assert np.array_equal(sim.moments(layout=N.LAYOUT_REF_TILED), vals)
    sub = sim.moments(["ux", "myz"])
    assert np.array_equal(sub.reshape(2, -1), lex[[1, 9]])


def test_diagnostics_match_host_sums(cuda_device):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.periodic_box(32, u0=0.05, re=400.0)
    sim = Simulation(desc, init=False)
    sim.init(N.INIT_TAYLOR_GREEN, cases.tgv_params(desc))
    sim.set_sampling(0, 1)
    sim.step(3)
    steps, vals = sim.diagnostics()
    assert list(steps) == [0, 1, 2]
    m = sim.moments().reshape(10, -1).astype(np.float64)
    mass = (1.0 + m[0]).sum()
    energy = 0.5 * (m[1] ** 2 + m[2] ** 2 + m[3] ** 2).sum()
    assert abs(vals[-1, 0] - mass) / mass < 1e-9
    assert abs(vals[-1, 1] - energy) / energy < 1e-5
    sim.close()
