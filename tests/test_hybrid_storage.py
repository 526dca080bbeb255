"""The hybrid storage mode (MRLBM_STORAGE_F16_U32): velocity in FP32, rho - rho0 and the
second moments as scaled FP16 (28 bytes per node instead of 40 / 20).

FP16 rounding of u is what moves the 16-bit runs away from FP32 (the velocity field carries
the lift and the shedding phase); the hybrid keeps u exact and rounds only the density
deviation and m.  These tests hold the mode to the invariants of the other storage modes:
results independent of the tiling and of batching, exact round trips of what it stores, and
checkpoint reloads that change nothing."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _desc(kind, sr=0):
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    if kind == "channel":
        d = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0, storage=N.STORAGE_F16_U32)
        init, params = N.INIT_REST, ()
    else:
        d = cases.periodic_box(40, 24, 12, u0=0.04, re=100.0, storage=N.STORAGE_F16_U32)
        init, params = N.INIT_NOISY_UNIFORM, (0.03, 0.01, -0.02, 0.3, 11)
    d.stochastic_rounding = sr
    return d, init, params


@pytest.mark.parametrize("kind", ["channel", "noisy_box"])
@pytest.mark.parametrize("sr", [0, 1])
def test_hybrid_is_tiling_independent(cuda_device, monkeypatch, kind, sr):
    from mrlbm_3d_cuda_gb300 import Simulation
    outs = []
    for env in ({}, {"MRLBM_TILE_Y": "8", "MRLBM_LZ": "5"}, {"MRLBM_TILE_Y": "4", "MRLBM_LZ": "3"}):
        for k in ("MRLBM_TILE_Y", "MRLBM_LZ"):
            monkeypatch.delenv(k, raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        d, init, params = _desc(kind, sr)
        sim = Simulation(d, init=False)
        sim.init(init, params)
        sim.step(15)
        outs.append(sim.moments())
        sim.close()
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


def test_hybrid_round_trip_and_precision(cuda_device):
    """u goes through the store unchanged; rho - rho0 and m come back within FP16's relative
    rounding of their scaled values."""
    from mrlbm_3d_cuda_gb300 import Simulation
    d, _, _ = _desc("noisy_box")
    sim = Simulation(d, init=False)
    rng = np.random.default_rng(5)
    v = np.zeros((10, sim.n), np.float32)
    v[0] = rng.uniform(-1e-3, 1e-3, sim.n)
    v[1:4] = rng.uniform(-0.04, 0.04, (3, sim.n))
    v[4:] = rng.uniform(-2e-3, 2e-3, (6, sim.n))
    sim.set_moments(v)
    got = sim.moments().reshape(10, -1)
    sim.close()
    assert np.array_equal(got[1:4], v[1:4])
    for k in [0] + list(range(4, 10)):
        assert np.abs(got[k] - v[k]).max() <= 2.0 ** -11 * np.abs(v[k]).max() * 1.01, k


def test_hybrid_batch_matches_single_cases(cuda_device):
    from mrlbm_3d_cuda_gb300 import Batch, Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    descs = [cases.cylinder_channel(96, 48, 16, 10, 30.3, 23.7, 0.05, 80.0, storage=N.STORAGE_F16_U32),
             cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0, storage=N.STORAGE_F16_U32)]
    single = []
    for d in descs:
        sim = Simulation(d, init=False)
        sim.init(N.INIT_REST)
        sim.step(12)
        single.append(sim.moments())
        sim.close()
    b = Batch(descs)
    for c in b.cases:
        c.init(N.INIT_REST)
    b.step(12)
    b.sync()
    for c, want in zip(b.cases, single):
        assert np.array_equal(c.moments(), want)
    b.close()


def test_hybrid_checkpoint_reload_is_exact(cuda_device, tmp_path):
    from mrlbm_3d_cuda_gb300 import Simulation
    d, init, params = _desc("channel", 1)
    a = Simulation(d, init=False)
    a.init(init, params)
    a.step(9)
    a.checkpoint_save(tmp_path / "restart.bin")
    a.step(7)
    want = a.moments()
    a.close()
    b = Simulation(d, init=False)
    b.checkpoint_load(tmp_path / "restart.bin")
    b.step(7)
    got = b.moments()
    b.close()
    # the checkpoint holds FP32 moments: a reload re-rounds rho - rho0 and m to FP16, which
    # reproduces the stored halves exactly, and u exactly
    assert np.array_equal(got, want)
