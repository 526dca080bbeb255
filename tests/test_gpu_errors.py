"""Error statuses the C ABI reports from device state, made on the host: the solver never
exits the process (the reference's checkCudaErrors does) and the context stays usable."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", [0, 1])
def test_non_finite_state_is_reported_as_diverged(cuda_device, storage):
    """A NaN planted in the field on the host spreads through the stream; the FP64 mass /
    energy watchdog of the sampled steps turns it into MRLBM_ERR_DIVERGED at mrlbm_sync, and
    a fresh initialisation of the same handle steps normally again."""
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.periodic_box(32, u0=0.05, re=400.0, storage=storage)
    sim = Simulation(desc, init=False)
    sim.init(N.INIT_TAYLOR_GREEN, cases.tgv_params(desc))
    m = sim.moments()
    m[1, 7, 11, 13] = np.nan
    sim.set_moments(m)
    sim.set_sampling(0, 1)
    sim.step(3)
    with pytest.raises(N.MrlbmError) as e:
        sim.sync()
    assert e.value.code == N.ERR_DIVERGED
    sim.init(N.INIT_TAYLOR_GREEN, cases.tgv_params(desc))
    sim.step(3)
    sim.sync()
    assert np.isfinite(sim.moments()).all()
    sim.close()


def test_bad_arguments_are_statuses(cuda_device):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    sim = Simulation(cases.periodic_box(16))
    with pytest.raises(N.MrlbmError) as e:
        sim.forces(123456)  # no force sample for that step
    assert e.value.code in (N.ERR_STATE, N.ERR_INVALID_ARG)
    with pytest.raises(N.MrlbmError) as e:
        sim.write_pressure("/nonexistent/dir/pressure.dat")
    assert e.value.code in (N.ERR_INVALID_ARG, N.ERR_UNSUPPORTED, N.ERR_IO)
    sim.step(2)
    sim.sync()
    sim.close()


def _planted_nan_sim(watchdog_every: int):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.periodic_box(32, u0=0.05, re=400.0)
    desc.watchdog_every = watchdog_every
    sim = Simulation(desc, init=False)
    sim.init(N.INIT_TAYLOR_GREEN, cases.tgv_params(desc))
    m = sim.moments()
    m[0, 3, 4, 5] = np.nan
    sim.set_moments(m)
    sim.set_sampling(0, 0)  # no diagnostics sampling: only the watchdog can see it
    return sim, desc


def test_watchdog_reports_divergence_without_sampling(cuda_device):
    """With sampling off, the divergence watchdog (every `watchdog_every` steps the step's FP64
    mass / energy sums are checked on the device) turns a NaN planted on the host into
    MRLBM_ERR_DIVERGED: mrlbm_step itself refuses to go on once the flag has come back, with no
    mrlbm_sync in between, and mrlbm_sync reports it too.  A fresh init clears it."""
    import time
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    sim, desc = _planted_nan_sim(8)
    with pytest.raises(N.MrlbmError) as e:
        for _ in range(400):
            sim.step(1)
            time.sleep(0.001)  # let a watchdog copy land; no synchronisation
    assert e.value.code == N.ERR_DIVERGED
    with pytest.raises(N.MrlbmError) as e:
        sim.sync()
    assert e.value.code == N.ERR_DIVERGED
    sim.init(N.INIT_TAYLOR_GREEN, cases.tgv_params(desc))
    sim.step(20)
    sim.sync()
    assert np.isfinite(sim.moments()).all()
    sim.close()


def test_watchdog_can_be_switched_off(cuda_device):
    """watchdog_every < 0: no check runs, so without sampling a NaN goes unreported (the
    caller chose to look only through diagnostics sampling)."""
    sim, _ = _planted_nan_sim(-1)
    sim.step(40)
    sim.sync()
    assert not np.isfinite(sim.moments()).all()
    sim.close()


def test_failed_autotune_restores_the_handle(cuda_device, monkeypatch):
    """A trial of mrlbm_autotune that fails (injected on the host: MRLBM_FAULT_AUTOTUNE_TRIAL
    makes trial 3 return a CUDA error before it launches) returns that status and leaves the
    handle as it was: the same field, step counter, tiling and sampling, and no device memory
    kept by the tuner."""
    torch = pytest.importorskip("torch")
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(96, 48, 16, 10, 30.0, 24.0, 0.05, 80.0)
    sim = Simulation(desc, init=False)
    sim.init(N.INIT_REST)
    sim.set_sampling(1, 1)
    sim.step(5)
    sim.sync()
    m0, info0 = sim.moments(), sim.get_info()
    free0 = torch.cuda.mem_get_info()[0]
    monkeypatch.setenv("MRLBM_FAULT_AUTOTUNE_TRIAL", "3")
    with pytest.raises(N.MrlbmError) as e:
        sim.autotune(2)
    monkeypatch.delenv("MRLBM_FAULT_AUTOTUNE_TRIAL")
    assert e.value.code == N.ERR_CUDA and "injected" in str(e.value)
    info1 = sim.get_info()
    assert info1.step == info0.step and list(info1.tile) == list(info0.tile)
    assert np.array_equal(sim.moments(), m0)
    assert torch.cuda.mem_get_info()[0] == free0
    sim.step(3)  # sampling is back on: steps 5, 6, 7 are sampled
    sim.sync()
    st, _ = sim.force_history()
    ds, _ = sim.diagnostics()
    assert list(st[-3:]) == [5, 6, 7] and list(ds[-3:]) == [5, 6, 7]
    sim.close()


def test_failed_batch_autotune_restores_the_batch(cuda_device, monkeypatch):
    """The same for mrlbm_batch_autotune: every case keeps its field and counters."""
    from mrlbm_3d_cuda_gb300 import Batch, cases
    from mrlbm_3d_cuda_gb300 import native as N
    descs = [cases.cylinder_channel(96, 48, 16, 10, 30.0, 24.0, 0.05, 80.0),
             cases.cylinder_channel(128, 64, 16, 12, 40.0, 32.0, 0.05, 120.0)]
    b = Batch(descs)
    for c in b.cases:
        c.init(N.INIT_REST)
    b.step(4)
    b.sync()
    before = [c.moments() for c in b.cases]
    monkeypatch.setenv("MRLBM_FAULT_AUTOTUNE_TRIAL", "2")
    with pytest.raises(N.MrlbmError) as e:
        b.autotune(2)
    monkeypatch.delenv("MRLBM_FAULT_AUTOTUNE_TRIAL")
    assert e.value.code == N.ERR_CUDA
    for c, m in zip(b.cases, before):
        assert np.array_equal(c.moments(), m)
        assert c.get_info().step == 4
    b.step(2)
    b.sync()
    b.close()
