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
