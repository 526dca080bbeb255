"""The allocation-free periodic step (mrlbm_step_periodic_noalloc) against the handle API.

The entry point keeps its scratch in one fixed array of the library's device image that
every call shares, so this file is collected last: it must pass in a fresh process (first
use of that array) and after every other test.  Two calls in a row ping-pong between two
caller-owned device buffers, and each call's output is checked against one mrlbm_step of a
handle started from the same state.  The fields must be bit-identical: the entry point runs the
handle's step kernel, whose results do not depend on the tiling or the work split.  The mass
and energy sums are FP64 sums of per-thread partials whose grouping follows the work split, so
they are compared within 1e-9 (mass) and 1e-5 (energy) relative."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

def to_storage(lex: np.ndarray, nx: int, ny: int, nz: int) -> np.ndarray:
    """(10, n) lexicographic moments -> the solver's x-blocked storage layout (flat)."""
    nxb = -(-nx // 32)
    pad = np.zeros((10, nz, ny, nxb * 32), np.float32)
    pad[..., :nx] = lex.reshape(10, nz, ny, nx)
    return np.ascontiguousarray(pad.reshape(10, nz, ny, nxb, 32).transpose(1, 2, 3, 0, 4)).reshape(-1)


def from_storage(buf: np.ndarray, nx: int, ny: int, nz: int) -> np.ndarray:
    nxb = -(-nx // 32)
    a = buf.reshape(nz, ny, nxb, 10, 32).transpose(3, 0, 1, 2, 4).reshape(10, nz, ny, nxb * 32)
    return np.ascontiguousarray(a[..., :nx]).reshape(10, -1)


def call_noalloc(lib, src, dst, nx, ny, nz, omega, rho0, diag, stream):
    return lib.mrlbm_step_periodic_noalloc(C.c_void_p(src), C.c_void_p(dst), nx, ny, nz, C.c_float(omega),
                                           C.c_float(rho0), diag, C.c_void_p(stream))


def test_noalloc_rejects_what_it_cannot_hold(built):
    """Host-side checks (no device work): a grid beyond the fixed scratch, overlapping or
    misaligned buffers."""
    from mrlbm_3d_cuda_gb300 import native as N
    lib = N.lib()
    a, b = 1 << 40, 1 << 44
    rc = call_noalloc(lib, a, b, 4096, 4096, 8, 1.0, 1.0, None, 0)
    assert rc == N.ERR_INVALID_ARG
    assert b"64 KiB" in lib.mrlbm_last_error(None)
    assert call_noalloc(lib, a, a + 256, 64, 64, 8, 1.0, 1.0, None, 0) == N.ERR_INVALID_ARG
    assert b"overlap" in lib.mrlbm_last_error(None)
    assert call_noalloc(lib, a + 4, b, 64, 64, 8, 1.0, 1.0, None, 0) == N.ERR_INVALID_ARG
    assert call_noalloc(lib, a, b, 60, 64, 8, 1.0, 1.0, None, 0) == N.ERR_INVALID_ARG
    assert call_noalloc(lib, a, b, 64, 64, 8, 2.5, 1.0, None, 0) == N.ERR_INVALID_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("shape,with_diag", [((40, 24, 12), True), ((40, 24, 12), False), ((64, 64, 64), True),
                                             ((32, 16, 4096), False)])
def test_noalloc_step_matches_handle_step(cuda_device, shape, with_diag):
    import torch
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    nx, ny, nz = shape
    u0 = 0.05
    desc = cases.periodic_box(nx, ny, nz, u0=u0, re=200.0)
    sim = Simulation(desc, init=False)
    if nx == ny == nz:
        sim.init(N.INIT_TAYLOR_GREEN, cases.tgv_params(desc))
    else:
        sim.init(N.INIT_NOISY_UNIFORM, (0.03, 0.01, -0.02, 0.3, 11))
    sim.set_sampling(0, 1)
    omega, rho0 = float(sim.get_info().omega), float(desc.rho0)
    start = to_storage(sim.moments(), nx, ny, nz)
    dev = torch.device("cuda", 0)
    bufs = [torch.from_numpy(start).to(dev), torch.zeros(start.size, dtype=torch.float32, device=dev)]
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize(dev)
    lib = N.lib()
    for call in range(2):
        src, dst = bufs[call % 2], bufs[(call + 1) % 2]
        diag = (C.c_double * 2)() if with_diag else None
        rc = call_noalloc(lib, src.data_ptr(), dst.data_ptr(), nx, ny, nz, omega, rho0, diag, stream)
        assert rc == N.OK, lib.mrlbm_last_error(None)
        torch.cuda.synchronize(dev)
        sim.step(1)
        want = sim.moments()
        got = from_storage(dst.cpu().numpy(), nx, ny, nz)
        assert np.isfinite(got).all()
        assert np.array_equal(got, want.reshape(10, -1)), (call, np.abs(got - want.reshape(10, -1)).max(axis=1))
        if with_diag:
            _, vals = sim.diagnostics()
            assert abs(diag[0] - vals[-1, 0]) <= 1e-9 * abs(vals[-1, 0]), (call, diag[0], vals[-1])
            assert abs(diag[1] - vals[-1, 1]) <= 1e-5 * abs(vals[-1, 1]), (call, diag[1], vals[-1])
    sim.close()
