"""The C-ABI library: loads without a GPU, exports every entry point of include/mrlbm.h,
and its host-side guards behave like the reference's (as status codes, never exits)."""
from __future__ import annotations

import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT


def header_symbols():
    text = (ROOT / "include" / "mrlbm.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(mrlbm_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    syms = header_symbols()
    assert "mrlbm_create" in syms and "mrlbm_step" in syms and len(syms) >= 20


def test_library_exports_every_declared_symbol(built):
    from mrlbm_3d_cuda_gb300 import native as N
    lib = C.CDLL(str(N.LIB_PATH))
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # and the Python binding binds exactly those
    assert set(N.EXPORTED) == set(header_symbols())


def test_abi_version(built):
    from mrlbm_3d_cuda_gb300 import native as N
    assert N.lib().mrlbm_abi_version() == 1


def test_descriptor_defaults_match_reference_constants(built):
    from mrlbm_3d_cuda_gb300 import native as N
    d = N.finalize(N.default_desc(N.GEOM_CYLINDER))
    assert (d.nx, d.ny, d.nz) == (336, 144, 48)
    assert (d.xc, d.yc, d.d_wall[0]) == (71.5, 71.5, 16.0)
    assert tuple(d.periodic) == (0, 1, 1) and d.convective_outlet == 1
    # OMEGA = 1 / (0.5 + 3 * (0.1f * 16 / 100)) with the reference's float/double mix
    visc = np.float32(np.float32(0.1) * np.float32(16.0) / np.float32(100.0))
    tau = np.float32(0.5 + 3.0 * float(visc))
    assert d.omega == np.float32(1.0 / float(tau))
    a = N.finalize(N.default_desc(N.GEOM_ANNULUS))
    assert (a.nx, a.ny, a.nz) == (136, 136, 256)
    assert (a.d_wall[0], a.d_wall[1], a.xc) == (64.0, 128.0, 67.5)
    assert abs(a.wall_u[0][1] - 0.03) < 1e-7


@pytest.mark.parametrize("field,value,code", [("re", 1e9, -1), ("re", 0.5, -1), ("u_max", 0.3, -1)])
def test_tau_and_mach_guards_are_error_codes(built, field, value, code):
    from mrlbm_3d_cuda_gb300 import native as N
    d = N.default_desc(N.GEOM_CYLINDER)
    setattr(d, field, value)
    with pytest.raises(N.MrlbmError) as e:
        N.finalize(d)
    assert e.value.code == code


def test_bad_grid_rejected(built):
    from mrlbm_3d_cuda_gb300 import native as N
    d = N.default_desc(N.GEOM_NONE)
    d.nx = 60  # not a multiple of 8 (initializeLBM.cuh:60-62)
    with pytest.raises(N.MrlbmError):
        N.finalize(d)


def test_host_only_handle_refuses_device_calls(built):
    from mrlbm_3d_cuda_gb300 import native as N
    from mrlbm_3d_cuda_gb300.simulation import Simulation
    s = Simulation(N.finalize(N.default_desc(N.GEOM_NONE)), host_only=True)
    assert s.info.n_nodes == 64 ** 3
    with pytest.raises(N.MrlbmError) as e:
        s.step(1)
    assert e.value.code == N.ERR_STATE
    with pytest.raises(N.MrlbmError):
        s.moments()
    s.close()


def test_header_and_library_usable_from_plain_c(built, tmp_path):
    """include/mrlbm.h compiles as C99 with warnings as errors, a C program links against the
    library and drives it: the shipped cylinder case on the host (2112 wall nodes, 768 BCFLUID
    nodes, the counts of the reference's own classification) and a status instead of an exit
    for device work on a host-only handle."""
    import shutil
    import subprocess
    from mrlbm_3d_cuda_gb300 import native as N
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path / "abi_from_c"
    lib_dir = N.LIB_PATH.parent
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "c" / "abi_from_c.c"), "-L", str(lib_dir), "-lmrlbm",
           f"-Wl,-rpath,{lib_dir}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    first, second = r.stdout.splitlines()
    nx, ny, nz, nb, nbf, rc, note = first.split()
    assert (int(nx), int(ny), int(nz)) == (336, 144, 48)
    assert (int(nb), int(nbf)) == (2112, 768)
    assert int(rc) == N.ERR_STATE and note == "error-reported"
    # window derived as LW-4 .. LW+D+4 with LW = XC - (D-1)/2 = 24, like cases.cylinder_channel
    x0, x1, y0, y1, nb2 = (int(v) for v in second.split())
    assert (x0, x1, y0, y1) == (20, 44, 20, 44) and nb2 > 0
