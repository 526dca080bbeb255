"""Files in the reference's formats: restart.bin, .vti / master.pvd, forces.dat / mass_flux.dat,
pressure.dat (MRLBM_3D/src/restart/restart_io.cu, output/saveData.cu,
statistics/stat_header.cuh, cases/cylinder/cylinder_kernels.cu{,h})."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN


def test_master_pvd_lists_the_vti_series(built, tmp_path):
    from mrlbm_3d_cuda_gb300.simulation import write_master_pvd
    p = tmp_path / "master.pvd"
    write_master_pvd(p, 5000, 12000)
    want = ('<VTKFile type="Collection" version="0.1">\n\t<Collection>\n'
            '\t\t<DataSet timestep="0" file="data10000000.vti" />\n'
            '\t\t<DataSet timestep="1" file="data10005000.vti" />\n'
            '\t\t<DataSet timestep="2" file="data10010000.vti" />\n'
            '\t</Collection>\n</VTKFile>\n')
    assert p.read_text() == want


def read_vti(path):
    raw = path.read_bytes()
    head, _, data = raw.partition(b'<AppendedData encoding="raw">\n_')
    names = [seg.split(b'"')[0].decode() for seg in head.split(b'Name="')[1:]]
    out, off = {}, 0
    for name in names:
        nbytes = int(np.frombuffer(data[off:off + 8], dtype=np.uint64)[0])
        out[name] = np.frombuffer(data[off + 8:off + 8 + nbytes], dtype=np.float32)
        off += 8 + nbytes
    assert data[off:] == b"\n  </AppendedData>\n</VTKFile>\n"
    return head.decode(), out


@pytest.mark.gpu
def test_checkpoint_round_trip_is_exact(cuda_device, tmp_path):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0)
    a = Simulation(desc, init=False)
    a.init(N.INIT_REST)
    a.step(10)
    p = tmp_path / "restart.bin"
    a.checkpoint_save(p)
    raw = p.read_bytes()
    n = desc.nx * desc.ny * desc.nz
    assert int(np.frombuffer(raw[:4], dtype=np.int32)[0]) == 10
    assert len(raw) == 4 + 40 * n + 4 * 9 * n
    b = Simulation(desc, init=False)
    b.checkpoint_load(p)
    assert b.get_info().step == 10
    assert np.array_equal(b.moments(), a.moments())
    a.step(7)
    b.step(7)
    assert np.array_equal(b.moments(), a.moments())
    a.close()
    b.close()


@pytest.mark.gpu
def test_checkpoint_matches_the_reference_restart_bin(cuda_device, tmp_path):
    """The moments and the six face-population arrays of restart.bin after 11 steps of the
    shipped cylinder case agree with the reference build's own checkpoint (sampled
    positions of every array); populations within 1e-5 of their scale."""
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    g = np.load(GOLDEN / "ref_cylinder_run_n10.npz")
    sim = Simulation(cases.reference_cylinder(), init=False)
    sim.init(N.INIT_REFERENCE_NOISE)
    sim.step(int(g["steps"]))
    p = tmp_path / "restart.bin"
    sim.checkpoint_save(p)
    sim.close()
    n = int(np.prod(g["nxyz"]))
    raw = p.read_bytes()
    assert int(np.frombuffer(raw[:4], dtype=np.int32)[0]) == int(g["steps"])
    mom = np.frombuffer(raw[4:4 + 40 * n], dtype=np.float32).reshape(10, n)
    from conftest import field_errors
    assert field_errors(mom[:, g["idx"]], g["moments"], 0.1)[:, 0].max() <= 1e-5
    halo = np.frombuffer(raw[4 + 40 * n:], dtype=np.float32)
    nbk = n // 256
    lens = [32 * nbk * 9] * 4 + [64 * nbk * 9] * 2
    assert halo.size == sum(lens)
    off = 0
    for k, ln in enumerate(lens):
        ours = halo[off + g["halo_pos"][k]]
        ref = g["halo_val"][k]
        assert np.abs(ours - ref).max() <= 1e-5 * np.abs(ref).max(), k
        off += ln


@pytest.mark.gpu
def test_vti_fields(cuda_device, tmp_path):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0)
    sim = Simulation(desc, init=False)
    sim.init(N.INIT_REST)
    sim.step(5)
    p = tmp_path / "data10000005.vti"
    sim.write_vti(p)
    head, f = read_vti(p)
    assert 'WholeExtent="0 63 0 39 0 11"' in head
    assert list(f) == ["rho", "ux", "uy", "uz"]
    m = sim.moments().reshape(10, -1)
    solid = (sim.node_types() >> 20) == 1  # NODE_SOLID
    assert np.array_equal(f["rho"], (np.float32(desc.rho0) + m[0]).astype(np.float32))
    for k, name in ((1, "ux"), (2, "uy"), (3, "uz")):
        assert np.isnan(f[name][solid]).all()
        assert np.array_equal(f[name][~solid], m[k][~solid])
    sim.close()
    ann = Simulation(cases.annulus(48, 48, 8, 8.0, 20.0, 0.05, 50.0), init=False)
    ann.init(N.INIT_REST)
    ann.step(3)
    ann.write_vti(tmp_path / "a.vti")
    _, fa = read_vti(tmp_path / "a.vti")
    assert list(fa) == ["rho", "uz", "u_theta", "u_radial"]
    ann.close()


@pytest.mark.gpu
def test_forces_and_mass_flux_files(cuda_device, tmp_path):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0)
    sim = Simulation(desc, init=False)
    sim.init(N.INIT_REST)
    sim.set_sampling(1, 0)
    sim.step(6)
    fp, mp = tmp_path / "forces.dat", tmp_path / "mass_flux.dat"
    sim.write_forces(fp, mp)
    sim.step(4)
    sim.write_forces(fp, mp, append=True)
    steps, f = sim.force_history()
    rows = np.loadtxt(fp)
    assert rows.shape == (10, 4)
    assert list(rows[:, 0].astype(int)) == list(steps)
    assert np.allclose(rows[:, 1:], f[:, 0, :3], rtol=0, atol=1e-15)
    line = fp.read_text().splitlines()[0].split()
    assert all(len(v.split(".")[1]) == 16 for v in line[1:])  # %.16f, fixed
    mass = np.loadtxt(mp)
    assert np.allclose(mass[:, 1], f[:, 0, 3], rtol=0, atol=1e-15)
    sim.close()


@pytest.mark.gpu
def test_surface_pressure_file(cuda_device, tmp_path):
    """One-sample window: pressure.dat equals the quadratic wall extrapolation of the
    bilinearly interpolated probe densities, computed here from the field."""
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0)
    sim = Simulation(desc, init=False)
    sim.init(N.INIT_REST)
    sim.set_pressure_window(29, 29)
    sim.step(30)
    p = tmp_path / "pressure.dat"
    sim.write_pressure(p)
    lines = p.read_text().splitlines()
    assert lines[0] == "theta z Cp"
    got = np.loadtxt(p, skiprows=1)
    b = sim.boundary(0)
    rho = sim.moments()[0].astype(np.float64) + desc.rho0  # (nz, ny, nx)
    xc, yc, r = desc.xc, desc.yc, 0.5 * desc.d_wall[0]
    nx_, ny_ = b["nx"].astype(np.float64), b["ny"].astype(np.float64)
    node = b["list"]
    x, y, z = node % desc.nx, (node // desc.nx) % desc.ny, node // (desc.nx * desc.ny)
    xw, yw = xc + r * nx_, yc + r * ny_
    rk, pk = [], []
    for k in (1, 2, 3):
        px, py = xw + k * nx_, yw + k * ny_
        x0, y0 = np.floor(px).astype(int), np.floor(py).astype(int)
        xd, yd = px - x0, py - y0
        v = ((1 - yd) * ((1 - xd) * rho[z, y0, x0] + xd * rho[z, y0, x0 + 1]) +
             yd * ((1 - xd) * rho[z, y0 + 1, x0] + xd * rho[z, y0 + 1, x0 + 1]))
        rk.append(np.hypot(px - xc, py - yc))
        pk.append(v / 3.0)
    rw = np.hypot(xw - xc, yw - yc)
    want = np.array([np.polyval(np.polyfit([rk[0][i], rk[1][i], rk[2][i]], [pk[0][i], pk[1][i], pk[2][i]], 2), rw[i])
                     for i in range(len(node))])
    theta = np.degrees(np.arctan2(y - yc, x - xc)) % 360.0
    assert got.shape == (len(node), 3)
    assert np.allclose(got[:, 0], theta, atol=1e-4)
    assert np.array_equal(got[:, 1].astype(int), z)
    assert np.allclose(got[:, 2], want, rtol=0, atol=5e-5)  # FP32 quadratic, cancellation ~1e-5
    sim.close()


@pytest.mark.gpu
def test_inlet_density_file(cuda_device, tmp_path):
    """inlet_density.dat over a statistics window: per step the mean density of the x = 0 face
    (computed here from the field after each step) and the running mean of the earlier samples
    (0 on the first line), %.16f."""
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0)
    sim = Simulation(desc, init=False)
    sim.init(N.INIT_NOISY_UNIFORM, (0.03, 0.01, 0.0, 0.3, 5))
    sim.set_pressure_window(3, 7)
    want, mean, n = [], 0.0, 0
    for it in range(10):
        sim.step(1)
        if 3 <= it <= 7:
            r_in = (np.float32(desc.rho0) + sim.moments()[0][:, :, 0]).astype(np.float64).mean()  # (nz, ny) face
            want.append((it, r_in, mean))
            n += 1
            mean += (r_in - mean) / n
    p = tmp_path / "inlet_density.dat"
    sim.write_inlet_density(p)
    rows = np.loadtxt(p)
    assert rows.shape == (5, 3)
    assert list(rows[:, 0].astype(int)) == [w[0] for w in want]
    assert np.allclose(rows[:, 1], [w[1] for w in want], rtol=0, atol=1e-12)
    assert np.allclose(rows[:, 2], [w[2] for w in want], rtol=0, atol=1e-12)
    assert rows[0, 2] == 0.0
    assert all(len(v.split(".")[1]) == 16 for v in p.read_text().splitlines()[0].split()[1:])
    sim.close()


@pytest.mark.gpu
def test_reference_style_run_writes_every_output(cuda_device, tmp_path):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    sim = Simulation(cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0), init=False)
    sim.init(N.INIT_REST)
    sim.run_reference_outputs(tmp_path, max_iter=20, macr_save=10, stat_start=12, stat_end=20, checkpoint_save=10)
    names = sorted(p.name for p in tmp_path.iterdir())
    assert names == ["checkpoint", "data10000000.vti", "data10000010.vti", "data10000020.vti", "forces.dat",
                     "grid_layout", "inlet_density.dat", "mass_flux.dat", "master.pvd", "pressure.dat"]
    assert np.loadtxt(tmp_path / "inlet_density.dat").shape == (9, 3)
    assert len(list((tmp_path / "grid_layout").glob("*.dat"))) == 9
    assert (tmp_path / "checkpoint" / "restart_step.txt").read_text().strip() == "21"
    assert np.loadtxt(tmp_path / "forces.dat").shape == (9, 4)
    sim.close()
