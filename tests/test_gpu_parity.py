"""GPU parity: the CUDA solver (through the C ABI) against the oracle on the same inputs.

Field metric (conftest.field_errors): per field, max |gpu - oracle| / max(|oracle|_inf, s_f)
with s_f the magnitude of the quantity as the FP32 algorithm computes it (rho: 1, u: U,
m_ab: cs2 = 1/3).  Criteria, per field:
  * strict:   <= 1e-5 against the FP32 oracle (reference arithmetic order) on short runs;
  * rounding: on longer runs FP32 rounding of the reference's own arithmetic grows past
    1e-5 in impulsively started flows, so the GPU must stay within max(1e-5, 2 x e32) of
    the FP32 oracle and within max(1e-5, 1.5 x e32) of the FP64 oracle, where e32 is the
    FP32 oracle's own distance from the FP64 oracle (the FP32 noise floor).
Forces: relative 5e-3 of |F| (the stated Cd / Cl tolerance), in practice far tighter."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import field_errors

pytestmark = pytest.mark.gpu
TOL = 1e-5


def run_pair(desc, steps, init_kind, params=(), forces=False, fp64=True):
    import oracle
    from mrlbm_3d_cuda_gb300 import Simulation
    sim = Simulation(desc, init=False)
    sim.init(init_kind, params)
    if forces:
        sim.set_sampling(1, 0)
    orc = {32: oracle.Oracle(desc, 32)}
    if fp64:
        orc[64] = oracle.Oracle(desc, 64)
    for o in orc.values():
        o.init(init_kind, params)
    # initial states agree exactly (same initialiser arithmetic)
    assert np.array_equal(sim.moments().astype(np.float64), orc[32].moments()), "initial state differs"
    sim.step(steps)
    for o in orc.values():
        if steps > 1:
            o.step(steps - 1)
        if steps > 0:
            o.step(1, forces=forces)
    sim.sync()
    res = {"gpu": sim.moments(), "oracle": orc[32].moments(), "types": sim.node_types()}
    if fp64:
        res["oracle64"] = orc[64].moments()
    if forces:
        res["gpu_f"] = sim.forces()
        res["oracle_f"] = orc[32].forces()
        if fp64:
            res["oracle64_f"] = orc[64].forces()
    sim.close()
    for o in orc.values():
        o.close()
    return res


def assert_fields(res, u_ref, strict=False):
    assert np.isfinite(res["gpu"]).all()
    e_g32 = field_errors(res["gpu"], res["oracle"], u_ref)[:, 0]
    if strict or "oracle64" not in res:
        assert e_g32.max() < TOL, "\n" + np.array2string(e_g32, precision=3)
        return e_g32
    e_3264 = field_errors(res["oracle"], res["oracle64"], u_ref)[:, 0]
    e_g64 = field_errors(res["gpu"], res["oracle64"], u_ref)[:, 0]
    table = "\n gpu-o32 " + np.array2string(e_g32, precision=2) + "\n o32-o64 " + \
            np.array2string(e_3264, precision=2) + "\n gpu-o64 " + np.array2string(e_g64, precision=2)
    assert (e_g32 <= np.maximum(TOL, 2.0 * e_3264)).all(), table
    assert (e_g64 <= np.maximum(TOL, 1.5 * e_3264)).all(), table
    return e_g32


def assert_forces(res, wall: int, comps=(0, 1, 4), rel=5e-3):
    """GPU force (FP64 integration) vs the FP64 oracle: within 5e-3 of the force scale, or
    within 3x the FP32 oracle's own distance from the FP64 oracle.  A force is one scalar
    sum of per-node in - out momentum differences that cancel most digits, so its FP32
    noise is a single random draw: the factor is wider than for the field maxima."""
    fg, f32, f64 = res["gpu_f"][wall], res["oracle_f"][wall], res["oracle64_f"][wall]
    scale = np.abs(f64[[0, 1]]).max()
    for k in comps:
        ref = abs(f64[k]) if k != 4 else max(abs(f64[4]), 1e-12)
        bound = max(rel * max(ref, rel * scale if k in (0, 1) else ref), 3.0 * abs(f32[k] - f64[k]))
        assert abs(fg[k] - f64[k]) <= bound, (wall, k, fg, f32, f64)


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
    assert_fields(res, 0.05, strict=True)


def test_non_multiple_of_tile_grid(cuda_device):
    """nx not a multiple of the 32-wide tile, ny not of the tile height: ragged tiles."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.periodic_box(40, 24, 12, u0=0.04, re=100.0)
    res = run_pair(desc, 12, N.INIT_NOISY_UNIFORM, (0.03, 0.01, -0.02, 0.3, 11))
    assert_fields(res, 0.05, strict=True)


@pytest.mark.parametrize("shape", [(8, 8, 4), (8, 24, 4), (72, 8, 12)])
def test_smallest_grids(cuda_device, shape):
    """Grids at the reference's minimum granularity (multiples of 8, 8, 4): one partial tile,
    a one-plane-deep z segment per item, a single x-block."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.periodic_box(*shape, u0=0.04, re=100.0)
    res = run_pair(desc, 10, N.INIT_NOISY_UNIFORM, (0.03, 0.01, -0.02, 0.3, 7), fp64=False)
    assert_fields(res, 0.05, strict=True)


def test_channel_short_run_strict(cuda_device):
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0)
    res = run_pair(desc, 6, N.INIT_REST, forces=True, fp64=False)
    assert_fields(res, 0.05, strict=True)


def test_channel_with_cylinder_walls_and_edges(cuda_device):
    """Inlet / outlet / no-slip faces and edges, BCFLUID nodes, curved wall, forces."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0)
    res = run_pair(desc, 40, N.INIT_REST, forces=True)
    assert_fields(res, 0.05)
    assert_forces(res, 0, comps=(0, 1, 3, 4))


@pytest.mark.parametrize("convective", [False, True])
def test_outlet_current_update(cuda_device, convective):
    """NEUMANN_CURRENT_UPDATE: the outlet takes the post-stream rho, u of its x-1 neighbour
    (and of itself when convective) instead of their stored moments."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0, convective=convective)
    desc.neumann_current_update = 1
    res = run_pair(desc, 6, N.INIT_REST, fp64=False)
    assert_fields(res, 0.05, strict=True)
    res = run_pair(desc, 40, N.INIT_REST)
    assert_fields(res, 0.05)


@pytest.mark.parametrize("steps", [8, 160])
def test_reference_cylinder_case(cuda_device, steps):
    """The reference's shipped case (convective outlet, periodic y) from its own initial
    state; after ~125 steps the inlet pressure wave has reached the cylinder and the force
    is no longer round-off."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    res = run_pair(cases.reference_cylinder(), steps, N.INIT_REFERENCE_NOISE, forces=True)
    assert_fields(res, 0.1)
    if steps > 125:
        assert_forces(res, 0, comps=(0, 1))


def test_annulus_two_walls(cuda_device):
    """Both walls' torques after 1000 steps.  Earlier the outer wall's torque is the arrival
    of the diffusion front started at the inner wall: a small difference of nearly equal
    in / out momenta that FP32 rounding moves by percents (the FP32 oracle is 0.5 % from the
    FP64 one at 200 steps and 3.8 % at 400; rounding-sized perturbations of the initial state
    move it by up to 1.4 % at 200), so it is no parity check there."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.annulus(48, 48, 8, 8.0, 20.0, 0.05, 50.0)
    res = run_pair(desc, 1000, N.INIT_REST, forces=True)
    assert_fields(res, 0.05)
    for w in range(2):
        assert_forces(res, w, comps=(4,))


@pytest.mark.parametrize("wall,bcf", [(1, 0), (0, 1), (1, 1)])
def test_strong_mass_conservation_variants(cuda_device, wall, bcf):
    """MassBC::Strong for the curved wall (numerical_solution.cu:124-279) and / or for the
    BCFLUID nodes (the Strong quadratic of boundaries.cuh:890-897 and its mirror images),
    against the oracle: strict on a short run, the FP32 rounding criterion on a longer one
    with forces."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0)
    desc.mass_bc = N.MASS_STRONG if wall else N.MASS_EQUILIBRIUM
    desc.bcf_mass_bc = N.MASS_STRONG if bcf else N.MASS_EQUILIBRIUM
    res = run_pair(desc, 6, N.INIT_REST, fp64=False)
    assert_fields(res, 0.05, strict=True)
    res = run_pair(desc, 40, N.INIT_REST, forces=True)
    assert_fields(res, 0.05)
    assert_forces(res, 0, comps=(0, 1, 3))


@pytest.mark.parametrize("option", ["staircase_z_walls", "periodic_x_array"])
def test_geometry_options(cuda_device, option):
    """Remaining combinations of the reference's compile-time switches: staircase wall nodes
    with no-slip z faces (X_PERIODIC 0, Z_PERIODIC 0, triangular false), and a cylinder in a
    box periodic in every axis (X_PERIODIC 1: no inlet or outlet; a periodic array of
    cylinders in a uniform noisy stream)."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    if option == "staircase_z_walls":
        desc = cases.cylinder_channel(64, 32, 12, 8, 20.0, 15.5, 0.05, 40.0, triangular=False, periodic_z=False)
        init, params = N.INIT_REST, ()
    else:
        desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0, periodic_y=True)
        desc.periodic[0] = 1
        init, params = N.INIT_NOISY_UNIFORM, (0.03, 0.0, 0.0, 0.2, 9)
    res = run_pair(desc, 6, init, params, fp64=False)
    assert_fields(res, 0.05, strict=True)
    res = run_pair(desc, 40, init, params, forces=True)
    assert_fields(res, 0.05)
    assert_forces(res, 0, comps=(0, 1))


BCSOLID_TAGS = [7, 11, 13, 14, 112, 176, 208, 224]


@pytest.mark.parametrize("geom", ["cylinder", "annulus"])
def test_z_walls_bcsolid(cuda_device, geom):
    """No-slip z faces (Z_PERIODIC 0): BACK / FRONT faces and their edges, the BCFLUID nodes
    above / below the body's end faces and the BCSOLID nodes where the z faces meet the body
    (boundaries.cuh:1039-1214).  BCSOLID nodes with a closure tag are held at rest: after the
    collision u = 0 and the diagonal and xy moments stay 0."""
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    if geom == "cylinder":
        desc = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0, periodic_z=False)
    else:
        desc = cases.annulus(48, 48, 8, 8.0, 20.0, 0.05, 50.0, periodic_z=False)
    res = run_pair(desc, 6, N.INIT_NOISY_UNIFORM, (0.03, 0.01, 0.0, 0.3, 5), fp64=False)
    assert_fields(res, 0.05, strict=True)
    t = res["types"]
    cls, tag = t >> 20, t & 0xFF
    sel = np.isin(cls, (N.NODE_BCSOLID_INNER, N.NODE_BCSOLID_OUTER)) & np.isin(tag, BCSOLID_TAGS)
    m = res["gpu"].reshape(10, -1)
    assert sel.sum() >= 8
    assert (m[1:8][:, sel] == 0).all()
    assert np.abs(m[8:10][:, sel]).max() > 0
    res = run_pair(desc, 60, N.INIT_REST, forces=True)
    assert_fields(res, 0.05)
    if geom == "cylinder":
        assert_forces(res, 0, comps=(0, 1))


def test_staircase_classification(cuda_device):
    from mrlbm_3d_cuda_gb300 import cases
    from mrlbm_3d_cuda_gb300 import native as N
    desc = cases.cylinder_channel(64, 32, 8, 8, 20.0, 15.5, 0.05, 40.0, triangular=False)
    res = run_pair(desc, 25, N.INIT_REST)
    assert_fields(res, 0.05)


@pytest.mark.parametrize("flow", ["channel", "noisy_box"])
@pytest.mark.parametrize("ty,lz", [(4, 3), (8, 5), (16, 64)])
def test_tile_shape_does_not_change_results(cuda_device, ty, lz, flow, monkeypatch):
    """Every (tile height, z-segment) choice of the step kernel gives bit-identical fields:
    a column rebuilt by a rim warp must round exactly like the same column rebuilt by its
    owner (the noisy box has non-zero velocity everywhere from the first step)."""
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    if flow == "channel":
        desc, kind, params = cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0), N.INIT_REST, ()
    else:
        desc, kind, params = (cases.periodic_box(40, 24, 12, u0=0.04, re=100.0), N.INIT_NOISY_UNIFORM,
                              (0.03, 0.01, -0.02, 0.3, 11))
    outs = []
    for env in ({}, {"MRLBM_TILE_Y": str(ty), "MRLBM_LZ": str(lz)}):
        for k in ("MRLBM_TILE_Y", "MRLBM_LZ"):
            monkeypatch.delenv(k, raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        sim = Simulation(desc, init=False)
        sim.init(kind, params)
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
