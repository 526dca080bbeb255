"""Node classification: the product's and the oracle's restatements against the reference's
own host code (golden fixture from tests/golden/make_golden.py), and against each other on
the benchmark geometries."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN

KEYS = [("list", "boundary_list"), ("nx", "unit_nx"), ("ny", "unit_ny"), ("delta", "delta"),
        ("in_mask", "in_mask"), ("out_mask", "out_mask"), ("fluid_list", "fluid_list"),
        ("tag_in_mask", "tag_in_mask"), ("tag_out_mask", "tag_out_mask")]


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN / "ref_cylinder_geometry.npz")


def test_golden_fixture_is_consistent(golden):
    t = golden["node_types"]
    cls = t >> 20
    assert int(golden["nb"]) == int((cls == 2).sum()) == len(golden["boundary_list"])
    assert int(golden["nb_fluid"]) == int((cls == 4).sum()) == len(golden["fluid_list"])
    # boundary indices are assigned in list order (cylinder_helpers.cuh:116-132)
    assert np.array_equal(t[golden["boundary_list"]] & 0xFFFFF, np.arange(int(golden["nb"])))


def test_product_geometry_matches_reference(built, golden):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    s = Simulation(cases.reference_cylinder(), host_only=True)
    assert np.array_equal(s.node_types(), golden["node_types"])
    b = s.boundary(0)
    for k, g in KEYS:
        assert np.array_equal(b[k], golden[g]), k
    assert s.info.omega == golden["omega"]


def test_oracle_geometry_matches_reference(built, golden):
    import oracle
    from mrlbm_3d_cuda_gb300 import cases
    o = oracle.Oracle(cases.reference_cylinder(), 64)
    assert np.array_equal(o.node_types(), golden["node_types"])
    b = o.boundary(0)
    for k, g in KEYS:
        assert np.array_equal(b[k], golden[g]), k


def test_reference_tiled_layout_round_trip(built, golden):
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    from mrlbm_3d_cuda_gb300 import native as N
    from tests.golden.make_golden import tiled_to_lex
    s = Simulation(cases.reference_cylinder(), host_only=True)
    tiled = s.node_types(N.LAYOUT_REF_TILED)
    nx, ny, nz = (int(v) for v in golden["shape"])
    lex = tiled_to_lex(np.arange(nx * ny * nz), nx, ny, nz)
    back = np.empty_like(tiled)
    back[lex] = tiled
    assert np.array_equal(back, golden["node_types"])


def test_product_and_oracle_staircase_geometry_match_reference(built):
    """The shipped cylinder case with the staircase classification (triangular = false,
    cases/cylinder/nodeClass.cuh:138-167, 289-297) against the reference's own host code."""
    import oracle
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    g = np.load(GOLDEN / "ref_cylinder_staircase_geometry.npz")
    desc = cases.reference_cylinder()
    desc.triangular = 0
    s = Simulation(desc, host_only=True)
    o = oracle.Oracle(desc, 64)
    for types, b in ((s.node_types(), s.boundary(0)), (o.node_types(), o.boundary(0))):
        assert np.array_equal(types, g["node_types"])
        for k, gk in KEYS[:6]:
            assert np.array_equal(b[k], g[gk]), k
        assert len(b["fluid_list"]) == 0
    assert int(g["nb"]) == 2880 and int(g["nb_fluid"]) == 0
    o.close()


@pytest.fixture(scope="module")
def golden_zwall():
    return np.load(GOLDEN / "ref_cylinder_zwall_geometry.npz")


def test_zwall_golden_fixture_is_consistent(golden_zwall):
    """Z_PERIODIC 0 build of the shipped case: BCSOLID nodes (class 6) only on the z = 0 and
    z = NZ-1 planes, inside the classification window, with fewer than four bulk octants."""
    g = golden_zwall
    t = g["node_types"]
    cls = t >> 20
    nx, ny, nz = (int(v) for v in g["shape"])
    assert int(g["z_periodic"]) == 0
    assert int(g["nb_solid"]) == int((cls == 6).sum()) == len(g["solid_list"]) > 0
    z = g["solid_list"] // (nx * ny)
    assert set(np.unique(z)) == {0, nz - 1}
    tags = t[g["solid_list"]] & 0xFF
    assert all(bin(int(v)).count("1") < 4 for v in tags)
    assert all(int(v) < 16 for v in tags[z == nz - 1]) and all(int(v) % 16 == 0 for v in tags[z == 0])
    # the eight tags with a closure (boundaries.cuh:1039-1214) all occur
    assert {7, 11, 13, 14, 112, 176, 208, 224} <= set(int(v) for v in tags)


def test_product_and_oracle_zwall_geometry_match_reference(built, golden_zwall):
    import oracle
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    desc = cases.reference_cylinder(periodic_z=False)
    s = Simulation(desc, host_only=True)
    o = oracle.Oracle(desc, 64)
    assert np.array_equal(s.node_types(), golden_zwall["node_types"])
    assert np.array_equal(o.node_types(), golden_zwall["node_types"])
    for b in (s.boundary(0), o.boundary(0)):
        for k, gk in KEYS + [("solid_list", "solid_list")]:
            assert np.array_equal(b[k], golden_zwall[gk]), k


@pytest.mark.parametrize("name", ["c1", "annulus_small", "annulus_ref", "channel_staircase", "cylinder_box_walls",
                                  "cylinder_z_walls", "annulus_z_walls"])
def test_product_and_oracle_classify_alike(built, name):
    import oracle
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    desc = {
        "c1": lambda: cases.c1_cylinder(),
        "annulus_small": lambda: cases.annulus(48, 48, 8, 8.0, 20.0, 0.05, 50.0),
        "annulus_ref": lambda: cases.reference_annulus(),
        "channel_staircase": lambda: cases.cylinder_channel(64, 32, 8, 8, 20.0, 15.5, 0.05, 40.0, triangular=False),
        "cylinder_box_walls": lambda: cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0),
        "cylinder_z_walls": lambda: cases.cylinder_channel(64, 40, 12, 10, 24.3, 19.7, 0.05, 60.0, periodic_z=False),
        "annulus_z_walls": lambda: cases.annulus(48, 48, 8, 8.0, 20.0, 0.05, 50.0, periodic_z=False),
    }[name]()
    s = Simulation(desc, host_only=True)
    o = oracle.Oracle(desc, 64)
    assert np.array_equal(s.node_types(), o.node_types())
    for w in range(2 if desc.geometry == 2 else 1):
        bs, bo = s.boundary(w), o.boundary(w)
        for k, _ in KEYS + [("solid_list", "")]:
            assert np.array_equal(bs[k], bo[k]), (w, k)
    if not desc.periodic[2]:
        assert (s.node_types() >> 20 == 6).sum() > 0
    cls = s.node_types() >> 20
    assert (cls == 2).any()
    if desc.geometry == 2:
        assert (cls == 3).any()


@pytest.mark.parametrize("variant", ["periodic_z", "z_walls"])
def test_geometry_files_match_reference_writer(built, tmp_path, variant):
    """grid_layout/*.dat byte for byte against the reference's own write_geometry_files
    (cylinder_helpers.cuh:388-470, run by the geometry harness; SHA-256 in the fixture)."""
    import hashlib
    import json
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    want = json.loads((GOLDEN / "ref_geometry_files.json").read_text())[variant]
    s = Simulation(cases.reference_cylinder(periodic_z=variant == "periodic_z"), host_only=True)
    s.write_geometry(tmp_path)
    got = {f.name: {"sha256": hashlib.sha256(f.read_bytes()).hexdigest(), "bytes": f.stat().st_size}
           for f in sorted(tmp_path.glob("*.dat"))}
    assert got == want
    if variant == "z_walls":
        assert want["bcsolid_inner.dat"]["bytes"] > 0


@pytest.mark.parametrize("fixture", ["ref_annulus_geometry.npz", "ref_annulus_zwall_geometry.npz"])
def test_product_and_oracle_annulus_geometry_match_reference(built, fixture):
    """The shipped annulus case (136 x 136 x 256, r 32 / 64), periodic in z and with z walls,
    against the reference's own classification of both walls (oracle/_ref/ref_geometry_annulus*,
    fixtures made by tests/golden/make_golden.py): every node type (SHA-256 of the whole array
    plus the end planes in full), each wall's list, normals, wall distances, masks and BCSOLID
    list, and the per-tag BCFLUID masks (the outer wall's pass writes last, as in
    annulus_kernels.cu:37-38)."""
    import hashlib
    import oracle
    from mrlbm_3d_cuda_gb300 import Simulation, cases
    g = np.load(GOLDEN / fixture)
    desc = cases.reference_annulus(periodic_z=bool(int(g["z_periodic"])))
    plane = desc.nx * desc.ny
    s = Simulation(desc, host_only=True)
    o = oracle.Oracle(desc, 64)
    for types, b0, b1 in ((s.node_types(), s.boundary(0), s.boundary(1)),
                          (o.node_types(), o.boundary(0), o.boundary(1))):
        assert np.array_equal(types[:plane], g["types_first_plane"])
        assert np.array_equal(types[-plane:], g["types_last_plane"])
        assert hashlib.sha256(types.astype(np.uint32).tobytes()).digest() == g["types_sha256"].tobytes()
        for w, b in (("inner", b0), ("outer", b1)):
            for k, gk in (("list", "boundary_list"), ("nx", "unit_nx"), ("ny", "unit_ny"), ("delta", "delta"),
                          ("in_mask", "in_mask"), ("out_mask", "out_mask"), ("fluid_list", "fluid_list"),
                          ("solid_list", "solid_list")):
                assert np.array_equal(b[k], g[f"{w}_{gk}"]), (w, k)
        assert np.array_equal(b0["tag_in_mask"], g["tag_in_mask"])
        assert np.array_equal(b0["tag_out_mask"], g["tag_out_mask"])
    assert list(g["nb"]) == [s.info.nb[0], s.info.nb[1]]
    assert list(g["nb_solid"]) == [s.info.nb_solid[0], s.info.nb_solid[1]]
    o.close()
