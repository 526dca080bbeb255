"""Case descriptors: the reference's shipped cases and the benchmark workloads.

The reference fixes a case at compile time in MRLBM_3D/src/cases/<case>/constants.cuh and
outputs.cuh; here each is a function returning a finalized :class:`native.CaseDesc`.
"""
from __future__ import annotations

import math

from . import native as N


def _finish(d: N.CaseDesc, storage: int = N.STORAGE_F32) -> N.CaseDesc:
    d.storage = storage
    return N.finalize(d)


def reference_cylinder(storage: int = N.STORAGE_F32, diameter: int = 16, *, periodic_z: bool = True) -> N.CaseDesc:
    """The reference's shipped cylinder case (cases/cylinder/constants.cuh:8-54):
    336 x 144 x 48, D = 16 at (71.5, 71.5), Re = 100, U = 0.1, periodic y and z, convective outlet.
    `diameter` rescales it as the reference's constants do when D is edited: LW = LN = LS = 4D,
    LE = 16D, NZ = 3D, centre LW + (D - 1) / 2, classification box +-4 nodes around the body.
    `periodic_z=False` is the reference built with Z_PERIODIC 0 (constants.cuh:10): no-slip
    z = 0 / NZ-1 faces, with BCSOLID nodes where they meet the body."""
    d = N.default_desc(N.GEOM_CYLINDER)
    d.periodic[2] = int(periodic_z)
    if diameter != 16:
        D = int(diameter)
        lw, le, ln = 4 * D, 16 * D, 4 * D
        d.nx, d.ny, d.nz = lw + D + le, 2 * ln + D, 3 * D
        d.d_wall[0] = float(D)
        d.xc = d.yc = lw + 0.5 * (D - 1)
        d.scan_box[0], d.scan_box[1], d.scan_box[2], d.scan_box[3] = lw - 4, lw + D + 4, ln - 4, ln + D + 4
        if d.length > 0:
            d.length = float(D)
    return _finish(d, storage)


def reference_annulus(storage: int = N.STORAGE_F32, *, periodic_z: bool = True) -> N.CaseDesc:
    """The reference's shipped annulus case (cases/annulus/constants.cuh:8-84):
    136 x 136 x 256, r = 32 / 64 about (67.5, 67.5), inner wall speed 0.03, Re = 70.
    `periodic_z=False` is that case with Z_PERIODIC 0 (constants.cuh:10)."""
    d = N.default_desc(N.GEOM_ANNULUS)
    d.periodic[2] = int(periodic_z)
    return _finish(d, storage)


def cylinder_channel(nx: int, ny: int, nz: int, d: float, xc: float, yc: float, u: float, re: float, *,
                     lw: int | None = None, ls: int | None = None, periodic_y: bool = False,
                     periodic_z: bool = True, convective: bool = False, storage: int = N.STORAGE_F32,
                     triangular: bool = True) -> N.CaseDesc:
    """Flow past a circular cylinder (axis z) in a channel: velocity inlet at x = 0,
    zero-gradient (or convective) outlet at x = nx-1, no-slip or periodic y, periodic or
    no-slip z (z walls add BCSOLID nodes where the z faces meet the body).
    `lw`, `ls` set the reference's classification window (LW-4 .. LW+D+4); by default it is
    centred on the cylinder."""
    desc = N.default_desc(N.GEOM_CYLINDER)
    desc.nx, desc.ny, desc.nz = nx, ny, nz
    desc.periodic[0], desc.periodic[1], desc.periodic[2] = 0, int(periodic_y), int(periodic_z)
    desc.d_wall[0] = float(d)
    desc.xc, desc.yc = float(xc), float(yc)
    desc.u_max, desc.re = float(u), float(re)
    desc.convective_outlet = int(convective)
    desc.triangular = int(triangular)
    if lw is None:
        lw = int(math.floor(xc - 0.5 * (d - 1)))
    if ls is None:
        ls = int(math.floor(yc - 0.5 * (d - 1)))
    di = int(math.ceil(d))
    desc.scan_box[0], desc.scan_box[1] = max(0, lw - 4), min(nx, lw + di + 4)
    desc.scan_box[2], desc.scan_box[3] = max(0, ls - 4), min(ny, ls + di + 4)
    return _finish(desc, storage)


def annulus(nx: int, ny: int, nz: int, r_in: float, r_out: float, u_inner: float, re: float, *,
            u_outer: float = 0.0, xc: float | None = None, yc: float | None = None,
            periodic_z: bool = True, storage: int = N.STORAGE_F32) -> N.CaseDesc:
    """Taylor-Couette annulus: concentric walls (axis z), wall speeds tangential in the
    rotated frame, Re on the gap width, periodic or no-slip z (BCSOLID nodes on both walls)."""
    desc = N.default_desc(N.GEOM_ANNULUS)
    desc.nx, desc.ny, desc.nz = nx, ny, nz
    desc.periodic[0], desc.periodic[1], desc.periodic[2] = 0, 0, int(periodic_z)
    desc.d_wall[0], desc.d_wall[1] = 2.0 * r_in, 2.0 * r_out
    desc.xc = 0.5 * (nx - 1) if xc is None else xc
    desc.yc = 0.5 * (ny - 1) if yc is None else yc
    desc.wall_u[0][0], desc.wall_u[0][1], desc.wall_u[0][2] = 0.0, float(u_inner), 0.0
    desc.wall_u[1][0], desc.wall_u[1][1], desc.wall_u[1][2] = 0.0, float(u_outer), 0.0
    desc.u_max = max(abs(u_inner), abs(u_outer))
    desc.re = float(re)
    desc.scan_box[0], desc.scan_box[1], desc.scan_box[2], desc.scan_box[3] = 0, nx, 0, ny
    return _finish(desc, storage)


def periodic_box(nx: int, ny: int | None = None, nz: int | None = None, *, u0: float = 0.05, re: float = 1600.0,
                 length: float | None = None, storage: int = N.STORAGE_F32) -> N.CaseDesc:
    """All-periodic box without walls (Taylor-Green vortex); L defaults to nx / 2 pi."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    desc = N.default_desc(N.GEOM_NONE)
    desc.nx, desc.ny, desc.nz = nx, ny, nz
    desc.u_max, desc.re = float(u0), float(re)
    desc.length = float(nx / (2.0 * math.pi) if length is None else length)
    return _finish(desc, storage)


# ---- benchmark workloads (seeded synthetic inputs of the named shapes) ----------------------

def c1_cylinder(storage: int = N.STORAGE_F32) -> N.CaseDesc:
    """Cylinder in a channel, 128 x 64 x 32, D = 16 at (32, 32), U = 0.05, zero-gradient outlet,
    no-slip y walls, periodic z, Re = 100 (2000 steps, rho = 1, u = 0 start)."""
    return cylinder_channel(128, 64, 32, 16, 32.0, 32.0, 0.05, 100.0, lw=24, ls=24, storage=storage)


def c2_taylor_green(n: int = 256, storage: int = N.STORAGE_F32) -> N.CaseDesc:
    """Taylor-Green vortex, periodic n^3, u0 = 0.05, Re = 1600, L = n / 2 pi."""
    return periodic_box(n, u0=0.05, re=1600.0, storage=storage)


def c3_annulus(storage: int = N.STORAGE_F32) -> N.CaseDesc:
    """Taylor-Couette annulus 160 x 160 x 128, r = 32 / 64 about (79.5, 79.5), inner wall 0.05,
    outer fixed, Re = 400 on the gap."""
    return annulus(160, 160, 128, 32.0, 64.0, 0.05, 400.0, storage=storage)


def c4_batch(n: int = 64, seed: int = 1234, storage: int = N.STORAGE_F32) -> list:
    """Independent cylinder-in-channel cases for batched stepping: per case D ~ U{8..40} and
    Re ~ U[20, 300) drawn in that order from numpy's default generator (PCG64) seeded with
    `seed`; Lx = 12D, Ly = 6D rounded up to multiples of 8 (<= 512 / 256), Lz = 3D rounded up
    to a multiple of 4 (<= 64), centre (4D, 3D), inlet u = 0.05, zero-gradient outlet,
    no-slip y walls, periodic z."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []

    def up(v, m):
        return ((v + m - 1) // m) * m

    for _ in range(n):
        d = int(rng.integers(8, 41))
        re = float(rng.uniform(20.0, 300.0))
        lx, ly, lz = min(up(12 * d, 8), 512), min(up(6 * d, 8), 256), min(up(3 * d, 4), 64)
        out.append(cylinder_channel(lx, ly, lz, d, 4.0 * d, 3.0 * d, 0.05, re, storage=storage))
    return out


def c5_turbulent_cylinder(storage: int = N.STORAGE_F16, re: float = 3900.0) -> N.CaseDesc:
    """Large cylinder: 1024 x 512 x 256, D = 64 at (256, 256), Re = 3900, U = 0.05."""
    return cylinder_channel(1024, 512, 256, 64, 256.0, 256.0, 0.05, re, storage=storage)


def tgv_params(desc: N.CaseDesc):
    """Initial-condition parameters (u0, L) of the Taylor-Green vortex for `desc`."""
    return (float(desc.u_max), float(desc.length))
