"""ORACLE — test infrastructure only (tests/, __graft_entry__.smoke(), bench.py's cpu_baseline).

ctypes binding of oracle/_build/liboracle.so, the CPU restatement of the reference MR-LBM
time step (mrlbm_oracle.cpp).  T = float32 follows the reference's FP32 arithmetic order;
T = float64 is the FP64 oracle run.  Nothing in the product imports this package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build_oracle
from .build_oracle import OUT as LIB_PATH

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build_oracle.build()
        L = C.CDLL(str(LIB_PATH))
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.c_void_p, C.c_int]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_init.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.oracle_step.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.oracle_get_moments.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_set_moments.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_get_forces.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_get_node_types.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_get_frozen.argtypes = [C.c_void_p, C.c_void_p]
        L.oracle_wall_size.restype = C.c_int
        L.oracle_wall_size.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.oracle_get_boundary.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_omega.restype = C.c_float
        L.oracle_omega.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def omega(desc) -> float:
    """The oracle's own relaxation rate for `desc` (the reference's tau chain restated from the
    descriptor's u_max, Re and length scale; an explicit omega when Re is not set)."""
    return float(lib().oracle_omega(C.byref(desc)))


def periodic_box_desc(n: int, u0: float = 0.05, re: float = 1600.0):
    """Descriptor of the all-periodic n^3 Taylor-Green box (L = n / 2 pi), filled here without
    the solver library: the CPU legs of bench.py run on it without loading libmrlbm.so.  Only
    the fields the oracle reads are set; the relaxation rate is the oracle's own."""
    import math

    from mrlbm_3d_cuda_gb300.native import CaseDesc, GEOM_NONE
    d = CaseDesc()
    d.struct_size = C.sizeof(CaseDesc)
    d.geometry = GEOM_NONE
    d.nx = d.ny = d.nz = int(n)
    d.periodic[0] = d.periodic[1] = d.periodic[2] = 1
    d.u_max, d.rho0, d.re = float(u0), 1.0, float(re)
    d.length = float(n / (2.0 * math.pi))
    d.omega = 0.0
    for k in range(3):
        d.storage_scale[k] = 1.0
    return d


class Oracle:
    """CPU oracle for one case.  `desc` is a finalized mrlbm_3d_cuda_gb300.native.CaseDesc."""

    def __init__(self, desc, bits: int = 64):
        self.desc = desc
        self.n = desc.nx * desc.ny * desc.nz
        self.shape = (desc.nz, desc.ny, desc.nx)
        p = lib().oracle_create(C.byref(desc), bits)
        if not p:
            raise RuntimeError(lib().oracle_last_error().decode())
        self._p = C.c_void_p(p)

    def close(self):
        if self._p:
            lib().oracle_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self, kind: int, params=()):
        arr = (C.c_double * max(8, len(params)))(*params)
        lib().oracle_init(self._p, kind, arr)

    def step(self, n: int = 1, forces: bool = False):
        lib().oracle_step(self._p, int(n), 1 if forces else 0)

    def moments(self) -> np.ndarray:
        out = np.empty((10, self.n), dtype=np.float64)
        lib().oracle_get_moments(self._p, out.ctypes.data_as(C.c_void_p))
        return out.reshape((10,) + self.shape)

    def set_moments(self, m: np.ndarray):
        a = np.ascontiguousarray(m, dtype=np.float64).reshape(10, self.n)
        lib().oracle_set_moments(self._p, a.ctypes.data_as(C.c_void_p))

    def forces(self) -> np.ndarray:
        out = np.zeros(10, dtype=np.float64)
        lib().oracle_get_forces(self._p, out.ctypes.data_as(C.c_void_p))
        return out.reshape(2, 5)

    def node_types(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.uint32)
        lib().oracle_get_node_types(self._p, out.ctypes.data_as(C.c_void_p))
        return out

    def frozen(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.uint8)
        lib().oracle_get_frozen(self._p, out.ctypes.data_as(C.c_void_p))
        return out

    def boundary(self, wall: int = 0) -> dict:
        L = lib()
        nb = L.oracle_wall_size(self._p, wall, 0)
        nbf = L.oracle_wall_size(self._p, wall, 1)
        nbs = L.oracle_wall_size(self._p, wall, 2)
        spec = [("list", 0, np.int64, nb), ("nx", 1, np.float32, nb), ("ny", 2, np.float32, nb),
                ("delta", 3, np.float32, nb), ("in_mask", 4, np.uint32, nb), ("out_mask", 5, np.uint32, nb),
                ("fluid_list", 6, np.int64, nbf), ("tag_in_mask", 7, np.uint32, 256),
                ("tag_out_mask", 8, np.uint32, 256), ("solid_list", 9, np.int64, nbs)]
        res = {}
        for name, what, dt, n in spec:
            a = np.zeros(max(n, 1), dtype=dt)
            L.oracle_get_boundary(self._p, wall, what, a.ctypes.data_as(C.c_void_p))
            res[name] = a[:n]
        return res
