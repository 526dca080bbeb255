"""ctypes binding of libmrlbm.so (include/mrlbm.h).

This is the reference-side binding a Python caller uses; it adds nothing to the solver —
every call goes to the C ABI, which runs the sm_103a kernels.  Loading fails loudly when the
library has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libmrlbm.so"

# ---- constants mirrored from include/mrlbm.h ---------------------------------------------
OK = 0
ERR_INVALID_ARG, ERR_CUDA, ERR_DIVERGED, ERR_TIMEOUT, ERR_IO, ERR_UNSUPPORTED, ERR_STATE, ERR_NOMEM = (
    -1, -2, -3, -4, -5, -6, -7, -8)
GEOM_NONE, GEOM_CYLINDER, GEOM_ANNULUS = 0, 1, 2
STORAGE_F32, STORAGE_F16, STORAGE_BF16, STORAGE_F16_U32 = 0, 1, 2, 3
MASS_EQUILIBRIUM, MASS_STRONG = 0, 1
INIT_REFERENCE_NOISE, INIT_REST, INIT_TAYLOR_GREEN, INIT_UNIFORM, INIT_NOISY_UNIFORM = 0, 1, 2, 3, 4
LAYOUT_LEXICOGRAPHIC, LAYOUT_REF_TILED = 0, 1
# node classes in the high bits of a node type (common/nodeTypeMap.cuh:39-80 order)
NODE_BULK, NODE_SOLID, NODE_INNER, NODE_OUTER, NODE_BCFLUID_INNER, NODE_BCFLUID_OUTER, NODE_BCSOLID_INNER, \
    NODE_BCSOLID_OUTER, NODE_NORTH, NODE_SOUTH, NODE_EAST, NODE_WEST, NODE_FRONT, NODE_BACK = range(14)
FIELDS = ("rho", "ux", "uy", "uz", "mxx", "myy", "mzz", "mxy", "mxz", "myz")
FIELD_ALL = 0x3FF
BND_LIST, BND_NORMAL_X, BND_NORMAL_Y, BND_DELTA, BND_IN_MASK, BND_OUT_MASK, BND_FLUID_LIST, BND_TAG_IN_MASK, \
    BND_TAG_OUT_MASK, BND_SOLID_LIST = range(10)


class CaseDesc(C.Structure):
    _fields_ = [
        ("struct_size", C.c_uint32),
        ("geometry", C.c_int32),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("periodic", C.c_int32 * 3),
        ("u_max", C.c_float), ("rho0", C.c_float), ("re", C.c_float), ("length", C.c_float),
        ("omega", C.c_float),
        ("xc", C.c_float), ("yc", C.c_float),
        ("d_wall", C.c_float * 2),
        ("wall_u", (C.c_float * 3) * 2),
        ("scan_box", C.c_int32 * 4),
        ("triangular", C.c_int32),
        ("mass_bc", C.c_int32), ("bcf_mass_bc", C.c_int32),
        ("convective_outlet", C.c_int32), ("neumann_current_update", C.c_int32),
        ("storage", C.c_int32),
        ("storage_scale", C.c_float * 3),
        ("stochastic_rounding", C.c_int32),
        ("watchdog_every", C.c_int32),
        ("reserved", C.c_int32 * 14),
    ]


class Info(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("n_nodes", C.c_int64),
        ("nb", C.c_int32 * 2), ("nb_fluid", C.c_int32 * 2),
        ("omega", C.c_float), ("tau", C.c_float),
        ("step", C.c_int64),
        ("storage", C.c_int32), ("bytes_per_value", C.c_int32),
        ("n_active_items", C.c_int32),
        ("tile", C.c_int32 * 3),
        ("nb_solid", C.c_int32 * 2),
        ("reserved", C.c_int32 * 6),
    ]


class MrlbmError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


_lib = None

_SIGS = {
    "mrlbm_abi_version": (C.c_int, []),
    "mrlbm_case_desc_default": (C.c_int, [C.POINTER(CaseDesc), C.c_int32]),
    "mrlbm_case_desc_finalize": (C.c_int, [C.POINTER(CaseDesc)]),
    "mrlbm_create": (C.c_int, [C.POINTER(CaseDesc), C.POINTER(C.c_void_p)]),
    "mrlbm_create_host": (C.c_int, [C.POINTER(CaseDesc), C.POINTER(C.c_void_p)]),
    "mrlbm_destroy": (C.c_int, [C.c_void_p]),
    "mrlbm_last_error": (C.c_char_p, [C.c_void_p]),
    "mrlbm_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "mrlbm_get_info": (C.c_int, [C.c_void_p, C.POINTER(Info)]),
    "mrlbm_init": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int32]),
    "mrlbm_step": (C.c_int, [C.c_void_p, C.c_int32]),
    "mrlbm_set_sampling": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "mrlbm_sync": (C.c_int, [C.c_void_p]),
    "mrlbm_get_moments": (C.c_int, [C.c_void_p, C.c_uint32, C.c_int32, C.c_void_p, C.c_size_t]),
    "mrlbm_set_moments": (C.c_int, [C.c_void_p, C.c_uint32, C.c_int32, C.c_void_p, C.c_size_t]),
    "mrlbm_get_node_types": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_size_t]),
    "mrlbm_get_boundary": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_size_t]),
    "mrlbm_get_forces": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
    "mrlbm_get_force_history": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(C.c_int32)]),
    "mrlbm_get_diagnostics": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.POINTER(C.c_int32)]),
    "mrlbm_checkpoint_save": (C.c_int, [C.c_void_p, C.c_char_p]),
    "mrlbm_checkpoint_load": (C.c_int, [C.c_void_p, C.c_char_p]),
    "mrlbm_write_vti": (C.c_int, [C.c_void_p, C.c_char_p]),
    "mrlbm_write_master_pvd": (C.c_int, [C.c_char_p, C.c_int32, C.c_int32]),
    "mrlbm_write_forces": (C.c_int, [C.c_void_p, C.c_int32, C.c_char_p, C.c_char_p, C.c_int32]),
    "mrlbm_set_pressure_window": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64]),
    "mrlbm_write_pressure": (C.c_int, [C.c_void_p, C.c_int32, C.c_char_p]),
    "mrlbm_write_inlet_density": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int32]),
    "mrlbm_write_geometry": (C.c_int, [C.c_void_p, C.c_char_p]),
    "mrlbm_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "mrlbm_batch_create": (C.c_int, [C.POINTER(CaseDesc), C.c_int32, C.POINTER(C.c_void_p)]),
    "mrlbm_batch_destroy": (C.c_int, [C.c_void_p]),
    "mrlbm_batch_size": (C.c_int, [C.c_void_p]),
    "mrlbm_batch_handle": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]),
    "mrlbm_batch_set_sampling": (C.c_int, [C.c_void_p, C.c_int32]),
    "mrlbm_batch_step": (C.c_int, [C.c_void_p, C.c_int32]),
    "mrlbm_batch_step_sequential": (C.c_int, [C.c_void_p, C.c_int32]),
    "mrlbm_batch_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "mrlbm_batch_sync": (C.c_int, [C.c_void_p]),
    "mrlbm_step_periodic_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_float,
                                              C.c_float, C.c_void_p, C.c_void_p]),
}

EXPORTED = tuple(_SIGS)


def lib() -> C.CDLL:
    """Load libmrlbm.so (built by ``mrlbm_3d_cuda_gb300.build``); raise if it is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | getattr(os, "RTLD_LOCAL", 0))
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int, handle=None):
    if rc != OK:
        msg = lib().mrlbm_last_error(handle)
        raise MrlbmError(rc, msg.decode() if msg else "")
    return rc


def default_desc(geometry: int) -> CaseDesc:
    d = CaseDesc()
    check(lib().mrlbm_case_desc_default(C.byref(d), geometry))
    return d


def finalize(d: CaseDesc) -> CaseDesc:
    check(lib().mrlbm_case_desc_finalize(C.byref(d)))
    return d


def field_mask(fields) -> int:
    if fields is None or fields == "all":
        return FIELD_ALL
    m = 0
    for f in fields:
        m |= 1 << FIELDS.index(f)
    return m


def as_f32(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)
