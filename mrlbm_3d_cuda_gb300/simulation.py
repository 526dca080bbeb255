"""Python mirror of the reference's case / simulation interface over the C ABI.

The reference selects a case at compile time (MRLBM_3D/src/config.h:8), fills a `struct Case`
hook table (MRLBM_3D/src/common/globalStructs.cuh:46-62) and runs
``streaming -> boundary_treatment -> post_streaming -> collision -> post_collision ->
post_step`` per iteration (MRLBM_3D/src/main.cu:21-35).  Here a :class:`Simulation` owns one
libmrlbm handle; one ``step`` runs that whole chain on the GPU, and the host-side hooks
(``post_process_step``, ``write_output``) are plain Python callables run between steps at the
reference's cadences.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np

from . import native as N


@dataclass
class Case:
    """A case: the descriptor plus optional host hooks (the reference's `struct Case`)."""

    desc: N.CaseDesc
    name: str = "case"
    init_kind: int = N.INIT_REFERENCE_NOISE
    init_params: Sequence[float] = ()
    post_process_step: Optional[Callable[["Simulation", int], None]] = None
    write_output: Optional[Callable[["Simulation", int], None]] = None
    finalize: Optional[Callable[["Simulation"], None]] = None
    extra: dict = field(default_factory=dict)


class Simulation:
    """One MR-LBM case resident on the current CUDA device."""

    def __init__(self, case: Case | N.CaseDesc, init: bool = True, host_only: bool = False,
                 _handle: C.c_void_p | None = None):
        if isinstance(case, N.CaseDesc):
            case = Case(case)
        self.case = case
        L = N.lib()
        desc = N.CaseDesc.from_buffer_copy(case.desc)
        self._owned = _handle is None
        if _handle is None:
            h = C.c_void_p()
            create = L.mrlbm_create_host if host_only else L.mrlbm_create
            N.check(create(C.byref(desc), C.byref(h)))
        else:
            h = _handle
        if host_only:
            init = False
        self._h = h
        self.desc = desc
        self.info = self.get_info()
        self.n = int(self.info.n_nodes)
        self.shape = (self.info.nz, self.info.ny, self.info.nx)
        if init:
            self.init(case.init_kind, case.init_params)

    # ---- lifecycle ----------------------------------------------------------------------
    def close(self):
        """Destroy the handle (mrlbm_destroy) unless a batch owns it."""
        if getattr(self, "_h", None) is not None and self._h.value:
            if getattr(self, "_owned", True):
                N.lib().mrlbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _ck(self, rc):
        return N.check(rc, self._h)

    def autotune(self, trial_steps: int = 5) -> tuple:
        """Pick the fastest tile height / z-segment (results are tiling independent)."""
        t = (C.c_int32 * 3)()
        self._ck(N.lib().mrlbm_autotune(self._h, int(trial_steps), t))
        self.info = self.get_info()
        return tuple(t)

    def get_info(self) -> N.Info:
        """Sizes, wall counts, omega / tau, step, storage and tiling (mrlbm_get_info)."""
        info = N.Info()
        self._ck(N.lib().mrlbm_get_info(self._h, C.byref(info)))
        return info

    def set_stream(self, stream_ptr: int | None):
        """Launch on the caller's cudaStream_t (a raw handle; None or 0: the handle's own stream)."""
        self._ck(N.lib().mrlbm_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    # ---- time stepping ------------------------------------------------------------------
    def init(self, kind: int = N.INIT_REFERENCE_NOISE, params: Sequence[float] = ()):
        """Initial field (mrlbm_init): INIT_REFERENCE_NOISE reproduces the reference's initial
        state bit for bit; TAYLOR_GREEN (u0, L), UNIFORM (ux, uy, uz), NOISY_UNIFORM (ux, uy,
        uz, amplitude, seed), REST."""
        arr = (C.c_double * max(1, len(params)))(*params)
        self._ck(N.lib().mrlbm_init(self._h, kind, arr, len(params)))

    def step(self, n: int = 1):
        """Advance n time steps, asynchronously on the handle's stream (mrlbm_step)."""
        self._ck(N.lib().mrlbm_step(self._h, int(n)))

    def set_sampling(self, force_every: int = 0, diag_every: int = 0):
        """Record wall forces every force_every steps and FP64 mass / energy every diag_every steps
        (0: off)."""
        self._ck(N.lib().mrlbm_set_sampling(self._h, int(force_every), int(diag_every)))

    def sync(self):
        """Wait for the queued steps; raises on a device error or non-finite diagnostics
        (MRLBM_ERR_DIVERGED)."""
        self._ck(N.lib().mrlbm_sync(self._h))

    def run(self, max_iter: int, macr_save: int = 0, stat_start: int = 0, stat_end: int = -1):
        """The reference's main loop: iterations start..max_iter inclusive (main.cu:21)."""
        for it in range(0, max_iter + 1):
            self.step(1)
            if self.case.post_process_step and stat_start <= it and (stat_end < 0 or it <= stat_end):
                self.case.post_process_step(self, it)
            if self.case.write_output and macr_save and it % macr_save == 0:
                self.case.write_output(self, it)
        if self.case.finalize:
            self.case.finalize(self)

    # ---- fields -----------------------------------------------------------------------------
    def moments(self, fields="all", layout: int = N.LAYOUT_LEXICOGRAPHIC, out: np.ndarray | None = None) -> np.ndarray:
        """FP32 moments, shape (n_fields, nz, ny, nx) for the lexicographic layout."""
        mask = N.field_mask(fields)
        nf = bin(mask).count("1")
        if out is None:
            out = np.empty((nf, self.n), dtype=np.float32)
        self._ck(N.lib().mrlbm_get_moments(self._h, mask, layout, out.ctypes.data_as(C.c_void_p), out.size))
        if layout == N.LAYOUT_LEXICOGRAPHIC:
            return out.reshape((nf,) + self.shape)
        return out.reshape(nf, self.n)

    def set_moments(self, values: np.ndarray, fields="all", layout: int = N.LAYOUT_LEXICOGRAPHIC):
        """Upload FP32 moments (shape as moments() returns) into both ping-pong buffers, storage-
        encoded."""
        mask = N.field_mask(fields)
        v = N.as_f32(values)
        self._ck(N.lib().mrlbm_set_moments(self._h, mask, layout, v.ctypes.data_as(C.c_void_p), v.size))

    def node_types(self, layout: int = N.LAYOUT_LEXICOGRAPHIC) -> np.ndarray:
        """Node types in the reference's encoding: class << 20 | wall index or BCFLUID / BCSOLID
        tag."""
        out = np.empty(self.n, dtype=np.uint32)
        self._ck(N.lib().mrlbm_get_node_types(self._h, layout, out.ctypes.data_as(C.c_void_p), out.size))
        return out

    def boundary(self, wall: int = 0, layout: int = N.LAYOUT_LEXICOGRAPHIC) -> dict:
        """Boundary arrays of a curved wall: lists, normals, wall distances, direction masks,
        BCFLUID and BCSOLID node lists."""
        nb = int(self.info.nb[wall])
        nbf = int(self.info.nb_fluid[wall])
        nbs = int(self.info.nb_solid[wall])
        L = N.lib()
        res = {}
        spec = [("list", N.BND_LIST, np.int64, nb), ("nx", N.BND_NORMAL_X, np.float32, nb),
                ("ny", N.BND_NORMAL_Y, np.float32, nb), ("delta", N.BND_DELTA, np.float32, nb),
                ("in_mask", N.BND_IN_MASK, np.uint32, nb), ("out_mask", N.BND_OUT_MASK, np.uint32, nb),
                ("fluid_list", N.BND_FLUID_LIST, np.int64, nbf), ("tag_in_mask", N.BND_TAG_IN_MASK, np.uint32, 256),
                ("tag_out_mask", N.BND_TAG_OUT_MASK, np.uint32, 256), ("solid_list", N.BND_SOLID_LIST, np.int64, nbs)]
        for name, what, dt, n in spec:
            a = np.zeros(max(n, 1), dtype=dt)
            self._ck(L.mrlbm_get_boundary(self._h, wall, what, layout, a.ctypes.data_as(C.c_void_p), a.size))
            res[name] = a[:n]
        return res

    # ---- statistics -------------------------------------------------------------------------
    def forces(self, step: int = -1) -> np.ndarray:
        """(2 walls, 5) array: Fx, Fy, Fz, mass flux, torque_z of one sampled step."""
        out = np.zeros(10, dtype=np.float64)
        self._ck(N.lib().mrlbm_get_forces(self._h, int(step), out.ctypes.data_as(C.c_void_p)))
        return out.reshape(2, 5)

    def force_history(self, max_steps: int = 1 << 16):
        """(steps, forces) of the sampled steps still in the ring; forces shaped (n, 2 walls, 5)."""
        steps = np.zeros(max_steps, dtype=np.int64)
        f = np.zeros((max_steps, 10), dtype=np.float64)
        n = C.c_int32()
        self._ck(N.lib().mrlbm_get_force_history(self._h, max_steps, steps.ctypes.data_as(C.c_void_p),
                                                  f.ctypes.data_as(C.c_void_p), C.byref(n)))
        return steps[: n.value], f[: n.value].reshape(-1, 2, 5)

    def diagnostics(self, max_steps: int = 1 << 16):
        """Sampled (step, mass, kinetic energy) over non-solid nodes, FP64."""
        steps = np.zeros(max_steps, dtype=np.int64)
        v = np.zeros((max_steps, 2), dtype=np.float64)
        n = C.c_int32()
        self._ck(N.lib().mrlbm_get_diagnostics(self._h, max_steps, steps.ctypes.data_as(C.c_void_p),
                                                v.ctypes.data_as(C.c_void_p), C.byref(n)))
        return steps[: n.value], v[: n.value]

    # ---- files ------------------------------------------------------------------------------
    def checkpoint_save(self, path: str):
        """Write restart.bin in the reference's format (step, tiled moments, face populations)."""
        self._ck(N.lib().mrlbm_checkpoint_save(self._h, str(path).encode()))

    def checkpoint_load(self, path: str):
        """Load a restart.bin written by this library or by the reference."""
        self._ck(N.lib().mrlbm_checkpoint_load(self._h, str(path).encode()))

    def write_vti(self, path: str):
        """Write the current field as the reference's raw-appended .vti (rho, ux, uy, uz)."""
        self._ck(N.lib().mrlbm_write_vti(self._h, str(path).encode()))

    def write_forces(self, forces_path: str | None, mass_path: str | None = None, wall: int = 0,
                     append: bool = False):
        """forces.dat (`iter Fx Fy Fz`) and mass_flux.dat (`iter m`) of the sampled steps."""
        enc = (lambda p: str(p).encode() if p is not None else None)
        self._ck(N.lib().mrlbm_write_forces(self._h, int(wall), enc(forces_path), enc(mass_path), int(bool(append))))

    def set_pressure_window(self, start: int, end: int):
        """Statistics window: average the wall pressure and sample the inlet density over
        steps start..end (start < 0: off)."""
        self._ck(N.lib().mrlbm_set_pressure_window(self._h, int(start), int(end)))

    def write_pressure(self, path: str, wall: int = 0):
        """pressure.dat (`theta z Cp`) of the statistics window's averaged wall pressure."""
        self._ck(N.lib().mrlbm_write_pressure(self._h, int(wall), str(path).encode()))

    def write_inlet_density(self, path: str, append: bool = False):
        """inlet_density.dat (`iter rho_in rho_in_average`) of the statistics window."""
        self._ck(N.lib().mrlbm_write_inlet_density(self._h, str(path).encode(), int(bool(append))))

    def write_geometry(self, directory: str):
        """grid_layout/*.dat node lists of the z = 0 slice into `directory`."""
        self._ck(N.lib().mrlbm_write_geometry(self._h, str(directory).encode()))

    def run_reference_outputs(self, out_dir: str, max_iter: int, macr_save: int, stat_start: int, stat_end: int,
                              checkpoint_save: int = 0):
        """The reference's time loop with its output cadence (main.cu:21-35, simulation.cu:121-159):
        iterations 0..max_iter; data<10000000+it>.vti every macr_save iterations (master.pvd
        lists them); checkpoint/restart.bin (+ restart_step.txt) every checkpoint_save
        iterations after the first; forces / mass flux sampled and the wall pressure averaged
        over stat_start..stat_end, written as forces.dat, mass_flux.dat, pressure.dat and (cylinder)
        inlet_density.dat; the node lists of grid_layout/ at the start."""
        import os
        os.makedirs(out_dir, exist_ok=True)
        write_master_pvd(os.path.join(out_dir, "master.pvd"), macr_save, max_iter)
        walls = self.desc.geometry != N.GEOM_NONE
        if walls:
            os.makedirs(os.path.join(out_dir, "grid_layout"), exist_ok=True)
            self.write_geometry(os.path.join(out_dir, "grid_layout"))
        start = int(self.get_info().step)
        if walls:
            self.set_pressure_window(stat_start, stat_end)
        for it in range(start, max_iter + 1):
            stats = walls and stat_start <= it <= stat_end
            self.set_sampling(1 if stats else 0, 0)
            self.step(1)
            if checkpoint_save and it > start and it % checkpoint_save == 0:
                os.makedirs(os.path.join(out_dir, "checkpoint"), exist_ok=True)
                self.checkpoint_save(os.path.join(out_dir, "checkpoint", "restart.bin"))
                with open(os.path.join(out_dir, "checkpoint", "restart_step.txt"), "w") as f:
                    f.write(f"{it + 1}\n")
            if macr_save and it % macr_save == 0:
                self.write_vti(os.path.join(out_dir, f"data{10000000 + it}.vti"))
        self.set_sampling(0, 0)
        if walls:
            self.write_forces(os.path.join(out_dir, "forces.dat"), os.path.join(out_dir, "mass_flux.dat"))
            self.write_pressure(os.path.join(out_dir, "pressure.dat"))
            if self.desc.geometry == N.GEOM_CYLINDER:
                self.write_inlet_density(os.path.join(out_dir, "inlet_density.dat"))


def write_master_pvd(path: str, macr_save: int, max_iter: int):
    """master.pvd listing data<10000000+it>.vti for it = 0, macr_save, ... <= max_iter."""
    N.check(N.lib().mrlbm_write_master_pvd(str(path).encode(), int(macr_save), int(max_iter)))


class Batch:
    """Independent cases advanced together by batched, graph-replayed launches
    (mrlbm_batch_*).  `cases[i]` is a :class:`Simulation` view of case i for init, moments and
    forces; step the cases only through the batch."""

    def __init__(self, descs: Sequence[N.CaseDesc]):
        L = N.lib()
        arr = (N.CaseDesc * len(descs))(*[N.CaseDesc.from_buffer_copy(d) for d in descs])
        b = C.c_void_p()
        N.check(L.mrlbm_batch_create(arr, len(descs), C.byref(b)))
        self._b = b
        self.cases = []
        for i, d in enumerate(descs):
            h = C.c_void_p()
            N.check(L.mrlbm_batch_handle(b, i, C.byref(h)))
            self.cases.append(Simulation(d, init=False, _handle=h))
        self.n_nodes = sum(c.n for c in self.cases)

    def __len__(self):
        return len(self.cases)

    def close(self):
        """Destroy the batch and its cases (mrlbm_batch_destroy)."""
        if getattr(self, "_b", None) is not None and self._b.value:
            for c in self.cases:
                c.close()
            N.lib().mrlbm_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_sampling(self, force_every: int):
        """Record every case's wall forces every force_every steps (0: off)."""
        N.check(N.lib().mrlbm_batch_set_sampling(self._b, int(force_every)))

    def step(self, n: int = 1):
        """Advance every case n steps with the batched, graph-replayed launches."""
        N.check(N.lib().mrlbm_batch_step(self._b, int(n)))

    def step_sequential(self, n: int = 1):
        """Advance every case n steps with plain per-case launches (the unbatched comparison)."""
        N.check(N.lib().mrlbm_batch_step_sequential(self._b, int(n)))

    def autotune(self, trial_steps: int = 3) -> tuple:
        """Pick the fastest common tile height / z segment for the batch; state unchanged."""
        t = (C.c_int32 * 3)()
        N.check(N.lib().mrlbm_batch_autotune(self._b, int(trial_steps), t))
        for c in self.cases:
            c.info = c.get_info()
        return tuple(t)

    def sync(self):
        """Wait for the batch's queued steps."""
        N.check(N.lib().mrlbm_batch_sync(self._b))
