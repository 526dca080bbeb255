"""GB300-native D3Q27 moment-representation LBM (MR-LBM) solver.

The solver itself is libmrlbm.so (C ABI in include/mrlbm.h, sm_103a kernels in csrc/);
this package builds it in-tree and binds it with ctypes:

    from mrlbm_3d_cuda_gb300 import Simulation, cases
    sim = Simulation(cases.reference_cylinder())
    sim.step(100)
    rho, ux, uy = sim.moments(["rho", "ux", "uy"])
"""
from . import native
from .native import MrlbmError
from .simulation import Batch, Case, Simulation
from . import cases

__all__ = ["native", "MrlbmError", "Batch", "Case", "Simulation", "cases"]
