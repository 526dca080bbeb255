"""FP64 oracle run of the 256^3 Taylor-Green vortex as configured: the energy curve that
FP32 / FP16 / BF16 storage on the GPU are compared against.

Workload: periodic 256^3, u0 = 0.05, Re = 1600, L = 256 / 2 pi, u = u0 sin(x/L) cos(y/L)
cos(z/L), v = -u0 cos(x/L) sin(y/L) cos(z/L), w = 0, rho from p - p0 = rho0 u0^2 / 16
(cos 2x/L + cos 2y/L)(cos 2z/L + 2), m_ab = u_a u_b; 5000 steps.  Every 50 steps (and at 0)
the script records

    E(t) = sum over nodes of |u|^2 / 2 (FP64),   mass(t) = sum over nodes of rho,

the same sums the solver's diagnostics sampling returns.  The oracle is the CPU restatement
of the reference step in double precision (oracle/mrlbm_oracle.cpp); the run takes about an
hour on 16 cores.

    python tests/golden/make_tgv_energy_golden.py tests/golden/tgv256_fp64_energy.npz [n] [steps] [every]
"""
from __future__ import annotations

import math
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def sums(o):
    m = o.moments().reshape(10, -1)
    e = 0.5 * float(np.sum(m[1] * m[1] + m[2] * m[2] + m[3] * m[3]))
    mass = float(m[0].size * float(o.desc.rho0) + np.sum(m[0]))
    return e, mass


def main(out: str, n: int = 256, steps: int = 5000, every: int = 50):
    import oracle
    desc = oracle.periodic_box_desc(n, 0.05, 1600.0)
    o = oracle.Oracle(desc, 64)
    o.init(2, (float(np.float32(0.05)), n / (2 * math.pi)))  # INIT_TAYLOR_GREEN
    t_steps, energy, mass = [], [], []
    t0 = time.time()
    for s in range(0, steps + 1, every):
        if s:
            o.step(every)
        e, m = sums(o)
        t_steps.append(s)
        energy.append(e)
        mass.append(m)
        print(f"step {s:5d}  E {e:.12e}  mass {m:.12e}  ({time.time() - t0:.0f} s)", flush=True)
        np.savez_compressed(out, steps=np.array(t_steps, dtype=np.int64), energy=np.array(energy),
                            mass=np.array(mass), n=np.int64(n), u0=np.float64(np.float32(0.05)),
                            re=np.float64(1600.0), omega=np.float64(oracle.omega(desc)),
                            complete=np.int32(s == steps))
    o.close()


if __name__ == "__main__":
    a = sys.argv[1:]
    main(a[0], *(int(v) for v in a[1:]))
