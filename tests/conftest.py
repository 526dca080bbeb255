"""Shared test setup.

Markers: `gpu` — needs a GB300 (sm_103a); everything else runs on the CPU.  The solver
library and the oracle are built in-tree on first use (incremental)."""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (sm_103a)")


@pytest.fixture(scope="session")
def built():
    from mrlbm_3d_cuda_gb300 import build as B
    from oracle import build_oracle
    B.build()
    build_oracle.build()
    return True


@pytest.fixture(scope="session")
def cuda_device(built):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    cap = torch.cuda.get_device_capability(0)
    if cap != (10, 3):
        pytest.skip(f"needs sm_103 (GB300), found sm_{cap[0]}{cap[1]}")
    torch.cuda.init()
    return 0


# Field scales for the parity metric: the magnitude of each quantity as the algorithm
# computes it in FP32.  rho is evaluated as a full density (~rho0) before the rho0 offset is
# removed; u as j / rho; m_ab as Pi_ab / rho - cs2 delta_ab with Pi_ab / rho ~ cs2, so its
# FP32 rounding floor is set by cs2 = 1/3 rather than by |m_ab|.
def field_scales(u_ref: float):
    return np.array([1.0, u_ref, u_ref, u_ref] + [1.0 / 3.0] * 6)


def field_errors(a: np.ndarray, b: np.ndarray, u_ref: float):
    """Per-field (scaled max error, plain ||a-b||inf / ||b||inf, relative L2) of (10, ...) arrays."""
    a = np.asarray(a, dtype=np.float64).reshape(10, -1)
    b = np.asarray(b, dtype=np.float64).reshape(10, -1)
    sc = field_scales(u_ref)
    out = []
    for k in range(10):
        d = np.abs(a[k] - b[k])
        binf = np.abs(b[k]).max()
        out.append((d.max() / max(binf, sc[k]), d.max() / binf if binf > 0 else d.max(),
                    np.linalg.norm(a[k] - b[k]) / max(np.linalg.norm(b[k]), 1e-300)))
    return np.array(out)


FIELD_NAMES = ("rho", "ux", "uy", "uz", "mxx", "myy", "mzz", "mxy", "mxz", "myz")
_PARITY_LOG: dict = {}


def record_parity(name: str, err: np.ndarray, **extra):
    """Keep one test's per-field errors (rows of field_errors: floored, plain, L2) for the
    parity report that MRLBM_PARITY_REPORT=<path> asks for at the end of the session."""
    err = np.asarray(err)
    _PARITY_LOG[name] = {
        "floored": {f: float(err[k, 0]) for k, f in enumerate(FIELD_NAMES)},
        "plain": {f: float(err[k, 1]) for k, f in enumerate(FIELD_NAMES)},
        "l2": {f: float(err[k, 2]) for k, f in enumerate(FIELD_NAMES)},
        **{k: (v.tolist() if isinstance(v, np.ndarray) else v) for k, v in extra.items()},
    }


def pytest_sessionfinish(session, exitstatus):
    path = os.environ.get("MRLBM_PARITY_REPORT")
    if path and _PARITY_LOG:
        Path(path).parent.mkdir(parents=True, exist_ok=True)
        Path(path).write_text(json.dumps(_PARITY_LOG, indent=1, sort_keys=True))
