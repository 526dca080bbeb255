"""Build recipe for the oracle (test infrastructure): oracle/_build/liboracle.so.

The oracle is the CPU restatement of the reference time step in mrlbm_oracle.cpp, compiled
with OpenMP and without floating-point contraction so x86-64 and aarch64 round alike.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "mrlbm_oracle.cpp"
OUT = HERE / "_build" / "liboracle.so"


def build(force: bool = False) -> Path:
    hdr = HERE.parent / "include" / "mrlbm.h"
    if not force and OUT.exists() and OUT.stat().st_mtime > max(SRC.stat().st_mtime, hdr.stat().st_mtime):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-Wall", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
