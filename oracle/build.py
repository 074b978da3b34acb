"""Builds oracle/_build/liboracle.so — TEST INFRASTRUCTURE ONLY.

Sources: cvr_oracle.cpp (the renderers restated from the reference shaders)
and oracle_tables.cpp (the transfer-function, cone-section and kernel-vector
tables and the seeded synthetic volumes), so the oracle needs nothing from the
product library.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
SRCS = [HERE / "cvr_oracle.cpp", HERE / "oracle_tables.cpp"]
HDR = HERE.parent / "include" / "cvr.h"


def build(verbose: bool = False) -> Path:
    deps = SRCS + [HDR]
    if LIB.exists() and LIB.stat().st_mtime > max(p.stat().st_mtime for p in deps):
        return LIB
    OUT.mkdir(exist_ok=True)
    cmd = ["g++", "-O3", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-Wall",
           "-o", str(LIB)] + [str(s) for s in SRCS]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        print(r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
