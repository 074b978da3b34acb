"""Builds oracle/_build/liboracle.so from oracle/cvr_oracle.cpp — TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
SRC = HERE / "cvr_oracle.cpp"
HDR = HERE.parent / "include" / "cvr.h"


def build(verbose: bool = False) -> Path:
    if LIB.exists() and LIB.stat().st_mtime > max(SRC.stat().st_mtime, HDR.stat().st_mtime):
        return LIB
    OUT.mkdir(exist_ok=True)
    cmd = ["g++", "-O3", "-fPIC", "-shared", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-Wall",
           "-o", str(LIB), str(SRC)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        print(r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
