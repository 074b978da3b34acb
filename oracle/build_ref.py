"""Builds oracle/_ref/libcvr_ref.so — TEST INFRASTRUCTURE ONLY.

Compiles the reference's own CPU table builders from its sources, in place
(nothing is copied into this repository), together with oracle/ref_shim.cpp:
  libs/volvis_utils/transferfunction1d.cpp, transferfunction.cpp,
  libs/volvis_utils/utils.cpp, structuredgridvolume.cpp, gridvolume.cpp
  (the gradient builders), libs/file_utils/pvm.cpp (the PVM / DDS reader; its
  MSVC runtime calls are mapped by oracle/ref_compat.h),
  libs/math_utils/utils.cpp,
  cppvolrend/structured/rc1pdosct/conegaussiansampler.cpp,
  libs/vis_utils/summedareatable.h (header only).
The reference checkout must be present ($CVR_REFERENCE_ROOT, or a `reference`
directory beside this repository, where fixtures are generated); without it
this script does nothing and the tests that need the library skip.
Output goes only to oracle/_ref/.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libcvr_ref.so"


def reference_root() -> Path | None:
    """The reference checkout: $CVR_REFERENCE_ROOT, else a `reference`
    directory beside this repository."""
    env = os.environ.get("CVR_REFERENCE_ROOT")
    p = Path(env) if env else HERE.parent.parent / "reference"
    return p if (p / "libs" / "vis_utils" / "summedareatable.h").exists() else None


def build(verbose: bool = False) -> Path | None:
    ref = reference_root()
    if ref is None:
        return None
    srcs = [
        HERE / "ref_shim.cpp",
        ref / "libs/volvis_utils/transferfunction1d.cpp",
        ref / "libs/volvis_utils/transferfunction.cpp",
        ref / "libs/math_utils/utils.cpp",
        ref / "cppvolrend/structured/rc1pdosct/conegaussiansampler.cpp",
        ref / "libs/volvis_utils/utils.cpp",
        ref / "libs/volvis_utils/structuredgridvolume.cpp",
        ref / "libs/volvis_utils/gridvolume.cpp",
        ref / "libs/file_utils/pvm.cpp",
    ]
    if LIB.exists() and all(s.stat().st_mtime < LIB.stat().st_mtime for s in srcs):
        return LIB
    OUT.mkdir(exist_ok=True)
    cmd = ["g++", "-O2", "-fPIC", "-shared", "-std=c++14", "-ffp-contract=off", "-fopenmp", "-w", "-fpermissive",
           "-DGLEW_NO_GLU", "-DGLEW_STATIC", "-include", str(HERE / "ref_compat.h"),
           # math_utils/matrix.h is not needed by these files and trips a GCC
           # template-shadowing error; its include guard is pre-defined.
           "-DMATH_UTILS_T_MATRIX_H",
           f"-I{ref / 'libs'}", f"-I{ref / 'include'}", f"-I{ref / 'cppvolrend'}",
           "-o", str(LIB)] + [str(s) for s in srcs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
