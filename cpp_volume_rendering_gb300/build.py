"""In-tree build of libcvr.so (CUDA kernels for sm_103a + the C ABI + host C++).

Objects and the shared library go to cpp_volume_rendering_gb300/_build/.
Translation units compile in parallel and are skipped when up to date.
Host C++ is compiled with -ffp-contract=off so that x86 and Arm hosts produce
bit-identical tables (transfer functions, cone sections, kernel vectors).
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libcvr.so"
TOOL = BUILD / "cvr_headless"

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", f"-I{ROOT / 'include'}", f"-I{CSRC}"] + ARCH
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-Wall", "-Wno-unused-function",
             f"-I{ROOT / 'include'}", f"-I{CSRC}"]


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted((CSRC / "host").glob("*.cpp"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted((CSRC / "host").glob("*.hpp")) + [ROOT / "include" / "cvr.h"]
    return cu, cpp, headers


def _stale(obj: Path, deps) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    cu, cpp, headers = _sources()
    jobs = jobs or max(2, min(16, os.cpu_count() or 4))
    tasks = []
    objs = []
    for src in cu:
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            cmd = [NVCC] + NVCC_FLAGS + ["-Xptxas", "-v"] * verbose + ["-c", str(src), "-o", str(obj)]
            tasks.append(cmd)
    for src in cpp:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            tasks.append([CXX] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)])
    if tasks:
        with ThreadPoolExecutor(jobs) as ex:
            for err in ex.map(_run, tasks):
                if verbose and err:
                    sys.stderr.write(err)
    if tasks or _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] +
             ["-Xcompiler", "-fopenmp", "-lgomp"])
    # the headless driver links the library through an rpath next to it
    tool_src = CSRC / "tools" / "cvr_headless.cpp"
    if _stale(TOOL, [tool_src, LIB] + headers):
        _run([CXX] + CXX_FLAGS + [str(tool_src), "-o", str(TOOL), f"-L{BUILD}", "-lcvr",
                                  "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
