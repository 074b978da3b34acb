"""Writes the PVM fixtures tests/golden/pvm/*.pvm (this project's own seeded
volumes, plain and DDS-compressed by tests/pvmfmt.py) and
tests/golden/pvm_reference.npz: what the reference's own .pvm loader
(libs/file_utils/pvm.cpp, compiled in place by oracle/build_ref.py) reads
from each of them (dims, bytes per voxel, spacing, voxel bytes).

Run where the reference checkout is available:

    python tests/golden/make_pvm_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle  # noqa: E402
import pvmfmt  # noqa: E402

OUT_DIR = HERE / "pvm"
OUT_NPZ = HERE / "pvm_reference.npz"


def volumes():
    rng = np.random.default_rng(2024)
    noise = rng.integers(0, 256, size=(9, 11, 13)).astype(np.uint8)
    walk = np.cumsum(np.cumsum(rng.integers(-2, 3, size=(9, 11, 13)), axis=2), axis=1)
    smooth = ((walk - walk.min()) % 256).astype(np.uint8)
    wide = rng.integers(0, 65536, size=(5, 6, 7)).astype(np.uint16)
    return noise, smooth, wide


# name: (volume index, PVM version, DDS skip (0 = no DDS), strip, v3e blocks)
CASES = {
    "noise_v1_plain": (0, 1, 0, 0, False),
    "noise_v3_dds": (0, 3, 1, 1, False),
    "smooth_v2_dds_strip13": (1, 2, 1, 13, False),
    "smooth_v3e_strip143": (1, 3, 1, 143, True),
    "wide_u16_v3_dds_skip2": (2, 3, 2, 7, False),
    "wide_u16_v3e_skip2": (2, 3, 2, 1, True),
}


def main():
    if not oracle.ref_available():
        raise SystemExit("reference checkout not available: cannot regenerate the PVM golden data")
    ref = oracle.load_ref()
    vols = volumes()
    OUT_DIR.mkdir(exist_ok=True)
    out = {}
    for name, (vi, ver, skip, strip, blocks) in CASES.items():
        body = pvmfmt.pvm_bytes(vols[vi], version=ver, scale=(1.0, 1.5, 0.75), comments=("seeded test volume",))
        data = body if skip == 0 else pvmfmt.dds_file(body, skip, strip, blocks)
        path = OUT_DIR / f"{name}.pvm"
        path.write_bytes(data)
        dims = (C.c_int * 3)()
        comps = C.c_int()
        scale = (C.c_double * 3)()
        assert ref.ref_read_pvm(str(path).encode(), dims, C.byref(comps), scale, None, C.c_size_t(0)) == 0
        n = dims[0] * dims[1] * dims[2] * comps.value
        voxels = np.zeros(n, np.uint8)
        assert ref.ref_read_pvm(str(path).encode(), dims, C.byref(comps), scale, C.c_void_p(voxels.ctypes.data),
                                C.c_size_t(n)) == 0
        out[f"{name}_dims"] = np.array(list(dims), np.int32)
        out[f"{name}_components"] = np.array([comps.value], np.int32)
        out[f"{name}_scale"] = np.array(list(scale), np.float64)
        out[f"{name}_voxels"] = voxels
    np.savez_compressed(OUT_NPZ, **out)
    print(f"wrote {len(CASES)} fixtures to {OUT_DIR} and {OUT_NPZ}")


if __name__ == "__main__":
    main()
