"""Generates tests/golden/reference_tables.npz from the reference's own C++.

Run where the reference checkout is available (it is compiled in place into
oracle/_ref/ by oracle/build_ref.py); the GPU machine and other machines then use
the committed .npz.  Every array is produced by reference code:
  tf_*        vis::TransferFunction1D (Get / GetExtN / opacity<->extinction)
  sat_*       vis::SummedAreaTable3D<double>::BuildSAT on a small grid
  cone_*      ConeGaussianSampler::ComputeConeIntegrationSteps
  gt_*        RodriguesRotation + std::default_random_engine as in
              RC1PConeLightGroundTruthSteps::Update
  grad_*      GenerateSobelFeldmanGradientTexture / GenerateGradientTexture
              (the float RGB texels they upload) on small u8 / u16 volumes
  filt_*      the image reconstruction kernels (filters/*.hpp operator())
              on a grid of x, and the B-spline / OMOMS digital filters on a line
The inputs (control points, grid values, sampler settings) are this
project's own test values.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_tables.npz"

# Transfer functions exercised: the benchmark TF and an own multi-segment one
# with a flat run, plus an extinction-input TF with a larger max density.
TFS = {
    "bench": dict(md=255, ext=0,
                  rgb=[(0.20, 0.30, 0.90, 0), (0.30, 0.80, 0.40, 80), (0.90, 0.70, 0.20, 160), (1.00, 0.95, 0.90, 255)],
                  alpha=[(0.0, 0), (0.05, 80), (0.4, 160), (0.9, 255)]),
    "steps": dict(md=255, ext=0,
                  rgb=[(0.1, 0.7, 0.1, 0), (0.1, 0.7, 0.1, 40), (0.0, 0.0, 0.0, 41), (0.65, 0.3, 0.05, 42),
                       (0.85, 0.6, 0.1, 255)],
                  alpha=[(0.0, 0), (0.0, 30), (0.45, 37), (0.7, 255)]),
    "extin": dict(md=1023, ext=1,
                  rgb=[(1.0, 0.0, 0.0, 0), (0.0, 0.0, 1.0, 1023)],
                  alpha=[(0.0, 0), (3.5, 600), (0.25, 1023)]),
}

CONES = {
    # name: (half angle, packing, covered distance, initial step, min sigma)
    "occ_default": (20.0, 1, 0.5 * 443.40500673763256, 3.0, 1.0),
    "sdw_default": (0.5, 0, 0.75 * 443.40500673763256, 3.0, 1.0),
    "occ_wide7": (45.0, 2, 150.0, 3.0, 1.0),
    "occ_small": (30.0, 2, 40.0, 2.0, 0.5),
}


def arr(pts, n):
    a = np.zeros((max(len(pts), 1), n), np.float64)
    for i, p in enumerate(pts):
        a[i] = p
    return np.ascontiguousarray(a)


# name: (model, gradient_sample_size, filter_nxnxn, normalized_gradient)
GRADIENT_CASES = {
    "sobel": (0, 1, 0, 1),
    "fd": (1, 1, 0, 1),
    "fd_n2_raw": (1, 2, 0, 0),
    "fd_filter3": (1, 1, 3, 1),
}


def gradient_volumes():
    """A u8 volume with a smooth blob, flat runs and noise (ragged dims), and
    a u16 one with full-range values."""
    rng = np.random.default_rng(11)
    z, y, x = np.meshgrid(np.arange(8), np.arange(9), np.arange(10), indexing="ij")
    blob = 255.0 * np.exp(-((x - 4.5) ** 2 + (y - 3.0) ** 2 + (z - 4.0) ** 2) / 9.0)
    u8 = np.clip(blob + rng.integers(-3, 4, size=blob.shape), 0, 255).astype(np.uint8)
    u8[:, :, 7:] = 40  # flat slab: zero gradients inside it
    u16 = rng.integers(0, 65536, size=(6, 7, 5)).astype(np.uint16)
    return {"u8": np.ascontiguousarray(u8), "u16": np.ascontiguousarray(u16)}


def main():
    if not oracle.ref_available():
        raise SystemExit("reference checkout not available: cannot regenerate golden vectors")
    ref = oracle.load_ref()
    P = C.c_void_p
    out = {}
    for name, t in TFS.items():
        rgb, al = arr(t["rgb"], 4), arr(t["alpha"], 2)
        n = t["md"] + 1
        rgbt = np.zeros((n, 4), np.float32)
        rgba = np.zeros((n, 4), np.float32)
        ref.ref_tf_tables(t["md"], len(t["rgb"]), P(rgb.ctypes.data), len(t["alpha"]), P(al.ctypes.data), t["ext"],
                          P(rgbt.ctypes.data), P(rgba.ctypes.data))
        out[f"tf_{name}_rgbt"] = rgbt
        out[f"tf_{name}_rgba"] = rgba
        for bpv in ((1, 2) if name == "bench" else (1,)):
            e = np.zeros(256 if bpv == 1 else 65536, np.float64)
            ref.ref_tf_ext_per_value(t["md"], len(t["rgb"]), P(rgb.ctypes.data), len(t["alpha"]), P(al.ctypes.data),
                                     t["ext"], bpv, P(e.ctypes.data))
            out[f"tf_{name}_ext_u{8 * bpv}"] = e
    # SAT of a ragged grid with a zero border (the shape GenerateExtinctionSAT3DTex builds).
    rng = np.random.default_rng(7)
    cells = np.zeros((7, 6, 9), np.float64)
    cells[1:-1, 1:-1, 1:-1] = rng.uniform(0.0, 2.5, size=(5, 4, 7))
    sat = np.zeros_like(cells)
    ref.ref_sat_build(9, 6, 7, P(cells.ctypes.data), P(sat.ctypes.data))
    out["sat_cells"] = cells
    out["sat_ref"] = sat
    for name, (ang, pk, cov, ist, sg) in CONES.items():
        secs = np.zeros((512, 4), np.float64)
        counts = np.zeros(3, np.int32)
        axes = np.zeros((10, 3), np.float32)
        w7 = C.c_double()
        n = ref.ref_cone_sampler(C.c_float(ang), pk, C.c_float(cov), C.c_float(ist), C.c_double(sg), 512,
                                 P(secs.ctypes.data), P(counts.ctypes.data), P(axes.ctypes.data), C.byref(w7))
        assert n > 0
        out[f"cone_{name}_sections"] = secs[:n]
        out[f"cone_{name}_counts"] = counts
        out[f"cone_{name}_axes"] = axes
        out[f"cone_{name}_w7"] = np.array([w7.value])
    for name, (n_occ, a_occ, n_sdw, a_sdw, seed) in {"default": (16, 90.0, 1, 0.0, 1),
                                                     "mixed": (24, 60.0, 8, 1.0, 5)}.items():
        occ = np.zeros((n_occ, 3), np.float32)
        sdw = np.zeros((n_sdw, 3), np.float32)
        ref.ref_gt_vectors(n_occ, C.c_float(a_occ), n_sdw, C.c_float(a_sdw), seed, P(occ.ctypes.data),
                           P(sdw.ctypes.data))
        out[f"gt_{name}_occ"] = occ
        out[f"gt_{name}_sdw"] = sdw
    for name, vol in gradient_volumes().items():
        d, h, w = vol.shape
        out[f"grad_{name}_volume"] = vol
        for cfg, (model, n, filt, norm) in GRADIENT_CASES.items():
            g = np.zeros((d, h, w, 3), np.float32)
            r = ref.ref_gradient(P(vol.ctypes.data), w, h, d, vol.itemsize, model, n, filt, norm, P(g.ctypes.data))
            assert r == 0
            out[f"grad_{name}_{cfg}"] = g
    xs = np.linspace(-2.6, 2.6, 1041).astype(np.float32)
    out["filt_x"] = xs
    for k in range(6):
        wts = np.zeros_like(xs)
        sup = C.c_int()
        assert ref.ref_filter_weights(k, P(xs.ctypes.data), len(xs), P(wts.ctypes.data), C.byref(sup)) == 0
        out[f"filt_{k}_weights"] = wts
        out[f"filt_{k}_support"] = np.array([sup.value], np.int32)
    line = np.random.default_rng(13).uniform(0.0, 1.0, size=53).astype(np.float32)
    out["filt_line"] = line
    for k in (4, 5):
        g = line.copy()
        assert ref.ref_digital_filter(k, P(g.ctypes.data), len(g)) == 0
        out[f"filt_{k}_digital"] = g
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    main()
