"""Host-side tables against the reference's own code (golden vectors generated
by tests/golden/make_golden.py from the reference's C++), CPU only."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from cpp_volume_rendering_gb300 import abi, scene

GOLD = np.load(Path(__file__).parent / "golden" / "reference_tables.npz")

TFS = {
    "bench": (255, 0, [(0.20, 0.30, 0.90, 0), (0.30, 0.80, 0.40, 80), (0.90, 0.70, 0.20, 160),
                       (1.00, 0.95, 0.90, 255)],
              [(0.0, 0), (0.05, 80), (0.4, 160), (0.9, 255)]),
    "steps": (255, 0, [(0.1, 0.7, 0.1, 0), (0.1, 0.7, 0.1, 40), (0.0, 0.0, 0.0, 41), (0.65, 0.3, 0.05, 42),
                       (0.85, 0.6, 0.1, 255)],
              [(0.0, 0), (0.0, 30), (0.45, 37), (0.7, 255)]),
    "extin": (1023, 1, [(1.0, 0.0, 0.0, 0), (0.0, 0.0, 1.0, 1023)], [(0.0, 0), (3.5, 600), (0.25, 1023)]),
}


@pytest.mark.parametrize("name", list(TFS))
def test_tf_tables_match_reference_bit_exact(lib, name):
    md, ext, rgb, al = TFS[name]
    tf = scene.TransferFunction(rgb, al, md, bool(ext))
    rgbt, rgba = tf.tables()
    assert np.array_equal(rgbt, GOLD[f"tf_{name}_rgbt"])
    assert np.array_equal(rgba, GOLD[f"tf_{name}_rgba"])
    e8 = tf.ext_per_value(abi.CVR_U8)
    assert np.array_equal(e8, GOLD[f"tf_{name}_ext_u8"])
    if f"tf_{name}_ext_u16" in GOLD:
        assert np.array_equal(tf.ext_per_value(abi.CVR_U16), GOLD[f"tf_{name}_ext_u16"])


def test_tf_known_answers(lib):
    """Hand-computed entries of BuildLinear for the benchmark points."""
    rgbt, rgba = scene.BENCH_TF.tables()
    assert rgba[0, 3] == 0.0 and rgbt[0, 3] == 0.0
    assert rgba[80, 3] == np.float32(0.05)
    # halfway between 80 (0.05) and 160 (0.4): float(0.4 - 0.05) widened, k = 0.5
    a120 = np.float64(np.float32(0.05)) + np.float64(np.float32(0.4) - np.float32(0.05)) * 0.5
    assert rgba[120, 3] == np.float32(a120)
    assert rgbt[255, 3] == np.float32(np.log(1.0 / (1.0 - np.float64(np.float32(0.9)))))
    assert abs(rgbt[255, 3] - np.log(10.0)) < 1e-6


def test_cone_tables_match_reference(lib):
    cases = {"occ_default": (20.0, 1, 0.5 * 443.40500673763256, 3.0, 1.0),
             "sdw_default": (0.5, 0, 0.75 * 443.40500673763256, 3.0, 1.0),
             "occ_wide7": (45.0, 2, 150.0, 3.0, 1.0),
             "occ_small": (30.0, 2, 40.0, 2.0, 0.5)}
    for name, (ang, pk, cov, ist, sg) in cases.items():
        t = scene.cone_table(ang, pk, cov, ist, 1.0, sg)
        ref = GOLD[f"cone_{name}_sections"]
        n = t.n_sections
        assert n == len(ref), name
        got = np.array([[t.sections[i][k] for k in range(4)] for i in range(n)], np.float32)
        assert np.array_equal(got, ref.astype(np.float32)), name
        assert list(t.integration_samples) == list(GOLD[f"cone_{name}_counts"]), name
        axes = np.array([[t.axes[i][k] for k in range(3)] for i in range(10)], np.float32)
        assert np.array_equal(axes, GOLD[f"cone_{name}_axes"]), name
        assert np.float32(t.ray7_adj_weight) == np.float32(GOLD[f"cone_{name}_w7"][0])


def test_gt_kernel_vectors_match_reference(lib):
    for name, (n_occ, a_occ, n_sdw, a_sdw, seed) in {"default": (16, 90.0, 1, 0.0, 1),
                                                     "mixed": (24, 60.0, 8, 1.0, 5)}.items():
        occ, sdw = scene.gt_vectors(n_occ, a_occ, n_sdw, a_sdw, seed)
        assert np.array_equal(occ, GOLD[f"gt_{name}_occ"]), name
        assert np.array_equal(sdw, GOLD[f"gt_{name}_sdw"]), name
        # unit vectors inside the aperture around +z
        assert np.allclose(np.linalg.norm(occ, axis=1), 1.0, atol=1e-6)
        assert (occ[:, 2] >= np.cos(np.radians(a_occ)) - 1e-6).all()


def test_oracle_sat_matches_reference_builder(oracle_mod):
    cells = GOLD["sat_cells"]
    ref = GOLD["sat_ref"]
    # The oracle's builder takes a volume + per-value extinction; encode the
    # interior cells as u16 voxel values indexing an extinction table.
    inner = cells[1:-1, 1:-1, 1:-1]
    vals = np.arange(inner.size, dtype=np.uint16).reshape(inner.shape)
    ext = np.zeros(65536)
    ext[: inner.size] = inner.ravel()
    o = oracle_mod.Oracle()
    o.set_volume(vals, (1.0, 1.0, 1.0))
    o.build_sat(ext)
    got = o.sat()
    assert got.shape == ref.shape
    assert np.array_equal(got, ref)  # same recurrence, same FP64 order


def test_sat_i64_reconstructs_voxels(oracle_mod):
    """The commented-out self-check of GenerateExtinctionSAT3DTex
    (ebsrenderer.cpp:666-697): every cell equals its 8-corner difference."""
    rng = np.random.default_rng(3)
    vol = rng.integers(0, 256, size=(5, 6, 7), dtype=np.uint8)
    q = rng.integers(0, 1 << 40, size=256, dtype=np.int64)
    s = oracle_mod.sat_i64(vol, q)
    d = (s[1:, 1:, 1:] - s[:-1, 1:, 1:] - s[1:, :-1, 1:] - s[1:, 1:, :-1] + s[:-1, :-1, 1:] + s[:-1, 1:, :-1]
         + s[1:, :-1, :-1] - s[:-1, :-1, :-1])
    assert np.array_equal(d[:-1, :-1, :-1], q[vol])
    assert (d[-1] == 0).all() and (d[:, -1] == 0).all() and (d[:, :, -1] == 0).all()


def test_synthetic_volumes_deterministic(lib):
    a = scene.synth_blobs(17, 13, 11, abi.CVR_U8, 8, seed=5)
    b = scene.synth_blobs(17, 13, 11, abi.CVR_U8, 8, seed=5)
    c = scene.synth_blobs(17, 13, 11, abi.CVR_U8, 8, seed=6)
    assert a.shape == (11, 13, 17) and np.array_equal(a, b) and not np.array_equal(a, c)
    n1 = scene.synth_value_noise(16, 16, 16, abi.CVR_U16, seed=1)
    n2 = scene.synth_value_noise(16, 16, 16, abi.CVR_U16, seed=1)
    assert np.array_equal(n1, n2)
    levels = np.unique(n1)
    assert len(levels) <= 5  # 4 nested shells -> at most 5 distinct values


# ---- the oracle's own table builders and generators (it never loads libcvr.so)


@pytest.mark.parametrize("name", list(TFS))
def test_oracle_tf_tables_match_reference_bit_exact(oracle_mod, name):
    md, ext, rgb, al = TFS[name]
    tf = scene.TransferFunction(rgb, al, md, bool(ext))
    rgbt, rgba = oracle_mod.GEN.tf_tables(tf)
    assert np.array_equal(rgbt, GOLD[f"tf_{name}_rgbt"])
    assert np.array_equal(rgba, GOLD[f"tf_{name}_rgba"])
    assert np.array_equal(oracle_mod.GEN.tf_ext_per_value(tf, abi.CVR_U8), GOLD[f"tf_{name}_ext_u8"])
    if f"tf_{name}_ext_u16" in GOLD:
        assert np.array_equal(oracle_mod.GEN.tf_ext_per_value(tf, abi.CVR_U16), GOLD[f"tf_{name}_ext_u16"])


def test_oracle_cone_tables_match_reference(oracle_mod):
    cases = {"occ_default": (20.0, 1, 0.5 * 443.40500673763256, 3.0, 1.0),
             "sdw_default": (0.5, 0, 0.75 * 443.40500673763256, 3.0, 1.0),
             "occ_wide7": (45.0, 2, 150.0, 3.0, 1.0),
             "occ_small": (30.0, 2, 40.0, 2.0, 0.5)}
    for name, (ang, pk, cov, ist, sg) in cases.items():
        t = oracle_mod.GEN.cone_table(ang, pk, cov, ist, 1.0, sg)
        ref = GOLD[f"cone_{name}_sections"]
        n = t.n_sections
        assert n == len(ref), name
        got = np.array([[t.sections[i][k] for k in range(4)] for i in range(n)], np.float32)
        assert np.array_equal(got, ref.astype(np.float32)), name
        assert list(t.integration_samples) == list(GOLD[f"cone_{name}_counts"]), name
        axes = np.array([[t.axes[i][k] for k in range(3)] for i in range(10)], np.float32)
        assert np.array_equal(axes, GOLD[f"cone_{name}_axes"]), name
        assert np.float32(t.ray7_adj_weight) == np.float32(GOLD[f"cone_{name}_w7"][0])


def test_oracle_gt_kernel_vectors_match_reference(oracle_mod):
    for name, (n_occ, a_occ, n_sdw, a_sdw, seed) in {"default": (16, 90.0, 1, 0.0, 1),
                                                     "mixed": (24, 60.0, 8, 1.0, 5)}.items():
        occ, sdw = oracle_mod.GEN.gt_vectors(n_occ, a_occ, n_sdw, a_sdw, seed)
        assert np.array_equal(occ, GOLD[f"gt_{name}_occ"]), name
        assert np.array_equal(sdw, GOLD[f"gt_{name}_sdw"]), name


def test_oracle_generators_equal_library_generators(lib, oracle_mod):
    """The workloads' seeded volumes: the oracle's restated generators give the
    library's bytes, so a CPU reference can build every workload on its own."""
    g = oracle_mod.GEN
    for args in [(17, 13, 11, abi.CVR_U8, 8, 5, 0.0), (21, 9, 14, abi.CVR_U16, 32, 3000, 20.0),
                 (16, 16, 16, abi.CVR_U8, 32, 4020, 20.0)]:
        assert np.array_equal(g.synth_blobs(*args), scene.synth_blobs(*args)), args
    for args in [(16, 16, 16, abi.CVR_U16, 1), (23, 17, 29, abi.CVR_U16, 2000), (40, 24, 32, abi.CVR_U8, 9)]:
        assert np.array_equal(g.synth_value_noise(*args), scene.synth_value_noise(*args)), args


def test_oracle_workload_builds_without_the_library(oracle_mod):
    """scene.workload(..., gen=oracle.GEN) yields the same volume and tables as
    the library's builders."""
    for name in ("extinction", "cone", "ground_truth", "plain"):
        a = scene.workload(name, n=20, image=16, gen=oracle_mod.GEN)
        b = scene.workload(name, n=20, image=16)
        assert np.array_equal(a.volume, b.volume), name
        for ca, cb in zip(a.cones, b.cones):
            assert bytes(ca) == bytes(cb), name
        for ga, gb in zip(a.gt, b.gt):
            assert np.array_equal(ga, gb), name
