"""The C ABI library: loads, exports every declared symbol, host entry points
validate their arguments, file readers report errors instead of exiting.
CPU only: no compute call touches a GPU here."""
import ctypes as C
import subprocess
import sys

import numpy as np
import pytest

from cpp_volume_rendering_gb300 import abi, scene


def test_exports_every_declared_symbol(lib):
    names = abi.exported_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and ctypes declares a signature for each of them
    assert not [n for n in names if n not in abi.SIGNATURES], [n for n in names if n not in abi.SIGNATURES]


def test_symbols_visible_to_nm(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(abi.LIB_PATH)], capture_output=True, text=True).stdout
    for n in abi.exported_symbols():
        assert f" T {n}" in out, n


def test_abi_version(lib):
    assert lib.cvr_abi_version() == 1


def test_null_and_bad_arguments_are_errors(lib):
    assert lib.cvr_create(None, 0) == abi.CVR_ERR_INVALID_ARG
    assert lib.cvr_sync(None) == abi.CVR_ERR_INVALID_ARG
    assert lib.cvr_set_volume(None, None, 1, 1, 1, 1, 1.0, 1.0, 1.0) == abi.CVR_ERR_INVALID_ARG
    assert lib.cvr_prepare_sat(None) == abi.CVR_ERR_INVALID_ARG
    assert lib.cvr_build_sat(None, None, 256) == abi.CVR_ERR_INVALID_ARG
    assert lib.cvr_batch_create(None, None, 0, None) == abi.CVR_ERR_INVALID_ARG
    lib.cvr_destroy(None)  # no-op
    rgb = np.zeros((1, 4))
    assert lib.cvr_tf_build_linear(0, 0, abi.dptr(rgb), 0, abi.dptr(rgb), 0, None, None) == abi.CVR_ERR_INVALID_ARG
    t = abi.ConeTable()
    assert lib.cvr_cone_sampler_build(20.0, 5, 100.0, 3.0, 1.0, 1.0, C.byref(t)) == abi.CVR_ERR_INVALID_ARG
    assert lib.cvr_cone_sampler_build(20.0, 1, 100.0, 3.0, 1.0, 0.0, C.byref(t)) == abi.CVR_ERR_INVALID_ARG


def test_raw_reader_name_convention_and_errors(lib, tmp_path):
    vol = (np.arange(3 * 4 * 5) % 251).astype(np.uint8).reshape(5, 4, 3)
    p = tmp_path / "blob.1.3x4x5.raw"
    vol.tofile(p)
    dims = (C.c_int * 3)()
    dt = C.c_int()
    sp = (C.c_float * 3)()
    assert lib.cvr_read_volume_info(str(p).encode(), dims, C.byref(dt), sp) == 0
    assert list(dims) == [3, 4, 5] and dt.value == abi.CVR_U8 and list(sp) == [1.0, 1.0, 1.0]
    out = np.zeros(60, np.uint8)
    assert lib.cvr_read_volume(str(p).encode(), abi.vptr(out), 60) == 0
    assert np.array_equal(out, vol.ravel())
    # 16-bit
    v16 = (np.arange(2 * 2 * 2) * 1000).astype(np.uint16)
    p16 = tmp_path / "w.2.2x2x2.raw"
    v16.tofile(p16)
    assert lib.cvr_read_volume_info(str(p16).encode(), dims, C.byref(dt), sp) == 0 and dt.value == abi.CVR_U16
    o16 = np.zeros(8, np.uint16)
    assert lib.cvr_read_volume(str(p16).encode(), abi.vptr(o16), 16) == 0 and np.array_equal(o16, v16)
    # short file -> IO error (the reference exits here, rawloader.cpp:29-35)
    short = tmp_path / "s.1.4x4x4.raw"
    short.write_bytes(b"\0" * 10)
    assert lib.cvr_read_volume(str(short).encode(), abi.vptr(np.zeros(64, np.uint8)), 64) == abi.CVR_ERR_IO
    # missing file / bad name
    assert lib.cvr_read_volume_info(str(tmp_path / "nope.1.2x2x2.raw").encode(), dims, C.byref(dt), sp) == abi.CVR_ERR_IO
    bad = tmp_path / "bad.raw"
    bad.write_bytes(b"\0")
    assert lib.cvr_read_volume_info(str(bad).encode(), dims, C.byref(dt), sp) == abi.CVR_ERR_FORMAT
    # output buffer too small
    assert lib.cvr_read_volume(str(p).encode(), abi.vptr(out), 10) == abi.CVR_ERR_INVALID_ARG


def test_syn_reader(lib, tmp_path):
    p = tmp_path / "box.syn"
    p.write_text("4 3 2\n1 0 0 0 2 3 1 200\n0 3 2 1 77\n")
    dims = (C.c_int * 3)()
    dt = C.c_int()
    assert lib.cvr_read_volume_info(str(p).encode(), dims, C.byref(dt), None) == 0
    assert list(dims) == [4, 3, 2] and dt.value == abi.CVR_U8
    out = np.zeros(24, np.uint8)
    assert lib.cvr_read_volume(str(p).encode(), abi.vptr(out), 24) == 0
    v = out.reshape(2, 3, 4)
    assert (v[0, :, :2] == 200).all() and v[1, 2, 3] == 77 and v[0, 0, 3] == 0
    trunc = tmp_path / "t.syn"
    trunc.write_text("2 2 2\n1 0 0\n")
    assert lib.cvr_read_volume(str(trunc).encode(), abi.vptr(np.zeros(8, np.uint8)), 8) == abi.CVR_ERR_FORMAT


def test_tf1d_reader_roundtrip(lib, tmp_path):
    p = tmp_path / "ramp.tf1d"
    p.write_text("linear\n0\n3\n0.0 0.5 1.0 0\n0.5 0.5 0.5 100\n1.0 0.0 0.0 255\n3\n0.0 0\n0.3 100\n0.8 255\n")
    tf = scene.TransferFunction.read_tf1d(str(p))
    assert tf.max_density == 255 and not tf.extinction_input
    assert len(tf.rgb) == 3 and tf.rgb[1] == (0.5, 0.5, 0.5, 100.0)
    assert tf.alpha[2] == (0.8, 255.0)
    p2 = tmp_path / "ext.tf1d"
    p2.write_text("linear\n2\n511 1\n2\n1 1 1 0\n1 1 1 511\n2\n0 0\n4.0 511\n")
    tf2 = scene.TransferFunction.read_tf1d(str(p2))
    assert tf2.max_density == 511 and tf2.extinction_input
    rgbt, rgba = tf2.tables()
    assert rgbt.shape == (512, 4) and rgbt[511, 3] == np.float32(4.0)
    bad = tmp_path / "bad.tf1d"
    bad.write_text("linear\n0\n2\n0 0 0\n")
    with pytest.raises(abi.CvrError):
        scene.TransferFunction.read_tf1d(str(bad))
    with pytest.raises(abi.CvrError):
        scene.TransferFunction.read_tf1d(str(tmp_path / "missing.tf1d"))


def _reference_fixture(rel):
    from oracle.build_ref import reference_root
    root = reference_root()
    p = root / rel if root is not None else None
    return p if p is not None and p.exists() else None


@pytest.mark.skipif(_reference_fixture("data/tf1dcp/bonsai_01.tf1d") is None,
                    reason="reference data fixtures not present")
def test_tf1d_reader_reads_reference_fixture(lib):
    tf = scene.TransferFunction.read_tf1d(str(_reference_fixture("data/tf1dcp/bonsai_01.tf1d")))
    assert len(tf.rgb) == 5 and len(tf.alpha) == 4 and tf.max_density == 255
    rgbt, rgba = tf.tables()
    assert rgbt.shape == (256, 4)


def test_create_without_gpu_reports_cuda_error(lib):
    """On a machine without a GPU, context creation fails with an error code
    (never a crash or a silent CPU fallback)."""
    code = subprocess.run([sys.executable, "-c", (
        "import ctypes as C\n"
        "from cpp_volume_rendering_gb300 import abi\n"
        "lib=abi.load(); h=C.c_void_p()\n"
        "r=lib.cvr_create(C.byref(h),0)\n"
        "print(r, lib.cvr_last_error(None).decode())\n"
        "if r==0: lib.cvr_destroy(h)\n")], capture_output=True, text=True, cwd=str(abi.PKG.parent))
    r = int(code.stdout.split()[0])
    assert r in (abi.CVR_OK, abi.CVR_ERR_CUDA)
    if r == abi.CVR_ERR_CUDA:
        assert "CUDA" in code.stdout or "device" in code.stdout


def test_mlp_parameter_count_matches_layout():
    from oracle import mlp_ref
    assert abi.MLP_PARAMS == mlp_ref.N_PARAMS == 64 * 48 + 64 + 64 * 64 + 64 + 2 * 64 + 2
    import re
    h = (abi.PKG.parent / "include" / "cvr.h").read_text()
    assert int(re.search(r"#define CVR_MLP_PARAMS (\d+)", h).group(1)) == abi.MLP_PARAMS
