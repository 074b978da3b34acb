"""Volume file readers (CPU): .pvm (plain and DDS-compressed) pinned to the
reference's own loader through committed fixtures and, where the reference
checkout is present, on freshly encoded volumes; .nrrd / .nhrd and .dat
against their restated header rules (the reference's reader.cpp does not
compile with GCC, see the design notes); error codes."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import oracle
from cpp_volume_rendering_gb300 import abi
from tests import pvmfmt
from tests.golden.make_pvm_golden import CASES

GOLDEN = Path(__file__).resolve().parent / "golden"


def read(lib, path):
    dims = (C.c_int * 3)()
    dt = C.c_int()
    sp = (C.c_float * 3)()
    r = lib.cvr_read_volume_info(str(path).encode(), dims, C.byref(dt), sp)
    if r != 0:
        return r, None
    w, h, d = dims
    n = w * h * d * (2 if dt.value == abi.CVR_U16 else 1)
    out = np.zeros(n, np.uint8)
    r = lib.cvr_read_volume(str(path).encode(), abi.vptr(out), n)
    return r, ((w, h, d), dt.value, tuple(sp), out)


@pytest.mark.parametrize("name", list(CASES))
def test_pvm_matches_reference_loader(lib, name):
    g = np.load(GOLDEN / "pvm_reference.npz")
    r, got = read(lib, GOLDEN / "pvm" / f"{name}.pvm")
    assert r == 0
    dims, dtype, spacing, voxels = got
    assert dims == tuple(g[f"{name}_dims"])
    assert dtype == (abi.CVR_U16 if g[f"{name}_components"][0] == 2 else abi.CVR_U8)
    assert np.allclose(spacing, g[f"{name}_scale"], rtol=0, atol=0)
    assert np.array_equal(voxels, g[f"{name}_voxels"])


def test_pvm_fresh_encodings_against_live_reference(lib, tmp_path):
    if not oracle.ref_available():
        pytest.skip("reference sources not available")
    ref = oracle.load_ref()
    rng = np.random.default_rng(77)
    for k in range(8):
        d, h, w = rng.integers(1, 12, size=3)
        u16 = bool(k & 1)
        vol = rng.integers(0, 65536 if u16 else 256, size=(d, h, w)).astype(np.uint16 if u16 else np.uint8)
        if k & 2:  # smooth data: small residuals, short codes
            vol = (np.cumsum(vol.astype(np.int64) % 5, axis=-1) % (65536 if u16 else 256)).astype(vol.dtype)
        skip = int(rng.integers(1, 5))
        strip = int(rng.integers(1, max(2, vol.nbytes)))
        body = pvmfmt.pvm_bytes(vol, version=int(rng.integers(1, 4)), scale=(0.5, 1.0, 2.0))
        p = tmp_path / f"v{k}.pvm"
        p.write_bytes(pvmfmt.dds_file(body, skip, strip, bool(k & 4)))
        dims = (C.c_int * 3)()
        comps = C.c_int()
        sc = (C.c_double * 3)()
        n = vol.nbytes
        want = np.zeros(n, np.uint8)
        assert ref.ref_read_pvm(str(p).encode(), dims, C.byref(comps), sc, C.c_void_p(want.ctypes.data),
                                C.c_size_t(n)) == 0
        r, got = read(lib, p)
        assert r == 0 and np.array_equal(got[3], want), (k, skip, strip)
        assert got[0] == tuple(dims)


def test_pvm_errors(lib, tmp_path):
    vol = np.arange(60, dtype=np.uint8).reshape(3, 4, 5)
    body = pvmfmt.pvm_bytes(vol, version=2)
    short = tmp_path / "short.pvm"
    short.write_bytes(body[:-7])
    assert read(lib, short)[0] == abi.CVR_ERR_IO
    rgb = tmp_path / "rgb.pvm"
    rgb.write_bytes(b"PVM\n2 2 2\n3\n" + bytes(24))
    assert read(lib, rgb)[0] == abi.CVR_ERR_FORMAT
    junk = tmp_path / "junk.pvm"
    junk.write_bytes(b"P6\n1 1\n255\n\0\0\0")
    assert read(lib, junk)[0] == abi.CVR_ERR_FORMAT
    assert read(lib, tmp_path / "missing.pvm")[0] == abi.CVR_ERR_IO
    truncated = tmp_path / "cut.pvm"
    truncated.write_bytes(pvmfmt.dds_file(body, 1, 1)[:20])  # stream ends early: zeros, then the end marker
    assert read(lib, truncated)[0] in (abi.CVR_ERR_IO, abi.CVR_ERR_FORMAT)


def test_nrrd_detached_header(lib, tmp_path):
    rng = np.random.default_rng(5)
    vol = rng.integers(0, 65536, size=(4, 5, 6)).astype(np.uint16)
    (tmp_path / "data.raw").write_bytes(vol.tobytes())
    # the reference matches keys by prefix in order, so 'space directions' is taken
    # by 'space' and the spacing stays 1 (reader.cpp:413-447)
    (tmp_path / "vol.nrrd").write_text(
        "NRRD0004\n# a comment\ntype: uint16\ndimension: 3\nspace: left-posterior-superior\n"
        "sizes: 6 5 4\nspace directions: (2,0,0) (0,2,0) (0,0,2)\nkinds: domain domain domain\n"
        "endian: little\nencoding: raw\ndata file: data.raw\n")
    r, got = read(lib, tmp_path / "vol.nrrd")
    assert r == 0
    assert got[0] == (6, 5, 4) and got[1] == abi.CVR_U16 and got[2] == (1.0, 1.0, 1.0)
    assert np.array_equal(got[3].view(np.uint16), vol.ravel())
    (tmp_path / "b.nhrd").write_text("NRRD0001\r\ntype: uint8\r\nsizes: 3 2 1\r\ndata file: b.raw\r\n")
    (tmp_path / "b.raw").write_bytes(bytes(range(6)))
    r, got = read(lib, tmp_path / "b.nhrd")
    assert r == 0 and got[0] == (3, 2, 1) and got[1] == abi.CVR_U8 and list(got[3]) == list(range(6))
    (tmp_path / "nofile.nrrd").write_text("NRRD0004\ntype: uint8\nsizes: 2 2 2\n")
    assert read(lib, tmp_path / "nofile.nrrd")[0] == abi.CVR_ERR_FORMAT
    (tmp_path / "gone.nrrd").write_text("NRRD0004\ntype: uint8\nsizes: 2 2 2\ndata file: gone.raw\n")
    assert read(lib, tmp_path / "gone.nrrd")[0] == abi.CVR_ERR_IO


def test_dat_header(lib, tmp_path):
    vol = np.arange(2 * 3 * 4, dtype=np.uint16).reshape(2, 3, 4) * 1000
    (tmp_path / "obj.raw").write_bytes(vol.tobytes())
    (tmp_path / "v.dat").write_text("ObjectFileName: obj.raw\nTaggedFileName: ---\nResolution:  4 3 2\n"
                                    "SliceThickness: 0.5 0.5 1.25\nFormat:\t\tUSHORT\nNbrTags: 0\n"
                                    "ObjectType: TEXTURE_VOLUME_OBJECT\n")
    r, got = read(lib, tmp_path / "v.dat")
    assert r == 0
    assert got[0] == (4, 3, 2) and got[1] == abi.CVR_U16 and got[2] == (0.5, 0.5, 1.25)
    assert np.array_equal(got[3].view(np.uint16), vol.ravel())
    (tmp_path / "short.raw").write_bytes(bytes(5))
    (tmp_path / "s.dat").write_text("ObjectFileName: short.raw\nResolution: 2 2 2\nFormat: UCHAR\n")
    assert read(lib, tmp_path / "s.dat")[0] == abi.CVR_ERR_IO
    (tmp_path / "n.dat").write_text("ObjectFileName: short.raw\nFormat: UCHAR\n")
    assert read(lib, tmp_path / "n.dat")[0] == abi.CVR_ERR_FORMAT
