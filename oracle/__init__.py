"""TEST INFRASTRUCTURE ONLY — Python binding of the CPU oracle (liboracle.so)
and of the reference's own table builders (oracle/_ref/libcvr_ref.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs may use this package; the product (libcvr.so and its package) never
imports it.  The oracle never loads libcvr.so: it builds its transfer-function,
cone and kernel-vector tables and the synthetic volumes with its own code
(oracle_tables.cpp, exposed as GEN), and takes only the parameter structs'
ctypes layouts from the product's header mirror (abi, which loads nothing
until abi.load() is called).  Parity status: the table builders are pinned
against the reference's own C++ (see build_ref.py) and committed golden
vectors; the marching loops are restatements of GLSL that cannot run on these
machines.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from cpp_volume_rendering_gb300 import abi

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libcvr_ref.so"

_lib = None
_ref = None


def build_lib():
    """Compiles liboracle.so (oracle/build.py) when it is missing or stale."""
    import importlib
    return importlib.import_module("oracle.build").build()


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build_lib()
        lib = C.CDLL(str(LIB))
        P, I, D = C.c_void_p, C.c_int, C.c_double
        sig = {
            "oracle_create": (P, []),
            "oracle_destroy": (None, [P]),
            "oracle_set_volume": (I, [P, P, I, I, I, I, D, D, D]),
            "oracle_set_tf": (I, [P, P, P, I]),
            "oracle_build_sat": (I, [P, P, I]),
            "oracle_get_sat": (I, [P, P]),
            "oracle_sat_i64": (I, [P, I, I, I, I, P, P]),
            "oracle_build_pyramid": (I, [P, C.POINTER(abi.PyramidParams)]),
            "oracle_get_pyramid_level": (I, [P, I, I, P]),
            "oracle_set_cone_tables": (I, [P, C.POINTER(abi.ConeTable), C.POINTER(abi.ConeTable)]),
            "oracle_set_gt_kernels": (I, [P, P, I, P, I]),
            "oracle_render": (I, [P, I, I, C.POINTER(abi.Camera), C.POINTER(abi.Light), P, I, I, I, I, P, P,
                                  C.POINTER(C.c_uint64), I]),
            "oracle_set_mlp": (I, [P, P, I]),
            "oracle_set_light_cache": (I, [P, I, I, I]),
            "oracle_build_gradient": (I, [P, C.POINTER(abi.GradientParams)]),
            "oracle_get_gradient": (I, [P, P]),
            "oracle_set_blinn_phong": (I, [P, C.POINTER(abi.BlinnPhong)]),
            "oracle_sur_features": (I, [P, I, C.POINTER(abi.Light), I, D, P, I, P, P]),
            "oracle_gt_points": (I, [P, C.POINTER(abi.Light), C.POINTER(abi.GtParams), P, I, P]),
            "oracle_tf_tables": (I, [I, I, P, I, P, I, P, P]),
            "oracle_tf_ext_per_value": (I, [I, I, P, I, P, I, I, P]),
            "oracle_cone_table": (I, [C.c_float, I, C.c_float, C.c_float, C.c_float, D, C.POINTER(abi.ConeTable)]),
            "oracle_gt_vectors": (I, [I, C.c_float, I, C.c_float, C.c_uint, P, P]),
            "oracle_synth_blobs": (I, [P, I, I, I, I, I, C.c_uint64, C.c_float]),
            "oracle_synth_value_noise": (I, [P, I, I, I, I, I, C.c_float, C.c_float, I, C.c_uint64]),
        }
        for k, (r, a) in sig.items():
            f = getattr(lib, k)
            f.restype, f.argtypes = r, a
        _lib = lib
    return _lib


def ref_available() -> bool:
    if REF_LIB.exists():
        return True
    try:
        import importlib
        return importlib.import_module("oracle.build_ref").build() is not None
    except Exception:
        return False


def load_ref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise FileNotFoundError("reference pieces are not built (needs the reference checkout)")
        _ref = C.CDLL(str(REF_LIB))
    return _ref


def _p(a):
    return C.c_void_p(a.ctypes.data)


class Oracle:
    """CPU renderer: FP64 (precision=64) is the parity oracle, FP32 the baseline."""

    def __init__(self):
        self.lib = load()
        self.h = C.c_void_p(self.lib.oracle_create())

    def __del__(self):
        try:
            self.lib.oracle_destroy(self.h)
        except Exception:
            pass

    def _ck(self, r):
        if r < 0:
            raise RuntimeError(f"oracle error {r}")
        return r

    def set_volume(self, vol, spacing):
        vol = np.ascontiguousarray(vol)
        d, h, w = vol.shape
        dt = abi.CVR_U8 if vol.dtype == np.uint8 else abi.CVR_U16
        self._ck(self.lib.oracle_set_volume(self.h, _p(vol), w, h, d, dt, *[float(s) for s in spacing]))
        self.vol = vol

    def set_tf(self, rgbt, rgba):
        rgbt = np.ascontiguousarray(rgbt, np.float32)
        rgba = np.ascontiguousarray(rgba, np.float32)
        self._ck(self.lib.oracle_set_tf(self.h, _p(rgbt), _p(rgba), len(rgbt)))

    def build_sat(self, ext):
        ext = np.ascontiguousarray(ext, np.float64)
        self._ck(self.lib.oracle_build_sat(self.h, _p(ext), len(ext)))

    def sat(self):
        d, h, w = self.vol.shape
        out = np.zeros((d + 2, h + 2, w + 2), np.float64)
        self._ck(self.lib.oracle_get_sat(self.h, _p(out)))
        return out

    def build_pyramid(self, base_dims, sigma0, n_levels):
        p = abi.PyramidParams()
        p.base_dims[:] = list(base_dims)
        p.sigma0 = sigma0
        p.n_levels = n_levels
        self.n_levels = self._ck(self.lib.oracle_build_pyramid(self.h, C.byref(p)))
        self.base_dims = tuple(base_dims)
        return self.n_levels

    def pyramid_level(self, level, precision=64):
        w, h, d = [max(1, b >> level) for b in self.base_dims]
        out = np.zeros((d, h, w), np.float64)
        self._ck(self.lib.oracle_get_pyramid_level(self.h, precision, level, _p(out)))
        return out

    def set_cone_tables(self, occ, sdw):
        self._ck(self.lib.oracle_set_cone_tables(self.h, C.byref(occ), C.byref(sdw)))

    def set_gt_kernels(self, occ, sdw):
        occ = np.ascontiguousarray(occ, np.float32)
        sdw = np.ascontiguousarray(sdw, np.float32)
        self._ck(self.lib.oracle_set_gt_kernels(self.h, _p(occ), len(occ), _p(sdw), len(sdw)))

    def set_light_cache(self, w, h, d):
        self._ck(self.lib.oracle_set_light_cache(self.h, w, h, d))

    def build_gradient(self, model=abi.GRADIENT_FINITE_DIFFERENCES, sample_size=1, filter_nxnxn=0, normalized=True):
        p = abi.GradientParams(model, sample_size, filter_nxnxn, int(normalized))
        self._ck(self.lib.oracle_build_gradient(self.h, C.byref(p)))

    def gradient(self):
        d, h, w = self.vol.shape
        out = np.zeros((d, h, w, 3), np.float32)
        self._ck(self.lib.oracle_get_gradient(self.h, _p(out)))
        return out

    def set_blinn_phong(self, apply=True, ka=0.5, kd=0.5, ks=0.8, shininess=30.0, specular=(1.0, 1.0, 1.0)):
        bp = abi.BlinnPhong(int(apply), ka, kd, ks, shininess, abi.F3(*specular))
        self._ck(self.lib.oracle_set_blinn_phong(self.h, C.byref(bp)))

    def set_mlp(self, params):
        params = np.ascontiguousarray(params, np.float32)
        self._ck(self.lib.oracle_set_mlp(self.h, _p(params), len(params)))

    def sur_features(self, lt, gt_params, pts, precision=64, with_outputs=False):
        """Surrogate inputs (n x 48) of points (n x 6) and, optionally, the
        BF16 network's outputs (n x 2) on them."""
        pts = np.ascontiguousarray(pts, np.float32)
        n = len(pts)
        x = np.zeros((n, 48), np.float64)
        y = np.zeros((n, 2), np.float64) if with_outputs else None
        self._ck(self.lib.oracle_sur_features(self.h, precision, C.byref(lt), gt_params.shadow_type,
                                              float(gt_params.sdw_distance), _p(pts), n, _p(x),
                                              _p(y) if y is not None else None))
        return (x, y) if with_outputs else x

    def gt_points(self, lt, params, pts):
        """Ground-truth (occlusion, shadow) of points (n x 6), FP64."""
        pts = np.ascontiguousarray(pts, np.float32)
        out = np.zeros((len(pts), 2), np.float64)
        self._ck(self.lib.oracle_gt_points(self.h, C.byref(lt), C.byref(params), _p(pts), len(pts), _p(out)))
        return out

    def render(self, method, cam, lt, params, w, h, precision=64, rows=None, threads=0):
        """Returns (image rows [y0,y1) x W x 4 float64, per-pixel step counts, total steps)."""
        import os
        y0, y1 = rows if rows else (0, h)
        out = np.zeros((y1 - y0, w, 4), np.float64)
        counts = np.zeros((y1 - y0, w), np.uint32)
        total = C.c_uint64()
        threads = threads or os.cpu_count() or 1
        self._ck(self.lib.oracle_render(self.h, precision, method, C.byref(cam), C.byref(lt) if lt else None,
                                        C.c_void_p(C.addressof(params)), w, h, y0, y1, _p(out), _p(counts),
                                        C.byref(total), threads))
        return out, counts, total.value


def sat_i64(vol, q):
    vol = np.ascontiguousarray(vol)
    d, h, w = vol.shape
    dt = abi.CVR_U8 if vol.dtype == np.uint8 else abi.CVR_U16
    q = np.ascontiguousarray(q, np.int64)
    out = np.zeros((d + 2, h + 2, w + 2), np.int64)
    load().oracle_sat_i64(_p(vol), w, h, d, dt, _p(q), _p(out))
    return out


def _ck(code, what):
    if code != 0:
        raise RuntimeError(f"oracle {what}: error {code}")


class Gen:
    """The oracle's volume generators and table builders (oracle_tables.cpp):
    the same interface as the library's scene.LIB_GEN, so scene.workload(...,
    gen=GEN) builds a workload without loading libcvr.so."""

    @staticmethod
    def _vol(w, h, d, dtype):
        return np.empty((d, h, w), np.uint8 if dtype == abi.CVR_U8 else np.uint16)

    def synth_blobs(self, w, h, d, dtype, n_blobs, seed, noise_max=0.0):
        out = self._vol(w, h, d, dtype)
        _ck(load().oracle_synth_blobs(_p(out), w, h, d, dtype, n_blobs, seed, noise_max), "synth_blobs")
        return out

    def synth_value_noise(self, w, h, d, dtype, seed, octaves=4, lacunarity=2.0, gain=0.5, shells=4):
        out = self._vol(w, h, d, dtype)
        _ck(load().oracle_synth_value_noise(_p(out), w, h, d, dtype, octaves, lacunarity, gain, shells, seed),
            "synth_value_noise")
        return out

    def cone_table(self, half_angle, packing, covered, initial_step, ui_weight, min_sigma):
        t = abi.ConeTable()
        _ck(load().oracle_cone_table(half_angle, packing, covered, initial_step, ui_weight, min_sigma, C.byref(t)),
            "cone_table")
        return t

    def gt_vectors(self, n_occ, occ_aperture, n_sdw, sdw_aperture, seed=1):
        occ = np.zeros((max(n_occ, 1), 3), np.float32)
        sdw = np.zeros((max(n_sdw, 1), 3), np.float32)
        _ck(load().oracle_gt_vectors(n_occ, occ_aperture, n_sdw, sdw_aperture, seed, _p(occ), _p(sdw)), "gt_vectors")
        return occ[:n_occ].copy(), sdw[:n_sdw].copy()

    @staticmethod
    def _points(tf):
        rgb = np.ascontiguousarray(np.array(tf.rgb, dtype=np.float64).reshape(-1, 4))
        al = np.ascontiguousarray(np.array(tf.alpha, dtype=np.float64).reshape(-1, 2))
        return rgb, al

    def tf_tables(self, tf):
        """(rgbt, rgba) tables of a scene.TransferFunction, (max_density+1) x 4 float32."""
        rgb, al = self._points(tf)
        n = tf.max_density + 1
        rgbt = np.zeros((n, 4), np.float32)
        rgba = np.zeros((n, 4), np.float32)
        _ck(load().oracle_tf_tables(tf.max_density, len(rgb), _p(rgb), len(al), _p(al), int(tf.extinction_input),
                                    _p(rgbt), _p(rgba)), "tf_tables")
        return rgbt, rgba

    def tf_ext_per_value(self, tf, dtype):
        rgb, al = self._points(tf)
        out = np.zeros(256 if dtype == abi.CVR_U8 else 65536, np.float64)
        _ck(load().oracle_tf_ext_per_value(tf.max_density, len(rgb), _p(rgb), len(al), _p(al),
                                           int(tf.extinction_input), dtype, _p(out)), "tf_ext_per_value")
        return out


GEN = Gen()


def prepare(orc: Oracle, wl):
    """Oracle-side Init() for a scene.Workload: every table from the oracle's
    own builders (the workload's transfer-function points and table specs)."""
    rgbt, rgba = GEN.tf_tables(wl.tf)
    orc.set_volume(wl.volume, wl.spacing)
    orc.set_tf(rgbt, rgba)
    cones = tuple(GEN.cone_table(*c) for c in wl.cone_spec) if wl.cone_spec else ()
    gt = GEN.gt_vectors(*wl.gt_spec) if wl.gt_spec else ()
    if wl.method == abi.EXTINCTION:
        orc.build_sat(GEN.tf_ext_per_value(wl.tf, wl.dtype))
    if wl.method == abi.CONE_DOS:
        orc.build_pyramid(wl.pyramid["base_dims"], wl.pyramid["sigma0"], wl.pyramid["n_levels"])
        orc.set_cone_tables(*cones)
    if wl.method == abi.GROUND_TRUTH:
        orc.set_gt_kernels(*gt)
    if wl.method == abi.SURROGATE:
        orc.build_pyramid(wl.pyramid["base_dims"], wl.pyramid["sigma0"], wl.pyramid["n_levels"])
        orc.set_gt_kernels(*gt)
        orc.set_cone_tables(*cones)
