"""ctypes mirror of include/cvr.h and the loader of the in-tree libcvr.so.

The library is the product; this module only declares its C ABI for Python
callers (tests, the benchmark).  Loading fails loudly when the shared library
is missing: there is no Python or CPU fallback for any rendering path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libcvr.so"

CVR_OK = 0
CVR_ERR_INVALID_ARG = -1
CVR_ERR_NO_VOLUME = -2
CVR_ERR_NOT_READY = -3
CVR_ERR_CUDA = -4
CVR_ERR_OUT_OF_MEMORY = -5
CVR_ERR_IO = -6
CVR_ERR_FORMAT = -7
CVR_ERR_TIMEOUT = -8
CVR_ERR_UNSUPPORTED = -9

CVR_U8 = 1
CVR_U16 = 2

PLAIN, EXTINCTION, CONE_DOS, GROUND_TRUTH, SURROGATE, ISO = 0, 1, 2, 3, 4, 5
LIGHT_POINT, LIGHT_SPOT, LIGHT_DIRECTIONAL = 0, 1, 2

MAX_AO_SHELLS = 32
MLP_PARAMS = 7426
MLP_INPUTS = 48
SURROGATE_LEVELS = 6
SAMPLING_TEX_FEATURES = 1
SAMPLING_TEX_VOLUME = 2
SAMPLING_TEX_PYRAMID = 4
# cvr_set_gradient_kernel / cvr_get_gradient_kernel
GRADIENT_KERNEL_AUTO = 0
GRADIENT_KERNEL_TILED = 1
GRADIENT_KERNEL_GENERIC = 2
GRADIENT_KERNEL_TMA = 3
# cvr_set_volume_layout
LAYOUT_PLAIN = 0
LAYOUT_QUADS = 1
MLP_NOALLOC_MAX_POINTS = 8192
MAX_VOLUMES = 16
MAX_CONE_SECTIONS = 512
GRADIENT_SOBEL_FELDMAN, GRADIENT_FINITE_DIFFERENCES, GRADIENT_COMPUTE_SOBEL, GRADIENT_NONE = 0, 1, 2, 3
MULTISCALE_SINGLE, MULTISCALE_MULTISAMPLE, MULTISCALE_DOWNSCALE, MULTISCALE_UPSCALE = 0, 1, 2, 3
(FILTER_BOX, FILTER_HAT, FILTER_CATMULL_ROM, FILTER_MITCHELL_NETRAVALI, FILTER_CARDINAL_BSPLINE3,
 FILTER_CARDINAL_OMOMS3) = range(6)

F3 = C.c_float * 3


class Camera(C.Structure):
    _fields_ = [("eye", F3), ("center", F3), ("up", F3), ("fovy_deg", C.c_float), ("aspect", C.c_float)]


class Light(C.Structure):
    _fields_ = [("type", C.c_int), ("position", F3), ("forward", F3), ("up", F3), ("right", F3),
                ("spot_cos_max", C.c_float)]


class PlainParams(C.Structure):
    _fields_ = [("step_size", C.c_float)]


class ExtParams(C.Structure):
    _fields_ = [("step_size", C.c_float), ("apply_occlusion", C.c_int), ("apply_shadow", C.c_int),
                ("ao_n_shells", C.c_int), ("ao_radii", C.c_float * MAX_AO_SHELLS),
                ("sdw_cone_angle_rad", C.c_float), ("sdw_sample_interval", C.c_float),
                ("sdw_initial_step", C.c_float), ("sdw_ui_weight", C.c_float), ("sdw_max_distance", C.c_float),
                ("shadow_type", C.c_int), ("ka", C.c_float), ("kd", C.c_float)]


class DosParams(C.Structure):
    _fields_ = [("step_size", C.c_float), ("apply_occlusion", C.c_int), ("apply_shadow", C.c_int),
                ("shadow_type", C.c_int), ("ka", C.c_float), ("kd", C.c_float)]


class GtParams(C.Structure):
    _fields_ = [("step_size", C.c_float), ("light_ray_initial_gap", C.c_float), ("light_ray_step_size", C.c_float),
                ("apply_occlusion", C.c_int), ("occ_distance", C.c_float), ("apply_shadow", C.c_int),
                ("sdw_distance", C.c_float), ("shadow_type", C.c_int), ("ka", C.c_float), ("kd", C.c_float)]


class IsoParams(C.Structure):
    _fields_ = [("step_size_small", C.c_float), ("step_size_large", C.c_float), ("step_size_range", C.c_float),
                ("isovalue", C.c_float), ("color", C.c_float * 4)]


class ConeTable(C.Structure):
    _fields_ = [("n_sections", C.c_int), ("sections", (C.c_float * 4) * MAX_CONE_SECTIONS),
                ("integration_samples", C.c_int * 3), ("axes", F3 * 10), ("initial_step", C.c_float),
                ("ray7_adj_weight", C.c_float), ("ui_weight", C.c_float)]


class PyramidParams(C.Structure):
    _fields_ = [("base_dims", C.c_int * 3), ("sigma0", C.c_float), ("n_levels", C.c_int)]


class FrameStats(C.Structure):
    _fields_ = [("samples", C.c_uint64), ("shaded_samples", C.c_uint64), ("aux_fetches", C.c_uint64),
                ("kernel_ms", C.c_float)]


class GradientParams(C.Structure):
    _fields_ = [("model", C.c_int), ("sample_size", C.c_int), ("filter_nxnxn", C.c_int), ("normalized", C.c_int)]


class BlinnPhong(C.Structure):
    _fields_ = [("apply", C.c_int), ("ka", C.c_float), ("kd", C.c_float), ("ks", C.c_float),
                ("shininess", C.c_float), ("specular", F3)]


class Job(C.Structure):
    _fields_ = [("volume", C.c_int), ("method", C.c_int), ("params", C.c_void_p), ("params_size", C.c_size_t),
                ("camera", Camera), ("light", Light), ("width", C.c_int), ("height", C.c_int),
                ("out_rgba_dev", C.c_void_p)]


PARAMS_OF_METHOD = {PLAIN: PlainParams, EXTINCTION: ExtParams, CONE_DOS: DosParams, GROUND_TRUTH: GtParams,
                    SURROGATE: GtParams, ISO: IsoParams}

_P = C.c_void_p
_I = C.c_int
_F = C.c_float
_D = C.POINTER(C.c_double)
_FP = C.POINTER(C.c_float)

SIGNATURES = {
    "cvr_abi_version": (_I, []),
    "cvr_create": (_I, [C.POINTER(_P), _I]),
    "cvr_destroy": (None, [_P]),
    "cvr_last_error": (C.c_char_p, [_P]),
    "cvr_sync": (_I, [_P]),
    "cvr_stream": (_P, [_P]),
    "cvr_set_volume": (_I, [_P, _P, _I, _I, _I, _I, _F, _F, _F]),
    "cvr_set_volume_device": (_I, [_P, _P, _I, _I, _I, _I, _F, _F, _F]),
    "cvr_set_transfer_function": (_I, [_P, _FP, _FP, _I]),
    "cvr_build_sat": (_I, [_P, _D, _I]),
    "cvr_prepare_sat": (_I, [_P]),
    "cvr_get_sat_info": (_I, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "cvr_download_sat": (_I, [_P, C.POINTER(C.c_int64)]),
    "cvr_build_ext_pyramid": (_I, [_P, C.POINTER(PyramidParams)]),
    "cvr_get_pyramid_info": (_I, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), _I]),
    "cvr_download_pyramid_level": (_I, [_P, _I, _FP]),
    "cvr_set_cone_tables": (_I, [_P, C.POINTER(ConeTable), C.POINTER(ConeTable)]),
    "cvr_set_gt_kernels": (_I, [_P, _FP, _I, _FP, _I]),
    "cvr_render": (_I, [_P, _I, C.POINTER(Camera), C.POINTER(Light), _P, C.c_size_t, _P, _I, _I, _P,
                        C.POINTER(FrameStats)]),
    "cvr_render_host": (_I, [_P, _I, C.POINTER(Camera), C.POINTER(Light), _P, C.c_size_t, _FP, _I, _I,
                             C.POINTER(FrameStats)]),
    "cvr_set_tuning": (_I, [_P, _I, _I, _I]),
    "cvr_get_tuning": (_I, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "cvr_autotune": (_I, [_P, _I, C.POINTER(Camera), C.POINTER(Light), _P, C.c_size_t, _I, _I, _I,
                          C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), _FP]),
    "cvr_get_frame_buffer": (_I, [_P, _I, _I, C.POINTER(_FP)]),
    "cvr_download_frame": (_I, [_P, _P, _I, _I, _FP]),
    "cvr_timer_start": (_I, [_P]),
    "cvr_timer_stop": (_I, [_P, _FP]),
    "cvr_flush_l2": (_I, [_P]),
    "cvr_measure_l1_bandwidth": (_I, [_P, _FP]),
    "cvr_tf_build_linear": (_I, [_I, _I, _D, _I, _D, _I, _FP, _FP]),
    "cvr_tf_ext_per_value": (_I, [_I, _I, _D, _I, _D, _I, _I, _D]),
    "cvr_read_tf1d": (_I, [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), _D, _I,
                           C.POINTER(C.c_int), _D, _I]),
    "cvr_read_volume_info": (_I, [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), _FP]),
    "cvr_read_volume": (_I, [C.c_char_p, _P, C.c_size_t]),
    "cvr_cone_sampler_build": (_I, [_F, _I, _F, _F, _F, C.c_double, C.POINTER(ConeTable)]),
    "cvr_gt_kernel_vectors": (_I, [_I, _F, _I, _F, C.c_uint, _FP, _FP]),
    "cvr_host_alloc_pinned": (_I, [C.c_size_t, C.POINTER(_P)]),
    "cvr_host_free_pinned": (None, [_P]),
    "cvr_synth_blobs": (_I, [_P, _I, _I, _I, _I, _I, C.c_uint64, _F]),
    "cvr_mlp_init": (_I, [_P, C.c_uint64]),
    "cvr_mlp_set_params": (_I, [_P, _FP, _I]),
    "cvr_mlp_get_params": (_I, [_P, _FP, _I]),
    "cvr_mlp_forward": (_I, [_P, _FP, _I, _FP]),
    "cvr_mlp_gradients": (_I, [_P, _FP, _FP, _I, _FP, _FP]),
    "cvr_mlp_set_training_data": (_I, [_P, _FP, _FP, _I]),
    "cvr_mlp_get_training_data": (_I, [_P, _FP, _FP, _I]),
    "cvr_mlp_training_size": (_I, [_P]),
    "cvr_mlp_train": (_I, [_P, _I, _I, _F, C.c_uint64, _FP]),
    "cvr_mlp_gradients_noalloc": (_I, [_P, _P, _P, _I, _P, _P]),
    "cvr_mlp_check": (_I, [_P]),
    "cvr_select_volume": (_I, [_P, _I]),
    "cvr_current_volume": (_I, [_P]),
    "cvr_batch_create": (_I, [_P, C.POINTER(Job), _I, C.POINTER(_P)]),
    "cvr_batch_run": (_I, [_P]),
    "cvr_batch_job_stats": (_I, [_P, _I, C.POINTER(FrameStats)]),
    "cvr_batch_destroy": (None, [_P]),
    "cvr_set_light_cache": (_I, [_P, _I, _I, _I]),
    "cvr_download_light_cache": (_I, [_P, _FP, C.c_size_t]),
    "cvr_set_brick_size": (_I, [_P, _I]),
    "cvr_get_brick_size": (_I, [_P]),
    "cvr_set_gradient_kernel": (_I, [_P, _I]),
    "cvr_get_gradient_kernel": (_I, [_P]),
    "cvr_set_warp_shape": (_I, [_P, _I]),
    "cvr_get_warp_shape": (_I, [_P]),
    "cvr_set_ray_refill": (_I, [_P, _I]),
    "cvr_get_ray_refill": (_I, [_P]),
    "cvr_set_brick_staging": (_I, [_P, _I]),
    "cvr_get_brick_staging": (_I, [_P]),
    "cvr_set_walk_tables": (_I, [_P, _I]),
    "cvr_get_walk_tables": (_I, [_P]),
    "cvr_set_volume_layout": (_I, [_P, _I]),
    "cvr_get_volume_layout": (_I, [_P]),
    "cvr_set_compact_sat": (_I, [_P, _I]),
    "cvr_get_compact_sat": (_I, [_P]),
    "cvr_set_multiscaling": (_I, [_P, _I, _I, _I, _I]),
    "cvr_get_multiscaling": (_I, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int)]),
    "cvr_rescale_frame": (_I, [_P, _I, _I, _P, _I, _I, _P, _I, _I]),
    "cvr_build_gradient": (_I, [_P, C.POINTER(GradientParams)]),
    "cvr_download_gradient": (_I, [_P, _FP, C.c_size_t]),
    "cvr_set_blinn_phong": (_I, [_P, C.POINTER(BlinnPhong)]),
    "cvr_get_blinn_phong": (_I, [_P, C.POINTER(BlinnPhong)]),
    "cvr_set_sampling": (_I, [_P, _I]),
    "cvr_get_sampling": (_I, [_P]),
    "cvr_mlp_save": (_I, [_P, C.c_char_p]),
    "cvr_mlp_load": (_I, [_P, C.c_char_p]),
    "cvr_surrogate_collect": (_I, [_P, C.POINTER(Camera), _I, _I, _F, _F, C.c_uint64, _I, C.POINTER(C.c_int)]),
    "cvr_surrogate_clear_points": (_I, [_P]),
    "cvr_surrogate_point_count": (_I, [_P]),
    "cvr_surrogate_set_points": (_I, [_P, _FP, _I]),
    "cvr_surrogate_get_points": (_I, [_P, _FP, _I]),
    "cvr_surrogate_label": (_I, [_P, C.POINTER(Light), C.POINTER(GtParams), _I, _FP, _FP, _I]),
    "cvr_surrogate_evaluate": (_I, [_P, C.POINTER(Light), C.POINTER(GtParams), C.POINTER(DosParams), _D]),
    "cvr_synth_value_noise": (_I, [_P, _I, _I, _I, _I, _I, _F, _F, _I, C.c_uint64]),
}

_lib = None


class CvrError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"cvr error {code}: {msg}")
        self.code = code


def load(path: Path | str | None = None) -> C.CDLL:
    """Loads libcvr.so and declares every exported signature; raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(code: int, ctx=None) -> None:
    if code != CVR_OK:
        lib = load()
        msg = lib.cvr_last_error(ctx)
        raise CvrError(code, msg.decode() if msg else "")


def fptr(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_FP)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def vptr(a: np.ndarray):
    assert a.flags.c_contiguous
    return C.c_void_p(a.ctypes.data)


def exported_symbols(header: Path | None = None) -> list[str]:
    """Names of every function declared in include/cvr.h."""
    import re
    h = header or (PKG.parent / "include" / "cvr.h")
    text = h.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cvr_[a-z0-9_]+)\s*\(", text)))
