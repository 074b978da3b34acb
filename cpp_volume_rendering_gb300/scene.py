"""Scenes for tests and the benchmark, built through the C ABI of libcvr.so.

* TransferFunction: control points -> the RGBt / RGBA tables and the per-voxel
  extinction (host code of the library, restating TransferFunction1D).
* Context: a cvr_ctx (device state of one renderer: volume, tables, frames).
* workload(): the seeded synthetic workloads (volume, transfer function,
  camera, light, method parameters, and the specifications of the cone and
  kernel-vector tables).  The volume generator and the table builders come
  from a `gen` object: by default this library's (LIB_GEN); any object with
  the same five methods can stand in, so a caller that must not load the
  library (a CPU reference) builds the same workload from its own code.

World units follow the reference: a volume of dims N and spacing s spans
[-N*s/2, N*s/2].  The plain-casting workload uses the unit cube (s = 1/64);
the illumination workloads use 1 world unit per voxel, the spacing the
reference's .raw / .syn readers set, because their cone, SAT and pyramid
parameters are expressed in those units.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .abi import check

# ---------------------------------------------------------------- TF


@dataclass
class TransferFunction:
    rgb: list  # (r, g, b, iso)
    alpha: list  # (a, iso)
    max_density: int = 255
    extinction_input: bool = False

    def _pts(self):
        rgb = np.ascontiguousarray(np.array(self.rgb, dtype=np.float64).reshape(-1, 4))
        al = np.ascontiguousarray(np.array(self.alpha, dtype=np.float64).reshape(-1, 2))
        return rgb, al

    def tables(self) -> tuple[np.ndarray, np.ndarray]:
        """(rgbt, rgba) tables, (max_density+1) x 4 float32."""
        rgb, al = self._pts()
        n = self.max_density + 1
        rgbt = np.zeros((n, 4), np.float32)
        rgba = np.zeros((n, 4), np.float32)
        check(abi.load().cvr_tf_build_linear(self.max_density, len(rgb), abi.dptr(rgb), len(al), abi.dptr(al),
                                             int(self.extinction_input), abi.fptr(rgbt), abi.fptr(rgba)))
        return rgbt, rgba

    def ext_per_value(self, dtype: int) -> np.ndarray:
        rgb, al = self._pts()
        out = np.zeros(256 if dtype == abi.CVR_U8 else 65536, np.float64)
        check(abi.load().cvr_tf_ext_per_value(self.max_density, len(rgb), abi.dptr(rgb), len(al), abi.dptr(al),
                                              int(self.extinction_input), dtype, abi.dptr(out)))
        return out

    @staticmethod
    def read_tf1d(path: str) -> "TransferFunction":
        md, ext, nr, na = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        rgb = np.zeros((4096, 4), np.float64)
        al = np.zeros((4096, 2), np.float64)
        check(abi.load().cvr_read_tf1d(path.encode(), C.byref(md), C.byref(ext), C.byref(nr), abi.dptr(rgb), 4096,
                                       C.byref(na), abi.dptr(al), 4096))
        return TransferFunction([tuple(r) for r in rgb[:nr.value]], [tuple(a) for a in al[:na.value]],
                                md.value, bool(ext.value))


# The benchmark transfer function: 4 piecewise-linear RGBA points at
# 0/80/160/255 with opacity 0/0.05/0.4/0.9 and a fixed colour ramp.
BENCH_TF = TransferFunction(
    rgb=[(0.20, 0.30, 0.90, 0), (0.30, 0.80, 0.40, 80), (0.90, 0.70, 0.20, 160), (1.00, 0.95, 0.90, 255)],
    alpha=[(0.0, 0), (0.05, 80), (0.4, 160), (0.9, 255)],
)

# ---------------------------------------------------------------- volumes


def synth_blobs(w, h, d, dtype, n_blobs, seed, noise_max=0.0) -> np.ndarray:
    out = np.empty((d, h, w), np.uint8 if dtype == abi.CVR_U8 else np.uint16)
    check(abi.load().cvr_synth_blobs(abi.vptr(out), w, h, d, dtype, n_blobs, seed, noise_max))
    return out


def synth_value_noise(w, h, d, dtype, seed, octaves=4, lacunarity=2.0, gain=0.5, shells=4) -> np.ndarray:
    out = np.empty((d, h, w), np.uint8 if dtype == abi.CVR_U8 else np.uint16)
    check(abi.load().cvr_synth_value_noise(abi.vptr(out), w, h, d, dtype, octaves, lacunarity, gain, shells, seed))
    return out


def cone_table(half_angle, packing, covered, initial_step, ui_weight, min_sigma) -> abi.ConeTable:
    t = abi.ConeTable()
    check(abi.load().cvr_cone_sampler_build(half_angle, packing, covered, initial_step, ui_weight, min_sigma,
                                            C.byref(t)))
    return t


def gt_vectors(n_occ, occ_aperture, n_sdw, sdw_aperture, seed=1):
    occ = np.zeros((max(n_occ, 1), 3), np.float32)
    sdw = np.zeros((max(n_sdw, 1), 3), np.float32)
    check(abi.load().cvr_gt_kernel_vectors(n_occ, occ_aperture, n_sdw, sdw_aperture, seed, abi.fptr(occ),
                                           abi.fptr(sdw)))
    return occ[:n_occ].copy(), sdw[:n_sdw].copy()


class LibGen:
    """The library's volume generators and table builders (the default `gen`)."""
    synth_blobs = staticmethod(lambda *a, **k: synth_blobs(*a, **k))
    synth_value_noise = staticmethod(lambda *a, **k: synth_value_noise(*a, **k))
    cone_table = staticmethod(lambda *a, **k: cone_table(*a, **k))
    gt_vectors = staticmethod(lambda *a, **k: gt_vectors(*a, **k))


LIB_GEN = LibGen()

# ---------------------------------------------------------------- camera / light


def camera(eye, center=(0, 0, 0), up=(0, 1, 0), fovy=30.0, aspect=0.0) -> abi.Camera:
    c = abi.Camera()
    c.eye[:] = [float(v) for v in eye]
    c.center[:] = [float(v) for v in center]
    c.up[:] = [float(v) for v in up]
    c.fovy_deg = fovy
    c.aspect = aspect
    return c


def orbit_eye(distance, azimuth_deg, elevation_deg):
    a, e = math.radians(azimuth_deg), math.radians(elevation_deg)
    return (distance * math.cos(e) * math.sin(a), distance * math.sin(e), distance * math.cos(e) * math.cos(a))


def _norm(v):
    v = np.asarray(v, np.float64)
    return v / np.linalg.norm(v)


def light(kind, position=(0, 0, 0), forward=(0, 0, 1), up=(0, 1, 0), right=(1, 0, 0), spot_cos=0.0) -> abi.Light:
    L = abi.Light()
    L.type = kind
    L.position[:] = [float(v) for v in position]
    L.forward[:] = [float(v) for v in forward]
    L.up[:] = [float(v) for v in up]
    L.right[:] = [float(v) for v in right]
    L.spot_cos_max = spot_cos
    return L


def light_frame(direction):
    """Orthonormal (forward, up, right) light-camera vectors for a direction."""
    f = _norm(direction)
    ref = np.array([0.0, 1.0, 0.0]) if abs(f[1]) < 0.9 else np.array([1.0, 0.0, 0.0])
    r = _norm(np.cross(ref, f))
    u = _norm(np.cross(f, r))
    return tuple(f), tuple(u), tuple(r)


# ---------------------------------------------------------------- params


def default_step(spacing) -> float:
    """Init(): 0.5 * |spacing| / sqrt(3) (rc1prenderer.cpp:63) = half a voxel."""
    s = np.asarray(spacing, np.float64)
    return float((0.5 / math.sqrt(3.0)) * math.sqrt(float((s * s).sum())))


def ext_params(step, diag, ao_radii=(2, 6, 16), shadow_type=1, apply_occ=True, apply_sdw=True,
               cone_angle_deg=1.0, interval=2.0, initial=2.0, ui_weight=1.0) -> abi.ExtParams:
    p = abi.ExtParams()
    p.step_size = step
    p.apply_occlusion = int(apply_occ)
    p.apply_shadow = int(apply_sdw)
    p.ao_n_shells = len(ao_radii)
    for i, r in enumerate(ao_radii):
        p.ao_radii[i] = float(r)
    p.sdw_cone_angle_rad = float(cone_angle_deg * math.pi / 180.0)
    p.sdw_sample_interval = interval
    p.sdw_initial_step = initial
    p.sdw_ui_weight = ui_weight
    p.sdw_max_distance = 0.75 * diag
    p.shadow_type = shadow_type
    p.ka, p.kd = 0.5, 0.5
    return p


def iso_params(isovalue=0.5, small=0.05, large=1.0, step_range=0.1, color=(0.66, 0.6, 0.05, 1.0)) -> abi.IsoParams:
    """RayCasting1PassIsoAdapt's defaults (rc1pisoadaptrenderer.cpp:10-19)."""
    p = abi.IsoParams()
    p.step_size_small, p.step_size_large, p.step_size_range, p.isovalue = small, large, step_range, isovalue
    p.color[:] = list(color)
    return p


def dos_params(step, apply_occ=True, apply_sdw=False, shadow_type=0) -> abi.DosParams:
    p = abi.DosParams()
    p.step_size = step
    p.apply_occlusion = int(apply_occ)
    p.apply_shadow = int(apply_sdw)
    p.shadow_type = shadow_type
    p.ka, p.kd = 0.5, 0.5
    return p


def gt_params(step, diag, occ_distance=None, sdw_distance=None, light_step=0.5, gap=1.0, apply_occ=True,
              apply_sdw=True, shadow_type=0) -> abi.GtParams:
    p = abi.GtParams()
    p.step_size = step
    p.light_ray_initial_gap = gap
    p.light_ray_step_size = light_step
    p.apply_occlusion = int(apply_occ)
    p.occ_distance = occ_distance if occ_distance is not None else 0.5 * diag
    p.apply_shadow = int(apply_sdw)
    p.sdw_distance = sdw_distance if sdw_distance is not None else 0.75 * diag
    p.shadow_type = shadow_type
    p.ka, p.kd = 0.5, 0.5
    return p


# ---------------------------------------------------------------- context


class Context:
    """One cvr_ctx: the device state a renderer plugin builds in Init()."""

    def __init__(self, device: int = 0):
        self.lib = abi.load()
        h = C.c_void_p()
        code = self.lib.cvr_create(C.byref(h), device)
        if code != abi.CVR_OK:
            raise abi.CvrError(code, self.lib.cvr_last_error(None).decode())
        self.h = h
        self.dims = None
        self.dtype = None
        self.spacing = None

    def close(self):
        if self.h:
            self.lib.cvr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, code):
        check(code, self.h)

    def set_volume(self, vol: np.ndarray, spacing=(1.0, 1.0, 1.0)):
        vol = np.ascontiguousarray(vol)
        d, h, w = vol.shape
        dtype = abi.CVR_U8 if vol.dtype == np.uint8 else abi.CVR_U16
        self._ck(self.lib.cvr_set_volume(self.h, abi.vptr(vol), w, h, d, dtype, *[float(s) for s in spacing]))
        self.dims, self.dtype, self.spacing = (w, h, d), dtype, tuple(float(s) for s in spacing)

    def set_transfer_function(self, tf: TransferFunction):
        rgbt, rgba = tf.tables()
        self._ck(self.lib.cvr_set_transfer_function(self.h, abi.fptr(rgbt), abi.fptr(rgba), len(rgbt)))

    def build_sat(self, ext_per_value: np.ndarray):
        ext = np.ascontiguousarray(ext_per_value, np.float64)
        self._ck(self.lib.cvr_build_sat(self.h, abi.dptr(ext), len(ext)))

    def sat(self) -> tuple[np.ndarray, int]:
        dims = (C.c_int * 3)()
        fb = C.c_int()
        self._ck(self.lib.cvr_get_sat_info(self.h, dims, C.byref(fb)))
        out = np.zeros((dims[2], dims[1], dims[0]), np.int64)
        self._ck(self.lib.cvr_download_sat(self.h, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out, fb.value

    def build_pyramid(self, base_dims=(128, 128, 128), sigma0=1.0, n_levels=0):
        p = abi.PyramidParams()
        p.base_dims[:] = list(base_dims)
        p.sigma0 = sigma0
        p.n_levels = n_levels
        self._ck(self.lib.cvr_build_ext_pyramid(self.h, C.byref(p)))

    def pyramid(self) -> list[np.ndarray]:
        n = C.c_int()
        dims = (C.c_int * 48)()
        self._ck(self.lib.cvr_get_pyramid_info(self.h, C.byref(n), dims, 16))
        levels = []
        for l in range(n.value):
            w, h, d = dims[3 * l], dims[3 * l + 1], dims[3 * l + 2]
            a = np.zeros((d, h, w), np.float32)
            self._ck(self.lib.cvr_download_pyramid_level(self.h, l, abi.fptr(a)))
            levels.append(a)
        return levels

    def set_cone_tables(self, occ: abi.ConeTable, sdw: abi.ConeTable):
        self._ck(self.lib.cvr_set_cone_tables(self.h, C.byref(occ), C.byref(sdw)))

    def set_gt_kernels(self, occ: np.ndarray, sdw: np.ndarray):
        occ = np.ascontiguousarray(occ, np.float32).reshape(-1, 3)
        sdw = np.ascontiguousarray(sdw, np.float32).reshape(-1, 3)
        if len(occ) == 0:
            occ = np.zeros((1, 3), np.float32)[:0]
        self._ck(self.lib.cvr_set_gt_kernels(self.h, abi.fptr(np.ascontiguousarray(occ)), len(occ),
                                             abi.fptr(np.ascontiguousarray(sdw)), len(sdw)))

    def select_volume(self, slot: int):
        self._ck(self.lib.cvr_select_volume(self.h, slot))

    def set_sampling(self, flags: int):
        self._ck(self.lib.cvr_set_sampling(self.h, flags))

    # ---- pixel multiscaling
    def set_multiscaling(self, mode: int, kernel: int = abi.FILTER_HAT, factor_w: int = 2, factor_h: int = 2):
        self._ck(self.lib.cvr_set_multiscaling(self.h, mode, kernel, factor_w, factor_h))

    # ---- gradient Blinn-Phong shading
    def build_gradient(self, model: int = abi.GRADIENT_FINITE_DIFFERENCES, sample_size: int = 1,
                       filter_nxnxn: int = 0, normalized: bool = True):
        p = abi.GradientParams(model, sample_size, filter_nxnxn, int(normalized))
        self._ck(self.lib.cvr_build_gradient(self.h, C.byref(p)))

    def gradient(self) -> np.ndarray:
        """The current volume's gradient, (d, h, w, 3) float32."""
        n = self.dims[0] * self.dims[1] * self.dims[2]
        out = np.zeros(3 * n, np.float32)
        self._ck(self.lib.cvr_download_gradient(self.h, out.ctypes.data_as(C.POINTER(C.c_float)), out.size))
        w, h, d = self.dims
        return out.reshape(d, h, w, 3)

    def set_blinn_phong(self, apply: bool = True, ka: float = 0.5, kd: float = 0.5, ks: float = 0.8,
                        shininess: float = 30.0, specular=(1.0, 1.0, 1.0)):
        bp = abi.BlinnPhong(int(apply), ka, kd, ks, shininess, abi.F3(*specular))
        self._ck(self.lib.cvr_set_blinn_phong(self.h, C.byref(bp)))

    # ---- surrogate network and shading points
    def mlp_init(self, seed: int):
        self._ck(self.lib.cvr_mlp_init(self.h, seed))

    def mlp_params(self) -> np.ndarray:
        p = np.zeros(abi.MLP_PARAMS, np.float32)
        self._ck(self.lib.cvr_mlp_get_params(self.h, abi.fptr(p), abi.MLP_PARAMS))
        return p

    def mlp_set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        self._ck(self.lib.cvr_mlp_set_params(self.h, abi.fptr(p), len(p)))

    def collect_points(self, cam, w, h, step, rate, seed, max_points) -> int:
        n = C.c_int()
        self._ck(self.lib.cvr_surrogate_collect(self.h, C.byref(cam), w, h, step, rate, seed, max_points,
                                                C.byref(n)))
        return n.value

    def clear_points(self):
        self._ck(self.lib.cvr_surrogate_clear_points(self.h))

    def point_count(self) -> int:
        return self.lib.cvr_surrogate_point_count(self.h)

    def points(self) -> np.ndarray:
        n = self.point_count()
        out = np.zeros((n, 6), np.float32)
        self._ck(self.lib.cvr_surrogate_get_points(self.h, abi.fptr(out), n))
        return out

    def set_points(self, pts: np.ndarray):
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 6)
        self._ck(self.lib.cvr_surrogate_set_points(self.h, abi.fptr(pts), len(pts)))

    def label_points(self, lt, gt_params, append_training=False, download=True):
        """Features (n x 48) and GT targets (n x 2) of the point list."""
        n = self.point_count()
        x = np.zeros((n, 48), np.float32) if download else None
        t = np.zeros((n, 2), np.float32) if download else None
        self._ck(self.lib.cvr_surrogate_label(self.h, C.byref(lt), C.byref(gt_params), int(append_training),
                                              abi.fptr(x) if download else None, abi.fptr(t) if download else None,
                                              n))
        return x, t

    def evaluate_points(self, lt, gt_params, cone_params=None) -> dict:
        out = np.zeros(8, np.float64)
        self._ck(self.lib.cvr_surrogate_evaluate(self.h, C.byref(lt), C.byref(gt_params),
                                                 C.byref(cone_params) if cone_params is not None else None,
                                                 abi.dptr(out)))
        keys = ("rmse_ao", "rmse_shadow", "cone_rmse_ao", "cone_rmse_shadow", "points", "mean_ao",
                "mean_shadow", "max_err_ao")
        return dict(zip(keys, out.tolist()))

    def render(self, method, cam, lt, params, w, h, stats=True):
        """Renders into host memory; returns (H x W x 4 float32 image, FrameStats)."""
        out = np.zeros((h, w, 4), np.float32)
        st = abi.FrameStats()
        self._ck(self.lib.cvr_render_host(self.h, method, C.byref(cam), C.byref(lt) if lt is not None else None,
                                          C.byref(params), C.sizeof(params), abi.fptr(out), w, h,
                                          C.byref(st) if stats else None))
        return out, st


# ---------------------------------------------------------------- workloads


@dataclass
class Workload:
    name: str
    method: int
    volume: np.ndarray
    spacing: tuple
    tf: TransferFunction
    cam: abi.Camera
    light: abi.Light
    params: object
    width: int
    height: int
    pyramid: dict = field(default_factory=dict)
    cones: tuple = ()
    gt: tuple = ()
    # the arguments the cone tables (occlusion, shadow) and the kernel vectors
    # were built from: cone_table(*spec) / gt_vectors(*spec)
    cone_spec: tuple = ()
    gt_spec: tuple = ()

    @property
    def dims(self):
        d, h, w = self.volume.shape
        return (w, h, d)

    @property
    def diagonal(self):
        w, h, d = self.dims
        s = self.spacing
        return math.sqrt((w * s[0]) ** 2 + (h * s[1]) ** 2 + (d * s[2]) ** 2)

    @property
    def dtype(self):
        return abi.CVR_U8 if self.volume.dtype == np.uint8 else abi.CVR_U16


def workload(name: str, n: int | None = None, image: int | None = None, gen=None) -> Workload:
    """The seeded synthetic workloads.  n / image shrink the volume side and
    image side for fast parity tests (same generator, same parameters).

    plain      : 64^3 u8, 8 Gaussian blobs, unit cube, 256^2, step 0.5 voxel
    plain_large: the same generator at 256^3 -> 1024^2
    extinction : 256^3 u16 4-octave value noise in 4 nested shells, SAT AO
                 (radii 2, 6, 16 voxels) + directional SAT cone shadow, 1024^2
    ground_truth / cone : 256^3 u8, 32 blobs + U[0,20] background; GT with 16
                 occlusion rays (90 deg, 32 voxels) and 1 shadow ray to a point
                 light at 1-voxel steps; cone method on a 5-level pyramid, 512^2
    iso        : the extinction volume (256^3 u16 value-noise shells) -> 1024^2, isovalue 0.5, the
                 iso-adaptive renderer's default steps (0.05 / 1.0 world units, range 0.1)
    surrogate  : held-out 512^3 u8 of the same blob generator (seed 4020), the
                 ground-truth camera, light and integrator parameters, network
                 inputs on a 6-level pyramid of base n/2, 1024^2
    gen        : volume generators and table builders (default: this library's)
    """
    gen = gen or LIB_GEN
    if name in ("plain", "plain_large"):
        n = n or (64 if name == "plain" else 256)
        image = image or (256 if name == "plain" else 1024)
        vol = gen.synth_blobs(n, n, n, abi.CVR_U8, 8, seed=1000)
        sp = (1.0 / n,) * 3
        cam = camera(orbit_eye(3.0, 35.0, 25.0), fovy=30.0)
        p = abi.PlainParams()
        p.step_size = 0.5 / n
        return Workload(name, abi.PLAIN, vol, sp, BENCH_TF, cam, light(abi.LIGHT_POINT), p, image, image)
    if name == "extinction":
        n = n or 256
        image = image or 1024
        vol = gen.synth_value_noise(n, n, n, abi.CVR_U16, seed=2000)
        sp = (1.0, 1.0, 1.0)
        cam = camera(orbit_eye(3.0 * n, 35.0, 25.0), fovy=30.0)
        fwd, up, right = light_frame((0.35, 0.8, 0.45))
        lt = light(abi.LIGHT_DIRECTIONAL, position=tuple(3.0 * n * np.array(fwd)), forward=fwd, up=up, right=right)
        wl = Workload(name, abi.EXTINCTION, vol, sp, BENCH_TF, cam, lt, None, image, image)
        wl.params = ext_params(default_step(sp), wl.diagonal, ao_radii=(2, 6, 16), shadow_type=1)
        return wl
    if name in ("ground_truth", "cone"):
        n = n or 256
        image = image or 512
        vol = gen.synth_blobs(n, n, n, abi.CVR_U8, 32, seed=3000, noise_max=20.0)
        sp = (1.0, 1.0, 1.0)
        cam = camera(orbit_eye(3.0 * n, -30.0, 20.0), fovy=30.0)
        lpos = tuple(2.0 * n * _norm((-0.5, 1.0, 0.4)))
        fwd, up, right = light_frame(lpos)
        lt = light(abi.LIGHT_POINT, position=lpos, forward=fwd, up=up, right=right)
        wl = Workload(name, abi.GROUND_TRUTH, vol, sp, BENCH_TF, cam, lt, None, image, image)
        diag = wl.diagonal
        if name == "ground_truth":
            wl.params = gt_params(default_step(sp), diag, occ_distance=32.0, light_step=1.0, gap=1.0,
                                  shadow_type=0)
            wl.gt_spec = (16, 90.0, 1, 0.0, 1)
            wl.gt = gen.gt_vectors(*wl.gt_spec)
        else:
            wl.method = abi.CONE_DOS
            wl.params = dos_params(default_step(sp), apply_occ=True, apply_sdw=True, shadow_type=0)
            # RC1PConeTracingDirOcclusionShading defaults (dosrcrenderer.cpp:47-59,112-113):
            # occlusion 20 deg, packing 3, weight 0.35, 0.5*diag; shadow 0.5 deg, packing 1, weight 1, 0.75*diag.
            wl.cone_spec = ((20.0, 1, 0.5 * diag, 3.0, 0.35, 1.0), (0.5, 0, 0.75 * diag, 3.0, 1.0, 1.0))
            wl.cones = tuple(gen.cone_table(*c) for c in wl.cone_spec)
            base = max(1, n // 2)
            wl.pyramid = dict(base_dims=(base, base, base), sigma0=1.0, n_levels=5)
        return wl
    if name == "iso":
        n = n or 256
        image = image or 1024
        vol = gen.synth_value_noise(n, n, n, abi.CVR_U16, seed=2000)
        sp = (1.0, 1.0, 1.0)
        cam = camera(orbit_eye(3.0 * n, 35.0, 25.0), fovy=30.0)
        lt = light(abi.LIGHT_POINT, position=tuple(2.0 * n * _norm((0.4, 1.0, 0.6))))
        return Workload(name, abi.ISO, vol, sp, BENCH_TF, cam, lt, iso_params(), image, image)
    if name == "surrogate":
        n = n or 512
        image = image or 1024
        vol = gen.synth_blobs(n, n, n, abi.CVR_U8, 32, seed=SURROGATE_SEED + SURROGATE_VOLUMES, noise_max=20.0)
        wl = surrogate_workload(vol, image, gen=gen)
        return wl
    raise KeyError(name)


def prepare(ctx: Context, wl: Workload):
    """Init(): uploads the volume and every table the workload's method needs."""
    ctx.set_volume(wl.volume, wl.spacing)
    ctx.set_transfer_function(wl.tf)
    if wl.method == abi.EXTINCTION:
        ctx.build_sat(wl.tf.ext_per_value(wl.dtype))
    if wl.method == abi.CONE_DOS:
        ctx.build_pyramid(**wl.pyramid)
        ctx.set_cone_tables(*wl.cones)
    if wl.method == abi.GROUND_TRUTH:
        ctx.set_gt_kernels(*wl.gt)
    if wl.method == abi.SURROGATE:
        ctx.build_pyramid(**wl.pyramid)
        ctx.set_gt_kernels(*wl.gt)
        ctx.set_cone_tables(*wl.cones)


# ---------------------------------------------------------------- surrogate
# Training data: shading points of random views of SURROGATE_VOLUMES seeded
# blob volumes (the ground-truth workload's generator, seeds 4000..4019) with
# sides from 160 to 448 voxels (the blob generator works in the unit cube, so
# the side sets the scale of the structures and light paths in voxels),
# labelled by the ground-truth integrator with the ground-truth workload's
# parameters (16 occlusion rays of 32 voxels over 90 degrees, 1 shadow ray,
# 1-voxel light steps); half the views use a point light, half a directional.
SURROGATE_SEED = 4000
SURROGATE_VOLUMES = 20
SURROGATE_SIZES = (160, 192, 224, 256, 288, 320, 352, 384, 416, 448)


def surrogate_workload(vol: np.ndarray, image: int, spacing=(1.0, 1.0, 1.0), gen=None) -> Workload:
    """Surrogate shading of a blob volume with the ground-truth workload's camera,
    point light and integrator parameters; the pyramid (base n/2, 6 levels),
    GT kernel vectors and cone tables (for the comparison) it needs."""
    gen = gen or LIB_GEN
    d, h, w = vol.shape
    n = max(w, h, d)
    cam = camera(orbit_eye(3.0 * n, -30.0, 20.0), fovy=30.0)
    lpos = tuple(2.0 * n * _norm((-0.5, 1.0, 0.4)))
    fwd, up, right = light_frame(lpos)
    lt = light(abi.LIGHT_POINT, position=lpos, forward=fwd, up=up, right=right)
    wl = Workload("surrogate", abi.SURROGATE, vol, tuple(spacing), BENCH_TF, cam, lt, None, image, image)
    diag = wl.diagonal
    wl.params = gt_params(default_step(spacing), diag, occ_distance=32.0, light_step=1.0, gap=1.0, shadow_type=0)
    wl.gt_spec = (16, 90.0, 1, 0.0, 1)
    wl.gt = gen.gt_vectors(*wl.gt_spec)
    wl.pyramid = dict(base_dims=(max(1, w // 2), max(1, h // 2), max(1, d // 2)), sigma0=1.0,
                      n_levels=abi.SURROGATE_LEVELS)
    wl.cone_spec = ((20.0, 1, 0.5 * diag, 3.0, 0.35, 1.0), (0.5, 0, 0.75 * diag, 3.0, 1.0, 1.0))
    wl.cones = tuple(gen.cone_table(*c) for c in wl.cone_spec)
    return wl


def cone_params_of(wl: Workload, shadow_type=None) -> abi.DosParams:
    """The cone method's parameters for the same scene (the comparison)."""
    st = wl.params.shadow_type if shadow_type is None else shadow_type
    return dos_params(wl.params.step_size, apply_occ=True, apply_sdw=True, shadow_type=st)


def random_view(rng: np.random.Generator, n: int, directional: bool):
    """A camera on the sphere of radius U[2.2, 3.2] n looking at the centre
    (30 degree field of view) and a light from a uniform random direction:
    a point light at 2 n, or a directional light."""
    v = rng.normal(size=3)
    eye = tuple(float(rng.uniform(2.2, 3.2)) * n * _norm(v))
    up = (0.0, 1.0, 0.0) if abs(_norm(v)[1]) < 0.95 else (1.0, 0.0, 0.0)
    cam = camera(eye, up=up, fovy=30.0)
    ldir = _norm(rng.normal(size=3))
    fwd, lup, right = light_frame(ldir)
    if directional:
        lt = light(abi.LIGHT_DIRECTIONAL, position=tuple(3.0 * n * ldir), forward=fwd, up=lup, right=right)
    else:
        lt = light(abi.LIGHT_POINT, position=tuple(2.0 * n * ldir), forward=fwd, up=lup, right=right)
    return cam, lt


def shaded_sample_count(ctx: Context, cam, w, h, step) -> int:
    """Shaded samples of a frame's primary rays (a plain render's statistics)."""
    p = abi.PlainParams()
    p.step_size = step
    _, st = ctx.render(abi.PLAIN, cam, None, p, w, h)
    return int(st.shaded_samples)


def build_surrogate_training_set(ctx: Context, n_volumes=SURROGATE_VOLUMES, size=None, points=8_000_000,
                                 views=4, image=256, seed=SURROGATE_SEED, log=None) -> int:
    """Appends ~points labelled shading points to the context's training set
    (the network must exist: cvr_mlp_init first).  size=None cycles through
    SURROGATE_SIZES.  Returns the points added."""
    rng = np.random.default_rng(seed)
    per_view = max(1, points // (n_volumes * views))
    added = 0
    for v in range(n_volumes):
        size_v = size or SURROGATE_SIZES[v % len(SURROGATE_SIZES)]
        vol = synth_blobs(size_v, size_v, size_v, abi.CVR_U8, 32, seed=seed + v, noise_max=20.0)
        wl = surrogate_workload(vol, image)
        prepare(ctx, wl)
        step = wl.params.step_size
        for k in range(views):
            directional = (k % 2) == 1
            cam, lt = random_view(rng, size_v, directional)
            shaded = shaded_sample_count(ctx, cam, image, image, step)
            if shaded == 0:
                continue
            rate = min(1.0, per_view / shaded)
            ctx.clear_points()
            got = ctx.collect_points(cam, image, image, step, rate, int(rng.integers(1 << 62)), per_view)
            gp = gt_params(step, wl.diagonal, occ_distance=32.0, light_step=1.0, gap=1.0,
                           shadow_type=2 if directional else 0)
            ctx.label_points(lt, gp, append_training=True, download=False)
            added += got
        if log:
            log(f"volume {v}: {added} points")
    return added


# Adam schedule: (epochs, learning rate) phases.
SURROGATE_SCHEDULE = ((24, 2e-3), (16, 7e-4), (12, 2e-4), (8, 5e-5))


def train_surrogate(ctx: Context, batch=4096, schedule=SURROGATE_SCHEDULE, seed=SURROGATE_SEED) -> list:
    """Adam over the context's training set; returns the per-epoch losses."""
    losses = []
    for i, (epochs, lr) in enumerate(schedule):
        out = np.zeros(epochs, np.float32)
        ctx._ck(ctx.lib.cvr_mlp_train(ctx.h, epochs, batch, lr, seed + i, abi.fptr(out)))
        losses.extend(out.tolist())
    return losses


def evaluate_surrogate(ctx: Context, wl: Workload, points=2_000_000, seed=7) -> dict:
    """RMSE of the network and of the cone method against the ground-truth
    integrator over a uniform sample of the shading points of wl's frame
    (wl prepared on ctx, the network trained)."""
    step = wl.params.step_size
    shaded = shaded_sample_count(ctx, wl.cam, wl.width, wl.height, step)
    rate = min(1.0, points / max(shaded, 1))
    ctx.clear_points()
    ctx.collect_points(wl.cam, wl.width, wl.height, step, rate, seed, points)
    r = ctx.evaluate_points(wl.light, wl.params, cone_params_of(wl))
    r["shaded_samples"] = shaded
    return r


# ---------------------------------------------------------------- batches
# The batched workload: 4 volumes of uneven size (128^3 u8, 192x256x160 u16,
# 256^3 u8, 384^3 u16, seeded value noise, seeds 5000..5003) x 16 views on a
# sphere x 4 directional lights, 512^2 images, extinction shading (SAT AO
# radii 2, 6, 16 + directional SAT cone shadow) and surrogate shading (the
# same views and lights, directional shadow), one job list.
BATCH_VOLUMES = ((128, 128, 128, abi.CVR_U8), (192, 256, 160, abi.CVR_U16), (256, 256, 256, abi.CVR_U8),
                 (384, 384, 384, abi.CVR_U16))
BATCH_LIGHTS = ((0.35, 0.8, 0.45), (-0.6, 0.5, 0.3), (0.2, 0.4, -0.9), (-0.3, 0.9, -0.2))


def sphere_views(n_views: int):
    """n_views unit directions on a Fibonacci sphere (elevation within +-60 deg)."""
    out = []
    golden = math.pi * (3.0 - math.sqrt(5.0))
    for i in range(n_views):
        y = 0.85 * (1.0 - 2.0 * (i + 0.5) / n_views)
        r = math.sqrt(max(0.0, 1.0 - y * y))
        out.append((r * math.cos(golden * i), y, r * math.sin(golden * i)))
    return out


@dataclass
class Batch:
    volumes: list            # (array, spacing)
    jobs: list               # abi.Job
    params: list             # kept alive: the params structs the jobs point at
    width: int
    height: int


def batch_volumes(scale: float = 1.0):
    """The batch's four volumes (value noise, 4 octaves, shells), optionally scaled down."""
    vols = []
    for i, (w, h, d, dt) in enumerate(BATCH_VOLUMES):
        w, h, d = max(8, int(w * scale)), max(8, int(h * scale)), max(8, int(d * scale))
        vols.append(synth_value_noise(w, h, d, dt, seed=5000 + i))
    return vols


def prepare_batch_volumes(ctx: Context, vols, pyramid=True):
    """Uploads each volume into its slot with its SAT and (for the surrogate)
    its pyramid of base n/2 and 6 levels; leaves slot 0 current."""
    for slot, vol in enumerate(vols):
        ctx.select_volume(slot)
        ctx.set_volume(vol, (1.0, 1.0, 1.0))
        if slot == 0:
            ctx.set_transfer_function(BENCH_TF)
        dtype = abi.CVR_U8 if vol.dtype == np.uint8 else abi.CVR_U16
        ctx.build_sat(BENCH_TF.ext_per_value(dtype))
        if pyramid:
            d, h, w = vol.shape
            ctx.build_pyramid(base_dims=(max(1, w // 2), max(1, h // 2), max(1, d // 2)), sigma0=1.0,
                              n_levels=abi.SURROGATE_LEVELS)
    ctx.select_volume(0)


def batch_jobs(vols, n_views=16, lights=BATCH_LIGHTS, image=512, methods=(abi.EXTINCTION, abi.SURROGATE),
               out_ptrs=None) -> Batch:
    """Job list: volume x view x light x method (in that nesting order).
    out_ptrs: device pointers, one per job, in the same order."""
    jobs, keep = [], []
    k = 0
    for slot, vol in enumerate(vols):
        d, h, w = vol.shape
        n = max(w, h, d)
        diag = math.sqrt(w * w + h * h + d * d)
        for v in sphere_views(n_views):
            cam = camera(tuple(2.6 * n * np.asarray(v)), fovy=30.0)
            for ldir in lights:
                fwd, up, right = light_frame(ldir)
                lt = light(abi.LIGHT_DIRECTIONAL, position=tuple(3.0 * n * np.asarray(fwd)), forward=fwd, up=up,
                           right=right)
                for m in methods:
                    if m == abi.EXTINCTION:
                        p = ext_params(default_step((1.0, 1.0, 1.0)), diag, ao_radii=(2, 6, 16), shadow_type=1)
                    else:
                        p = gt_params(default_step((1.0, 1.0, 1.0)), diag, occ_distance=32.0, light_step=1.0,
                                      gap=1.0, shadow_type=2)
                    keep.append(p)
                    j = abi.Job()
                    j.volume, j.method = slot, m
                    j.params, j.params_size = C.addressof(p), C.sizeof(p)
                    j.camera, j.light = cam, lt
                    j.width = j.height = image
                    j.out_rgba_dev = out_ptrs[k] if out_ptrs is not None else None
                    jobs.append(j)
                    k += 1
    return Batch(list(vols), jobs, keep, image, image)
