"""Gradient Blinn-Phong shading: the per-voxel gradient builders and the
gradient branch of every ShadeSample.

The oracle's builders are pinned bit-for-bit (after the RGB16F rounding the
reference's texture applies) against the reference's own
GenerateGradientTexture / GenerateSobelFeldmanGradientTexture, compiled from
its sources, through the committed golden vectors.  GPU gradients must equal
the oracle's FP16 values except for rare FP32-vs-FP64 rounding ties (one
FP16 ulp); images with gradient shading meet the renderers' bar (max
|error| <= 1/255, PSNR >= 50 dB against the FP64 oracle) on the FP32
sampling path.
"""
import ctypes as C
import math
from pathlib import Path

import numpy as np
import pytest

import oracle
from cpp_volume_rendering_gb300 import abi, scene

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_tables.npz"
# name: (model, gradient_sample_size, filter_nxnxn, normalized_gradient), as in make_golden.py
CASES = {
    "sobel": (abi.GRADIENT_SOBEL_FELDMAN, 1, 0, 1),
    "fd": (abi.GRADIENT_FINITE_DIFFERENCES, 1, 0, 1),
    "fd_n2_raw": (abi.GRADIENT_FINITE_DIFFERENCES, 2, 0, 0),
    "fd_filter3": (abi.GRADIENT_FINITE_DIFFERENCES, 1, 3, 1),
}


def half(a):
    return np.asarray(a, np.float32).astype(np.float16).astype(np.float32)


# ------------------------------------------------------------------ CPU: oracle
@pytest.mark.parametrize("vol_name", ["u8", "u16"])
@pytest.mark.parametrize("case", list(CASES))
def test_oracle_gradient_matches_reference_golden(vol_name, case):
    g = np.load(GOLDEN)
    vol = g[f"grad_{vol_name}_volume"]
    orc = oracle.Oracle()
    orc.set_volume(vol, (1.0, 1.0, 1.0))
    orc.build_gradient(*CASES[case])
    assert np.array_equal(orc.gradient(), half(g[f"grad_{vol_name}_{case}"]))


def test_oracle_gradient_matches_live_reference():
    """A larger ragged u8 volume through the reference's compiled builders."""
    if not oracle.ref_available():
        pytest.skip("reference sources not available")
    ref = oracle.load_ref()
    rng = np.random.default_rng(3)
    vol = rng.integers(0, 256, size=(11, 17, 14)).astype(np.uint8)
    vol[3:8, 4:12, 2:9] = 200
    orc = oracle.Oracle()
    orc.set_volume(vol, (1.0, 1.0, 1.0))
    d, h, w = vol.shape
    for model, n, filt, norm in [(0, 1, 0, 1), (1, 1, 0, 1), (1, 3, 5, 1), (1, 1, 0, 0)]:
        out = np.zeros((d, h, w, 3), np.float32)
        assert ref.ref_gradient(C.c_void_p(vol.ctypes.data), w, h, d, 1, model, n, filt, norm,
                                C.c_void_p(out.ctypes.data)) == 0
        orc.build_gradient(model, n, filt, bool(norm))
        assert np.array_equal(orc.gradient(), half(out)), (model, n, filt, norm)


def test_oracle_gradient_shading_identities():
    """With ks = 0, ka = 1, kd = 0 the plain renderer's ShadeBlinnPhong is the
    identity (clr * 1); a brighter specular term only adds light."""
    wl = scene.workload("plain", n=24, image=24)
    wl.light = scene.light(abi.LIGHT_POINT, position=(2.0, 3.0, 1.5))
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    base, _, _ = orc.render(wl.method, wl.cam, wl.light, wl.params, 24, 24)
    orc.build_gradient(abi.GRADIENT_FINITE_DIFFERENCES)
    orc.set_blinn_phong(True, ka=1.0, kd=0.0, ks=0.0)
    same, _, _ = orc.render(wl.method, wl.cam, wl.light, wl.params, 24, 24)
    assert np.allclose(same, base, atol=1e-12)
    orc.set_blinn_phong(True, ka=0.5, kd=0.5, ks=0.0)
    dull, _, _ = orc.render(wl.method, wl.cam, wl.light, wl.params, 24, 24)
    orc.set_blinn_phong(True, ka=0.5, kd=0.5, ks=0.8)
    shiny, _, _ = orc.render(wl.method, wl.cam, wl.light, wl.params, 24, 24)
    assert (shiny[..., :3] >= dull[..., :3] - 1e-12).all() and shiny[..., :3].sum() > dull[..., :3].sum()
    assert np.array_equal(shiny[..., 3], base[..., 3])  # shading never changes opacity
    orc.set_blinn_phong(False)
    off, _, _ = orc.render(wl.method, wl.cam, wl.light, wl.params, 24, 24)
    assert np.array_equal(off, base)


def test_separable_sobel_sums_equal_the_27_tap_sums():
    """The TMA builder's separable form of Sobel-Feldman (in-plane partial sums
    D, E, Q of three planes, weights (2 >> |v1|)(2 >> |v2|)) gives the same
    integers as the direct 27-tap sums with weights 4 >> (|v1| + |v2|)."""
    rng = np.random.default_rng(8)
    v = np.zeros((9, 10, 11), np.int64)
    v[1:-1, 1:-1, 1:-1] = rng.integers(0, 65536, size=(7, 8, 9))  # 0 outside the grid
    z, y, x = np.meshgrid(np.arange(1, 8), np.arange(1, 9), np.arange(1, 10), indexing="ij")
    sx = np.zeros_like(z); sy = np.zeros_like(z); sz = np.zeros_like(z)
    for v1 in (-1, 0, 1):
        for v2 in (-1, 0, 1):
            w = 4 >> (abs(v1) + abs(v2))
            sz += w * (v[z - 1, y + v2, x + v1] - v[z + 1, y + v2, x + v1])
            sy += w * (v[z + v2, y - 1, x + v1] - v[z + v2, y + 1, x + v1])
            sx += w * (v[z + v1, y + v2, x - 1] - v[z + v1, y + v2, x + 1])

    def partial(zz):  # the in-plane sums of plane zz at every (y, x)
        row_s = lambda yy: v[zz, yy, x - 1] + 2 * v[zz, yy, x] + v[zz, yy, x + 1]
        row_d = lambda yy: v[zz, yy, x - 1] - v[zz, yy, x + 1]
        D = row_d(y - 1) + 2 * row_d(y) + row_d(y + 1)
        E = row_s(y - 1) - row_s(y + 1)
        Q = row_s(y - 1) + 2 * row_s(y) + row_s(y + 1)
        return D, E, Q

    (D0, E0, Q0), (D1, E1, Q1), (D2, E2, Q2) = partial(z - 1), partial(z), partial(z + 1)
    assert np.array_equal(D0 + 2 * D1 + D2, sx)
    assert np.array_equal(E0 + 2 * E1 + E2, sy)
    assert np.array_equal(Q0 - Q2, sz)


# ------------------------------------------------------------------ GPU
def _gpu_vs_oracle_gradient(ctx, vol, model, n=1, filt=0, norm=True):
    ctx.set_volume(vol, (1.0, 1.0, 1.0))
    ctx.build_gradient(model, n, filt, norm)
    got = ctx.gradient()
    orc = oracle.Oracle()
    orc.set_volume(vol, (1.0, 1.0, 1.0))
    orc.build_gradient(model, n, filt, norm)
    want = orc.gradient()
    diff = np.abs(got - want)
    # one FP16 ulp at the value's magnitude: 2^-10 relative (2^-24 absolute near 0)
    ulp = np.maximum(np.abs(want) * 2.0 ** -10, 2.0 ** -24)
    assert (diff <= ulp * 1.0001).all(), (model, float(diff.max()))
    assert (diff == 0).mean() >= 0.999, (model, float((diff == 0).mean()))


@pytest.mark.gpu
@pytest.mark.parametrize("case", list(CASES))
def test_gpu_gradient_golden_volumes(ctx, case):
    g = np.load(GOLDEN)
    for vol_name in ("u8", "u16"):
        _gpu_vs_oracle_gradient(ctx, g[f"grad_{vol_name}_volume"], *CASES[case])


@pytest.mark.gpu
def test_gpu_gradient_larger_volumes(ctx):
    u8 = scene.synth_blobs(48, 40, 36, abi.CVR_U8, 6, seed=21)
    u16 = scene.synth_value_noise(33, 29, 31, abi.CVR_U16, seed=22)
    for vol in (u8, u16):
        for model, n, filt, norm in [(0, 1, 0, True), (1, 1, 0, True), (1, 2, 0, False), (2, 1, 0, True)]:
            _gpu_vs_oracle_gradient(ctx, vol, model, n, filt, norm)


@pytest.mark.gpu
@pytest.mark.parametrize("dims,dtype,tma", [((48, 37, 29), abi.CVR_U8, True), ((40, 23, 35), abi.CVR_U16, True),
                                             ((64, 64, 70), abi.CVR_U8, True), ((16, 9, 5), abi.CVR_U8, True),
                                             ((37, 20, 18), abi.CVR_U8, False), ((36, 17, 9), abi.CVR_U16, False)])
def test_gradient_builders_agree_bit_for_bit(ctx, dims, dtype, tma):
    """The tensor-memory-accelerator builder (rows a multiple of 16 bytes;
    ragged tiles in x, y and z, out-of-grid halo filled by the copy engine),
    the shared-memory ring builder and the per-voxel builder give the same
    FP16 gradients for every 3x3x3 stencil."""
    w, h, d = dims
    rng = np.random.default_rng(w * 10000 + h * 100 + d)
    top = 256 if dtype == abi.CVR_U8 else 65536
    vol = rng.integers(0, top, size=(d, h, w)).astype(np.uint8 if dtype == abi.CVR_U8 else np.uint16)
    vol[: d // 2, : h // 2, : w // 2] = top // 3  # a flat block: zero gradients
    ctx.set_volume(vol, (1.0, 1.0, 1.0))
    want_first = abi.GRADIENT_KERNEL_TMA if tma else abi.GRADIENT_KERNEL_TILED
    try:
        for model, n, filt, norm in [(0, 1, 0, True), (1, 1, 0, True), (1, 1, 0, False), (1, 1, 3, True),
                                     (2, 1, 0, True)]:
            outs, kinds = [], []
            for kern in (abi.GRADIENT_KERNEL_AUTO, abi.GRADIENT_KERNEL_TILED, abi.GRADIENT_KERNEL_GENERIC):
                ctx._ck(ctx.lib.cvr_set_gradient_kernel(ctx.h, kern))
                ctx.build_gradient(model, n, filt, norm)
                outs.append(ctx.gradient())
                kinds.append(ctx.lib.cvr_get_gradient_kernel(ctx.h))
            assert kinds == [want_first, abi.GRADIENT_KERNEL_TILED, abi.GRADIENT_KERNEL_GENERIC], kinds
            assert np.array_equal(outs[0], outs[1]), (model, n, filt, norm)
            assert np.array_equal(outs[0], outs[2]), (model, n, filt, norm)
            assert np.abs(outs[0]).max() > 0
    finally:
        ctx._ck(ctx.lib.cvr_set_gradient_kernel(ctx.h, abi.GRADIENT_KERNEL_AUTO))
    assert ctx.lib.cvr_set_gradient_kernel(ctx.h, abi.GRADIENT_KERNEL_TMA) == abi.CVR_ERR_INVALID_ARG


def _shaded_pair(ctx, wl, model, bp, cache=None, sampling=0):
    scene.prepare(ctx, wl)
    ctx.build_gradient(model)
    ctx.set_blinn_phong(True, **bp)
    ctx.set_sampling(sampling)
    if cache:
        ctx._ck(ctx.lib.cvr_set_light_cache(ctx.h, *cache))
    try:
        img, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
    finally:
        ctx.set_blinn_phong(False)
        ctx.set_sampling(abi.SAMPLING_TEX_FEATURES)
        if cache:
            ctx._ck(ctx.lib.cvr_set_light_cache(ctx.h, 0, 0, 0))
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    orc.build_gradient(model)
    orc.set_blinn_phong(True, **bp)
    if cache:
        orc.set_light_cache(*cache)
    ref, _, total = orc.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height, precision=64)
    return img, st, ref, total


def _stats(img, ref):
    err = np.abs(img.astype(np.float64) - ref)
    mse = float(np.mean(err ** 2))
    return float(err.max()), (float("inf") if mse == 0 else 10 * math.log10(1.0 / mse))


SHADED = [
    ("plain", 40, 72, abi.GRADIENT_FINITE_DIFFERENCES, None),
    ("plain", 40, 64, abi.GRADIENT_SOBEL_FELDMAN, None),
    ("extinction", 40, 64, abi.GRADIENT_FINITE_DIFFERENCES, None),
    ("extinction", 36, 48, abi.GRADIENT_SOBEL_FELDMAN, (16, 16, 16)),
    ("cone", 40, 64, abi.GRADIENT_FINITE_DIFFERENCES, None),
    ("cone", 40, 48, abi.GRADIENT_FINITE_DIFFERENCES, (20, 20, 20)),
    ("ground_truth", 32, 48, abi.GRADIENT_SOBEL_FELDMAN, None),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,n,image,model,cache", SHADED)
def test_gradient_shaded_frames_match_oracle(ctx, name, n, image, model, cache):
    wl = scene.workload(name, n=n, image=image)
    if name == "plain":
        wl.light = scene.light(abi.LIGHT_POINT, position=(1.5, 2.5, 1.0))
    bp = dict(ka=0.4, kd=0.6, ks=0.8, shininess=30.0, specular=(1.0, 0.9, 0.7))
    img, st, ref, total = _shaded_pair(ctx, wl, model, bp, cache)
    mx, p = _stats(img, ref)
    print(f"gradient {name} model {model} cache {cache}: max {mx:.2e} psnr {p:.1f} dB")
    assert np.isfinite(img).all()
    assert mx <= 1.0 / 255.0, mx
    assert p >= 50.0, p
    assert abs(int(st.samples) - int(total)) <= max(2, total // 2000)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["plain", "extinction"])
def test_gradient_texture_sampling(ctx, name):
    """The texture-unit path (volume and gradient through hardware trilinear
    filtering, as the reference samples them) stays close to the FP64 oracle."""
    wl = scene.workload(name, n=40, image=64)
    if name == "plain":
        wl.light = scene.light(abi.LIGHT_POINT, position=(1.5, 2.5, 1.0))
    bp = dict(ka=0.5, kd=0.5, ks=0.8, shininess=30.0)
    img, st, ref, total = _shaded_pair(ctx, wl, abi.GRADIENT_FINITE_DIFFERENCES, bp,
                                       sampling=abi.SAMPLING_TEX_VOLUME | abi.SAMPLING_TEX_FEATURES)
    mx, p = _stats(img, ref)
    print(f"gradient {name} texture sampling: max {mx:.2e} psnr {p:.1f} dB")
    # measured on GB300: plain 69 dB / max 1.1e-2, extinction 53.5 dB / max 3.5e-2
    assert np.isfinite(img).all()
    assert mx <= 16.0 / 255.0, mx
    assert p >= 45.0, p


@pytest.mark.gpu
def test_gradient_shading_switch_and_errors(ctx):
    wl = scene.workload("plain", n=32, image=32)
    scene.prepare(ctx, wl)
    ctx.build_gradient(abi.GRADIENT_NONE)  # the slot may keep a model from an earlier frame
    base, _ = ctx.render(wl.method, wl.cam, wl.light, wl.params, 32, 32)
    # apply without a gradient model: the reference's ApplyGradientPhongShading is 0 then
    ctx.set_blinn_phong(True)
    try:
        same, _ = ctx.render(wl.method, wl.cam, wl.light, wl.params, 32, 32)
        assert np.array_equal(same, base)
        ctx.build_gradient(abi.GRADIENT_FINITE_DIFFERENCES)
        lit = scene.light(abi.LIGHT_POINT, position=(1.5, 2.5, 1.0))
        shaded, _ = ctx.render(wl.method, wl.cam, lit, wl.params, 32, 32)
        assert not np.array_equal(shaded, base)
        # a volume change keeps the model and rebuilds the gradient on the next frame
        ctx.set_volume(wl.volume, wl.spacing)
        again, _ = ctx.render(wl.method, wl.cam, lit, wl.params, 32, 32)
        assert np.array_equal(again, shaded)
        # the light position is required
        with pytest.raises(abi.CvrError):
            ctx.render(wl.method, wl.cam, None, wl.params, 32, 32)
        bad = abi.GradientParams(7, 1, 0, 1)
        assert ctx.lib.cvr_build_gradient(ctx.h, C.byref(bad)) == abi.CVR_ERR_INVALID_ARG
        bad = abi.GradientParams(abi.GRADIENT_FINITE_DIFFERENCES, 0, 0, 1)
        assert ctx.lib.cvr_build_gradient(ctx.h, C.byref(bad)) == abi.CVR_ERR_INVALID_ARG
        # model NONE drops it: frames are unshaded again
        ctx.build_gradient(abi.GRADIENT_NONE)
        off, _ = ctx.render(wl.method, wl.cam, lit, wl.params, 32, 32)
        assert np.array_equal(off, base)
    finally:
        ctx.set_blinn_phong(False)
