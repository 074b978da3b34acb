"""Pixel multiscaling (BaseVolumeRenderer::MULTISCALING + RenderFrameToScreen):
the oracle's kernels and digital filters pinned to the reference's filter
classes (golden vectors), properties of the restated post-passes (CPU), and
the device post-passes and multiscaled frames against the FP64 oracle (GPU):
post-pass alone within 1e-5 of the image range, frames within 1/255."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import oracle
from cpp_volume_rendering_gb300 import abi, scene
from oracle import postpass as pp
from tests.devmem import DeviceMemory
from tests.test_gpu_parity import compare

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_tables.npz"


@pytest.mark.parametrize("k", range(6))
def test_oracle_kernels_match_reference(k):
    g = np.load(GOLDEN)
    xs = g["filt_x"]
    assert pp.support(k) == g[f"filt_{k}_support"][0]
    mine = np.array([pp.weight(k, float(x)) for x in xs])
    assert np.abs(mine - g[f"filt_{k}_weights"]).max() <= 1e-6


@pytest.mark.parametrize("k", [abi.FILTER_CARDINAL_BSPLINE3, abi.FILTER_CARDINAL_OMOMS3])
def test_oracle_digital_filter_matches_reference(k):
    g = np.load(GOLDEN)
    mine = pp.linear_solve(pp.LU[k], g["filt_line"].astype(np.float64))
    assert np.abs(mine - g[f"filt_{k}_digital"]).max() <= 1e-5


def _chunked_solve(L, f, chunk=64, warm=32):
    """The device digital filter's schedule (k_df_forward / k_df_reverse):
    every chunk of a line recomputed from a zero state 'warm' entries before
    it, forward then reverse; exact starts at the line's ends."""
    m, L_inf = len(L), L[-1]
    v_inv = L_inf / (1.0 + L_inf)
    n = len(f)
    y, o = np.zeros_like(f), np.zeros_like(f)
    for s in range(0, n, chunk):
        e = min(s + chunk, n)
        i, prev = s - warm, 0.0
        if i <= 0:
            prev, i = f[0], 1
            if s == 0:
                y[0] = prev
        for i in range(i, e):
            prev = f[i] - (L[i - 1] if i < m else L_inf) * prev
            if i >= s:
                y[i] = prev
    for s in range(0, n, chunk):
        e = min(s + chunk, n)
        i, nxt = e - 1 + warm, 0.0
        if i >= n - 1:
            nxt, i = y[n - 1] * v_inv, n - 2
            if e == n:
                o[n - 1] = nxt
        for i in range(i, s - 1, -1):
            nxt = (L_inf if i >= m - 1 else L[i]) * (y[i] - nxt)
            if i < e:
                o[i] = nxt
    return o


@pytest.mark.parametrize("k", [pp.CARDINAL_BSPLINE3, pp.CARDINAL_OMOMS3])
def test_chunked_digital_filter_schedule_matches_sequential_solve(k):
    """Starting a chunk 32 entries early from zero leaves an error scaled by
    L^32 (< 2e-15): the chunked schedule equals the sequential LU solve to
    FP64 rounding on lines of every length class."""
    rng = np.random.default_rng(k)
    for n in (len(pp.LU[k]), 10, 33, 64, 65, 96, 97, 129, 200, 1024):
        f = rng.uniform(0.0, 1.0, n)
        assert np.abs(_chunked_solve(pp.LU[k], f) - pp.linear_solve(pp.LU[k], f)).max() <= 1e-14, n


def test_oracle_postpass_properties():
    rng = np.random.default_rng(3)
    lo = rng.uniform(0, 1, size=(6, 7, 4))
    hi = np.repeat(np.repeat(lo, 2, axis=0), 2, axis=1)  # each texel a 2x2 block
    # a 2x2 multisample / box down-scale of a block image gives the blocks back
    assert np.allclose(pp.rescale(hi, pp.MULTISAMPLE, pp.HAT, 7, 6), lo, atol=1e-12)
    assert np.allclose(pp.rescale(hi, pp.DOWNSCALE, pp.BOX, 7, 6), lo, atol=1e-12)
    # the interpolating kernels reproduce a constant away from the border
    const = np.full((9, 11, 4), 0.25)
    for k in (pp.HAT, pp.CATMULL_ROM, pp.CARDINAL_BSPLINE3, pp.CARDINAL_OMOMS3):
        up = pp.rescale(const, pp.UPSCALE, k, 22, 18)
        assert np.allclose(up[4:-4, 4:-4], 0.25, atol=2e-6), k
    # Mitchell-Netravali weights sum to 1 at integer shifts
    assert abs(sum(pp.weight(pp.MITCHELL_NETRAVALI, x) for x in (-2, -1, 0, 1, 2)) - 1.0) < 1e-12
    assert pp.generated_size(pp.UPSCALE, 2, 2, 33, 21) == (16, 10)


@pytest.mark.gpu
def test_multiscaling_validation(ctx):
    assert ctx.lib.cvr_set_multiscaling(ctx.h, 4, 1, 2, 2) == abi.CVR_ERR_INVALID_ARG
    assert ctx.lib.cvr_set_multiscaling(ctx.h, 1, 6, 2, 2) == abi.CVR_ERR_INVALID_ARG
    assert ctx.lib.cvr_set_multiscaling(ctx.h, 1, 1, 0, 2) == abi.CVR_ERR_INVALID_ARG
    m, k, fw, fh = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    assert ctx.lib.cvr_get_multiscaling(ctx.h, C.byref(m), C.byref(k), C.byref(fw), C.byref(fh)) == 0
    assert (m.value, k.value, fw.value, fh.value) == (0, abi.FILTER_HAT, 2, 2)  # the reference's defaults


CASES = [(abi.MULTISCALE_MULTISAMPLE, abi.FILTER_HAT, 74, 58, 37, 29)]
CASES += [(abi.MULTISCALE_DOWNSCALE, k, 74, 58, 37, 29) for k in range(6)]
CASES += [(abi.MULTISCALE_UPSCALE, k, 19, 15, 38, 30) for k in range(6)]


@pytest.mark.gpu
@pytest.mark.parametrize("mode,k,sw,sh,w,h", CASES)
def test_device_postpass_matches_oracle(ctx, mode, k, sw, sh, w, h):
    rng = np.random.default_rng(10 * mode + k)
    src = rng.uniform(0.0, 1.0, size=(sh, sw, 4)).astype(np.float32)
    mem = DeviceMemory()
    try:
        ps = mem.upload(src)
        pd = mem.alloc(w * h * 16, fill=0)
        abi.check(ctx.lib.cvr_rescale_frame(ctx.h, mode, k, ps, sw, sh, pd, w, h), ctx.h)
        abi.check(ctx.lib.cvr_sync(ctx.h), ctx.h)
        got = mem.download(pd, (h, w, 4))
        again = mem.download(ps, (sh, sw, 4))
    finally:
        mem.close()
    assert np.array_equal(again, src)  # the source is not modified
    want = pp.rescale(src, mode, k, w, h)
    scale = max(1.0, float(np.abs(want).max()))
    assert np.abs(got - want).max() <= 1e-5 * scale, (mode, k, float(np.abs(got - want).max()))


@pytest.mark.gpu
@pytest.mark.parametrize("name,mode,k", [("plain", abi.MULTISCALE_MULTISAMPLE, abi.FILTER_HAT),
                                         ("extinction", abi.MULTISCALE_DOWNSCALE, abi.FILTER_HAT),
                                         ("extinction", abi.MULTISCALE_DOWNSCALE, abi.FILTER_CARDINAL_OMOMS3),
                                         ("plain", abi.MULTISCALE_UPSCALE, abi.FILTER_CATMULL_ROM),
                                         ("cone", abi.MULTISCALE_UPSCALE, abi.FILTER_CARDINAL_BSPLINE3)])
def test_multiscaled_frames_match_oracle(ctx, name, mode, k):
    wl = scene.workload(name, n=36, image=48)
    scene.prepare(ctx, wl)
    ctx.set_multiscaling(mode, k)
    try:
        img, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, 48, 40)
    finally:
        ctx.set_multiscaling(abi.MULTISCALE_SINGLE)
    gw, gh = pp.generated_size(mode, 2, 2, 48, 40)
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    cam = abi.Camera.from_buffer_copy(wl.cam)
    cam.aspect = 48.0 / 40.0  # the generated frame keeps the output's aspect
    gen, _, total = orc.render(wl.method, cam, wl.light, wl.params, gw, gh, precision=64)
    ref = pp.rescale(gen, mode, k, 48, 40)
    compare(img, ref, f"{name} multiscale mode {mode} kernel {k}")
    assert abs(int(st.samples) - int(total)) <= max(2, total // 2000)
