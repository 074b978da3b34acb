"""The adaptive-step isosurface caster (RayCasting1PassIsoAdapt) against the
FP64 oracle.  First-hit isosurfaces are discontinuous: a ray that grazes the
surface, or whose small/large step choice sits on the StepSizeRange edge,
can flip between hit and miss under FP32 vs FP64 arithmetic, so the bar is
max |error| <= 1/255 on all but 0.2 % of the pixels (the flips are counted
and reported) and PSNR >= 40 dB; with texture-unit sampling 2 % and 25 dB."""
import math

import numpy as np
import pytest

import oracle
from cpp_volume_rendering_gb300 import abi, scene


def flip_stats(img, ref):
    err = np.abs(img.astype(np.float64) - ref).max(axis=-1)
    mse = float(np.mean((img.astype(np.float64) - ref) ** 2))
    psnr = float("inf") if mse == 0 else 10 * math.log10(1.0 / mse)
    return float((err > 1.0 / 255.0).mean()), float(err.max()), psnr


def test_oracle_iso_properties():
    wl = scene.workload("iso", n=32, image=32)
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    img, _, total = orc.render(wl.method, wl.cam, wl.light, wl.params, 32, 32)
    a = img[..., 3]
    assert set(np.unique(a)) <= {0.0, 1.0} and a.mean() > 0.1  # opaque colour: first hit only
    hit = a > 0
    assert np.allclose(img[hit][:, :3], [0.66, 0.6, 0.05], atol=1e-7)
    p = scene.iso_params(isovalue=1.5)  # above every normalised density: nothing
    empty, _, _ = orc.render(wl.method, wl.cam, wl.light, p, 32, 32)
    assert not empty.any()
    p = scene.iso_params(color=(1.0, 0.5, 0.25, 0.3))  # translucent: several crossings composite
    multi, _, _ = orc.render(wl.method, wl.cam, wl.light, p, 32, 32)
    assert multi[..., 3].max() > 0.3 + 1e-6


CASES = [("opaque", dict(), 0, False), ("translucent", dict(color=(1.0, 0.5, 0.25, 0.35)), 0, False),
         ("gradient", dict(), 0, True), ("small_range", dict(step_range=0.02, small=0.1, large=0.75), 0, False),
         ("texture", dict(), abi.SAMPLING_TEX_VOLUME, False)]


@pytest.mark.gpu
@pytest.mark.parametrize("label,kw,sampling,grad", CASES)
def test_iso_frames_match_oracle(ctx, label, kw, sampling, grad):
    wl = scene.workload("iso", n=48, image=96)
    wl.params = scene.iso_params(**kw)
    scene.prepare(ctx, wl)
    if grad:
        ctx.build_gradient(abi.GRADIENT_FINITE_DIFFERENCES)
        ctx.set_blinn_phong(True)
    ctx.set_sampling(sampling)
    try:
        img, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, 96, 96)
    finally:
        ctx.set_sampling(abi.SAMPLING_TEX_FEATURES)
        ctx.set_blinn_phong(False)
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    if grad:
        orc.build_gradient(abi.GRADIENT_FINITE_DIFFERENCES)
        orc.set_blinn_phong(True)
    ref, _, total = orc.render(wl.method, wl.cam, wl.light, wl.params, 96, 96, precision=64)
    frac, mx, psnr = flip_stats(img, ref)
    print(f"iso {label}: {frac * 100:.3f} % of pixels beyond 1/255 (max {mx:.3e}), PSNR {psnr:.1f} dB, "
          f"samples {st.samples} vs {total}")
    assert np.isfinite(img).all()
    # 8-bit texture weights move more crossings (measured on GB300: 0.29 % of the
    # pixels flip, PSNR 28.8 dB, every flip a full hit/miss difference)
    limit = 0.02 if sampling else 0.002
    assert frac <= limit, frac
    assert psnr >= (25.0 if sampling else 40.0), psnr
    if not sampling:
        assert abs(int(st.samples) - int(total)) <= max(8, total // 500)


@pytest.mark.gpu
def test_iso_needs_no_transfer_function(lib):
    ctx = scene.Context(0)
    try:
        vol = scene.synth_blobs(24, 24, 24, abi.CVR_U8, 4, seed=3)
        ctx.set_volume(vol, (1.0, 1.0, 1.0))
        cam = scene.camera(scene.orbit_eye(80.0, 20.0, 10.0))
        img, st = ctx.render(abi.ISO, cam, None, scene.iso_params(), 32, 32)
        assert img[..., 3].max() == 1.0 and st.shaded_samples > 0
        bad = scene.iso_params(large=0.0)
        with pytest.raises(abi.CvrError):
            ctx.render(abi.ISO, cam, None, bad, 32, 32)
    finally:
        ctx.close()
