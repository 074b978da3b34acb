"""GPU parity at the benchmarked sizes: the full frame is rendered on the GPU
(autotuned, as bench.py renders it) and a band of rows through the densest
part of the image is compared with the FP64 oracle.

  * extinction: 256^3 u16 value-noise shells -> 1024^2, AO radii {2, 6, 16} +
    directional SAT cone shadow (the headline configuration);
  * ground truth and cone DOS: 256^3 u8 blobs + noise -> 512^2;
  * surrogate: the held-out 512^3 u8 blob volume -> 1024^2 with a seeded
    network (the frame's arithmetic, not the training, is under test).

Bar: max per-channel |error| <= 1/255 and PSNR >= 50 dB (texture-unit
sampling of the surrogate's inputs: <= 8/255 and >= 40 dB), and the band's
primary step count within 1/2000 of the oracle's.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from cpp_volume_rendering_gb300 import abi, scene
from tests.test_gpu_parity import psnr

pytestmark = pytest.mark.gpu


def autotune(ctx, wl):
    tw, th, tv, ms = C.c_int(), C.c_int(), C.c_int(), C.c_float()
    abi.check(ctx.lib.cvr_autotune(ctx.h, wl.method, C.byref(wl.cam), C.byref(wl.light), C.byref(wl.params),
                                   C.sizeof(wl.params), wl.width, wl.height, 1, C.byref(tw), C.byref(th),
                                   C.byref(tv), C.byref(ms)), ctx.h)


def reset(ctx):
    abi.check(ctx.lib.cvr_set_tuning(ctx.h, 16, 8, 0), ctx.h)
    abi.check(ctx.lib.cvr_set_brick_size(ctx.h, 0), ctx.h)
    abi.check(ctx.lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_PLAIN), ctx.h)
    abi.check(ctx.lib.cvr_set_warp_shape(ctx.h, 8), ctx.h)
    abi.check(ctx.lib.cvr_set_ray_refill(ctx.h, 0), ctx.h)
    ctx.set_sampling(abi.SAMPLING_TEX_FEATURES)


def render_with_oracle(ctx, wl, tuned=True, prepared=False):
    """GPU frame (autotuned unless told otherwise) + its per-pixel step counts,
    and an oracle prepared with the same workload."""
    if not prepared:
        scene.prepare(ctx, wl)
    if tuned:
        autotune(ctx, wl)
    img, _ = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
    counts = np.zeros((wl.height, wl.width), np.uint32)
    _render_counts(ctx, wl, counts)
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    return orc, img, counts


def _render_counts(ctx, wl, counts):
    """The same frame with per-pixel primary step counts (device buffers)."""
    out = C.POINTER(C.c_float)()
    abi.check(ctx.lib.cvr_get_frame_buffer(ctx.h, wl.width, wl.height, C.byref(out)), ctx.h)
    from tests.devmem import DeviceMemory
    mem = DeviceMemory()
    try:
        dc = mem.alloc(counts.nbytes, fill=0)
        abi.check(ctx.lib.cvr_render(ctx.h, wl.method, C.byref(wl.cam), C.byref(wl.light), C.byref(wl.params),
                                     C.sizeof(wl.params), C.cast(out, C.c_void_p), wl.width, wl.height, dc, None),
                  ctx.h)
        abi.check(ctx.lib.cvr_sync(ctx.h), ctx.h)
        counts[:] = mem.download(dc, counts.shape, np.uint32)
    finally:
        mem.close()


def check_bands(orc, wl, img, counts, bands, what, max_abs=1.0 / 255.0, min_psnr=50.0):
    checked = 0
    for y0, y1 in bands:
        ref, ref_counts, _ = orc.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height, precision=64,
                                        rows=(y0, y1))
        band = img[y0:y1]
        err = np.abs(band.astype(np.float64) - ref)
        assert np.isfinite(band).all(), f"{what} rows {y0}..{y1}: non-finite pixels"
        assert err.max() <= max_abs, f"{what} rows {y0}..{y1}: max abs {err.max():.3e}"
        assert psnr(band, ref) >= min_psnr, f"{what} rows {y0}..{y1}: PSNR {psnr(band, ref):.1f} dB"
        # the Msamples numerator: the band's primary step count (single vs double
        # precision may move an early-termination step)
        got, want = int(counts[y0:y1].astype(np.int64).sum()), int(ref_counts.astype(np.int64).sum())
        assert abs(got - want) <= max(2, want // 2000), (got, want)
        checked += int((ref[..., 3] > 0).sum())
    assert checked > 0, f"{what}: the bands hit no volume"


def test_extinction_headline_config_bands(ctx):
    reset(ctx)
    wl = scene.workload("extinction")
    assert wl.dims == (256, 256, 256) and (wl.width, wl.height) == (1024, 1024)
    orc, img, counts = render_with_oracle(ctx, wl)
    check_bands(orc, wl, img, counts, [(504, 520), (300, 304), (760, 764)], "extinction 256^3 -> 1024^2")
    reset(ctx)


@pytest.mark.parametrize("name", ["ground_truth", "cone"])
def test_gt_and_cone_config_bands(ctx, name):
    reset(ctx)
    wl = scene.workload(name)
    assert wl.dims == (256, 256, 256) and (wl.width, wl.height) == (512, 512)
    orc, img, counts = render_with_oracle(ctx, wl)
    check_bands(orc, wl, img, counts, [(250, 258), (150, 152), (380, 382)], f"{name} 256^3 -> 512^2")
    reset(ctx)


@pytest.mark.parametrize("sampling", [0, abi.SAMPLING_TEX_FEATURES])
def test_surrogate_heldout_config_bands(ctx, sampling):
    """The surrogate-shaded frame of the held-out 512^3 volume at 1024^2 with a
    seeded network whose outputs span [0, 1], against the oracle's FP64
    restatement of the same frame (BF16 operands, exact accumulation)."""
    reset(ctx)
    wl = scene.workload("surrogate")
    assert wl.dims == (512, 512, 512) and (wl.width, wl.height) == (1024, 1024)
    scene.prepare(ctx, wl)
    ctx.mlp_init(11)
    p = ctx.mlp_params()
    p[abi.MLP_PARAMS - 2:] = 0.5
    p[64 * 48 + 64 + 64 * 64 + 64:abi.MLP_PARAMS - 2] *= 0.05
    ctx.mlp_set_params(p)
    ctx.set_sampling(sampling)
    orc, img, counts = render_with_oracle(ctx, wl, tuned=False, prepared=True)
    orc.set_mlp(p)
    tol = (1.0 / 255.0, 50.0) if sampling == 0 else (8.0 / 255.0, 40.0)
    check_bands(orc, wl, img, counts, [(508, 516), (330, 332)], f"surrogate 512^3 -> 1024^2 sampling {sampling}",
                max_abs=tol[0], min_psnr=tol[1])
    reset(ctx)
