"""Object-space light cache (PreIlluminationStructuredVolume): the cache
kernels and the object-space marcher against the oracle's restatement of
lightcachecomputation.comp + obj_ray_marching.comp; same bar as the other
renderers (max |error| <= 1/255, PSNR >= 50 dB)."""
import numpy as np
import pytest

import oracle
from cpp_volume_rendering_gb300 import abi, scene
from tests.test_gpu_parity import compare

pytestmark = pytest.mark.gpu


def run_cached(ctx, wl, dims):
    scene.prepare(ctx, wl)
    ctx._ck(ctx.lib.cvr_set_light_cache(ctx.h, *dims))
    try:
        img, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
    finally:
        ctx._ck(ctx.lib.cvr_set_light_cache(ctx.h, 0, 0, 0))
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    orc.set_light_cache(*dims)
    ref, _, total = orc.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height, precision=64)
    return img, st, ref, total


@pytest.mark.parametrize("name,n,image,dims,shadow", [("extinction", 40, 64, (32, 32, 32), 1),
                                                      ("extinction", 36, 48, (20, 24, 16), 0),
                                                      ("cone", 40, 64, (32, 32, 32), 0),
                                                      ("cone", 40, 48, (16, 16, 16), 2)])
def test_cached_frames_match_oracle(ctx, name, n, image, dims, shadow):
    wl = scene.workload(name, n=n, image=image)
    if name == "extinction" and shadow == 0:
        f, u, r = scene.light_frame((0.3, 0.8, 0.5))
        wl.light = scene.light(abi.LIGHT_POINT, position=tuple(2.0 * n * np.array(f)), forward=f, up=u, right=r)
    wl.params.shadow_type = shadow
    if name == "cone" and shadow == 2:
        f, u, r = scene.light_frame((0.2, 0.9, -0.3))
        wl.light = scene.light(abi.LIGHT_DIRECTIONAL, forward=f, up=u, right=r)
    img, st, ref, total = run_cached(ctx, wl, dims)
    compare(img, ref, f"{name} cached {dims} shadow {shadow}")
    assert abs(int(st.samples) - int(total)) <= max(2, total // 2000)


def test_cache_contents_and_no_terms_quirk(ctx):
    wl = scene.workload("extinction", n=32, image=32)
    scene.prepare(ctx, wl)
    ctx._ck(ctx.lib.cvr_set_light_cache(ctx.h, 8, 8, 8))
    try:
        img, _ = ctx.render(wl.method, wl.cam, wl.light, wl.params, 32, 32)
        cache = np.zeros(8 * 8 * 8 * 2, np.float32)
        ctx._ck(ctx.lib.cvr_download_light_cache(ctx.h, abi.fptr(cache), cache.size))
        assert (cache >= 0).all() and (cache <= 1.0 + 1e-6).all() and cache.min() < 1.0
        # obj_ray_marching.comp composites only shaded samples: with both terms off the frame is empty
        wl.params.apply_occlusion = 0
        wl.params.apply_shadow = 0
        empty, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, 32, 32)
        assert st.samples > 0 and not empty.any()
    finally:
        ctx._ck(ctx.lib.cvr_set_light_cache(ctx.h, 0, 0, 0))
    assert ctx.lib.cvr_set_light_cache(ctx.h, 4, 0, 4) == abi.CVR_ERR_INVALID_ARG
