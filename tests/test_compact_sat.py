"""The compact 32-bit SAT (wrapped prefix sums of per-frame fixed point):
frames that use it and frames that keep the int64 table both meet the
renderers' bar against the FP64 oracle (max |error| <= 1/255, PSNR >= 50 dB)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from cpp_volume_rendering_gb300 import abi, scene
from tests.test_gpu_parity import compare

pytestmark = pytest.mark.gpu


# (AO radii, shadow type, cone angle, sample interval): directional lights use
# the per-frame box table; point lights the per-sample cone bound (a 0.7 rad
# cone is unbounded: int64); AO radius 40 exceeds the compact table's
# resolution floor (int64).  Integer box widths everywhere (radii 2, 6, 16;
# 1, 3; interval 2) take the equal-fraction query; radii 2.3, 5.1 (widths
# 4.6, 10.2) or a 1.5-voxel interval take the general compact query.
@pytest.mark.parametrize("radii,shadow_type,angle,interval",
                         [((2, 6, 16), 1, None, 2.0), ((1, 3), 1, None, 2.0), ((3, 9, 40), 1, None, 2.0),
                          ((2, 6), 0, None, 2.0), ((2, 6), 0, 0.7, 2.0), ((2.3, 5.1), 1, None, 2.0),
                          ((2, 6, 16), 1, None, 1.5), ((2.5, 7.5), 1, 0.05, 3.0)])
def test_compact_and_int64_frames_match_oracle(ctx, radii, shadow_type, angle, interval):
    wl = scene.workload("extinction", n=48, image=80)
    wl.params = scene.ext_params(scene.default_step(wl.spacing), wl.diagonal, ao_radii=radii, shadow_type=shadow_type,
                                 interval=interval)
    if angle is not None:
        wl.params.sdw_cone_angle_rad = angle
    if shadow_type == 0:
        f, u, r = scene.light_frame((0.3, 0.8, 0.5))
        wl.light = scene.light(abi.LIGHT_POINT, position=tuple(100.0 * np.array(f)), forward=f, up=u, right=r)
    scene.prepare(ctx, wl)
    imgs = {}
    for on in (1, 0):
        abi.check(ctx.lib.cvr_set_compact_sat(ctx.h, on), ctx.h)
        imgs[on], _ = ctx.render(wl.method, wl.cam, wl.light, wl.params, 80, 80)
    abi.check(ctx.lib.cvr_set_compact_sat(ctx.h, 1), ctx.h)
    assert ctx.lib.cvr_get_compact_sat(ctx.h) == 1
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    ref, _, _ = orc.render(wl.method, wl.cam, wl.light, wl.params, 80, 80, precision=64)
    for on in (1, 0):
        compare(imgs[on], ref, f"extinction radii {radii} shadow {shadow_type} compact {on}")
    assert np.abs(imgs[1] - imgs[0]).max() <= 1.0 / 255.0


def test_compact_table_follows_the_volume(ctx):
    """A new volume (and a new SAT) rebuilds the compact table."""
    wl = scene.workload("extinction", n=40, image=48)
    scene.prepare(ctx, wl)
    a, _ = ctx.render(wl.method, wl.cam, wl.light, wl.params, 48, 48)
    wl2 = scene.workload("extinction", n=40, image=48)
    wl2.volume = scene.synth_value_noise(40, 40, 40, abi.CVR_U16, seed=77)
    scene.prepare(ctx, wl2)
    b, _ = ctx.render(wl2.method, wl2.cam, wl2.light, wl2.params, 48, 48)
    orc = oracle.Oracle()
    oracle.prepare(orc, wl2)
    ref, _, _ = orc.render(wl2.method, wl2.cam, wl2.light, wl2.params, 48, 48, precision=64)
    compare(b, ref, "extinction after a volume change")
    assert not np.array_equal(a, b)


# directional lights whose walk runs along x, y or z, either way
@pytest.mark.parametrize("direction", [(0.9, 0.3, 0.2), (-0.2, 0.85, 0.3), (0.25, -0.3, -0.9), (-0.8, -0.4, 0.3)])
def test_walk_tables_equal_quads_and_match_oracle(ctx, direction):
    """Shadow boxes read from the walk table (sums differenced along the walk
    axis) give the bits of the quad-table query, and the oracle's image."""
    wl = scene.workload("extinction", n=44, image=72)
    f, u, r = scene.light_frame(direction)
    wl.light = scene.light(abi.LIGHT_DIRECTIONAL, position=tuple(130.0 * np.array(f)), forward=f, up=u, right=r)
    scene.prepare(ctx, wl)
    imgs = {}
    for on in (1, 0):
        abi.check(ctx.lib.cvr_set_walk_tables(ctx.h, on), ctx.h)
        assert ctx.lib.cvr_get_walk_tables(ctx.h) == on
        imgs[on], _ = ctx.render(wl.method, wl.cam, wl.light, wl.params, 72, 72)
    abi.check(ctx.lib.cvr_set_walk_tables(ctx.h, 1), ctx.h)
    assert np.array_equal(imgs[1], imgs[0])
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    ref, _, _ = orc.render(wl.method, wl.cam, wl.light, wl.params, 72, 72, precision=64)
    compare(imgs[1], ref, f"extinction walk table, light {direction}")
