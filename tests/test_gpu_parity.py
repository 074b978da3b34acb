"""GPU parity: every CUDA path through the C ABI against the CPU oracle.

Tolerances (stated by the specification of this project): images within
max per-channel |error| <= 1/255 and PSNR >= 50 dB of the FP64 oracle; the
extinction SAT bit-exact against the oracle's integer SAT and within relative
error 1e-5 of the reference's FP64 builder; pyramid levels within 1e-4
relative (FP32 sums of 343 taps).
"""
import math

import numpy as np
import pytest

import oracle
from cpp_volume_rendering_gb300 import abi, scene

pytestmark = pytest.mark.gpu

MAX_ABS = 1.0 / 255.0
MIN_PSNR = 50.0


def psnr(a, b):
    mse = float(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2))
    return float("inf") if mse == 0 else 10.0 * math.log10(1.0 / mse)


def compare(img_gpu, img_ref, what):
    err = np.abs(img_gpu.astype(np.float64) - img_ref)
    p = psnr(img_gpu, img_ref)
    assert np.isfinite(img_gpu).all(), f"{what}: non-finite pixels"
    assert err.max() <= MAX_ABS, f"{what}: max abs {err.max():.3e} at {np.unravel_index(err.argmax(), err.shape)}"
    assert p >= MIN_PSNR, f"{what}: PSNR {p:.1f} dB"
    return err.max(), p


def run_both(ctx, wl, rows=None):
    scene.prepare(ctx, wl)
    img, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    ref, counts, total = orc.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height, precision=64,
                                    rows=rows)
    if rows:
        img = img[rows[0]:rows[1]]
    return img, st, ref, total


@pytest.mark.parametrize("name,n,image", [("plain", 64, 256), ("plain", 33, 61), ("extinction", 40, 96),
                                          ("cone", 40, 80), ("ground_truth", 32, 64)])
def test_workload_parity(ctx, name, n, image):
    wl = scene.workload(name, n=n, image=image)
    img, st, ref, total = run_both(ctx, wl)
    compare(img, ref, f"{name} n={n}")
    # the primary-ray step count is the Msamples numerator: GPU and oracle must agree
    assert abs(int(st.samples) - int(total)) <= max(2, total // 2000), (st.samples, total)


def test_plain_full_config_parity(ctx):
    """The plain workload at its benchmark size (64^3 -> 256^2) in full."""
    wl = scene.workload("plain")
    img, st, ref, total = run_both(ctx, wl)
    compare(img, ref, "plain 64^3 256^2")


def test_extinction_u8_point_light_and_shells(ctx):
    """u8 volume, point-light shadow (TypeOfShadow 0), the reference's
    uniform AO shells (radius R*(i+1), K = 5)."""
    vol = scene.synth_blobs(36, 30, 28, abi.CVR_U8, 6, seed=11)
    wl = scene.workload("extinction", n=8, image=8)
    wl.volume = vol
    lp = (50.0, 70.0, -40.0)
    wl.light = scene.light(abi.LIGHT_POINT, position=lp)
    wl.params = scene.ext_params(scene.default_step(wl.spacing), wl.diagonal, ao_radii=(1, 2, 3, 4, 5),
                                 shadow_type=0)
    wl.cam = scene.camera(scene.orbit_eye(110.0, 200.0, -30.0), fovy=35.0)
    wl.width, wl.height = 72, 56
    img, st, ref, total = run_both(ctx, wl)
    compare(img, ref, "extinction u8 point light")


def test_extinction_anisotropic_spacing_and_aspect(ctx):
    vol = scene.synth_value_noise(40, 24, 32, abi.CVR_U16, seed=9)
    wl = scene.workload("extinction", n=8, image=8)
    wl.volume = vol
    wl.spacing = (1.0, 1.5, 0.75)
    wl.params = scene.ext_params(scene.default_step(wl.spacing), wl.diagonal, ao_radii=(2, 4))
    wl.cam = scene.camera(scene.orbit_eye(120.0, 60.0, 35.0), fovy=40.0)
    wl.width, wl.height = 80, 48
    img, st, ref, total = run_both(ctx, wl)
    compare(img, ref, "extinction anisotropic")


@pytest.mark.parametrize("dtype", [abi.CVR_U8, abi.CVR_U16])
def test_quad_layout_is_bit_identical_on_ragged_volumes(ctx, dtype):
    """The x-y quad copies of the volume and of the pyramid (successors
    clamped at the high faces, texel coordinates raised to 0 at the low faces)
    render the plain layout's bits on odd, non-cubic volumes with anisotropic
    spacing, rays entering through every face."""
    vol = scene.synth_value_noise(37, 23, 29, dtype, seed=12)
    for name in ("plain", "ground_truth", "iso", "cone"):
        wl = scene.workload(name, n=8, image=8)
        wl.volume = vol
        wl.spacing = (1.0, 1.5, 0.75)
        wl.width, wl.height = 64, 48
        if name == "cone":  # a ragged pyramid: its quad copy is read as well
            wl.pyramid = dict(base_dims=(19, 12, 15), sigma0=1.0, n_levels=4)
        scene.prepare(ctx, wl)
        for eye in ((120.0, 60.0, 35.0), (120.0, -150.0, -40.0)):
            wl.cam = scene.camera(scene.orbit_eye(*eye), fovy=40.0)
            abi.check(ctx.lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_PLAIN), ctx.h)
            a, _ = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
            abi.check(ctx.lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_QUADS), ctx.h)
            try:
                b, _ = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
            finally:
                abi.check(ctx.lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_PLAIN), ctx.h)
            assert np.array_equal(a, b), (name, eye)
            assert np.abs(a).max() > 0


def test_sat_bit_exact_and_relative_error(ctx):
    vol = scene.synth_value_noise(48, 40, 36, abi.CVR_U16, seed=4)
    ext = scene.BENCH_TF.ext_per_value(abi.CVR_U16)
    ctx.set_volume(vol, (1.0, 1.0, 1.0))
    ctx.set_transfer_function(scene.BENCH_TF)
    ctx.build_sat(ext)
    sat, F = ctx.sat()
    q = np.floor(ext * 2.0 ** F + 0.5).astype(np.int64)
    assert np.array_equal(sat, oracle.sat_i64(vol, q))
    orc = oracle.Oracle()
    orc.set_volume(vol, (1, 1, 1))
    orc.build_sat(ext)
    ref = orc.sat()
    got = sat.astype(np.float64) * 2.0 ** -F
    big = ref > 1e-3 * ref.max()
    rel = np.abs(got - ref)[big] / ref[big]
    assert rel.max() <= 1e-5, rel.max()
    assert np.abs(got - ref).max() / ref.max() <= 1e-9


def test_int64_sat_is_built_when_first_read(ctx):
    # cvr_build_sat defers the int64 table: a frame the compact table serves
    # does not build it, a later download does, from the latest table; a
    # volume upload drops the pending build with the table
    wl = scene.workload("extinction", n=40, image=48)
    scene.prepare(ctx, wl)
    ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
    ext = wl.tf.ext_per_value(wl.dtype)
    ctx.build_sat(ext * 0.5)
    ctx.build_sat(ext)
    ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
    sat, F = ctx.sat()
    q = np.floor(ext * 2.0 ** F + 0.5).astype(np.int64)
    assert np.array_equal(sat, oracle.sat_i64(wl.volume, q))
    ctx.set_volume(wl.volume, wl.spacing)
    with pytest.raises(abi.CvrError):
        ctx.sat()
    assert ctx.lib.cvr_prepare_sat(ctx.h) == abi.CVR_OK


# (volume dims, base dims, sigma0): the reference geometry (base = half the
# volume, S0 = 1 voxel), where every level has the separable form; an odd
# volume over a half base (separable, odd-sized lattices); a base that does
# not divide the volume and a non-integer sigma (the direct 343-tap kernels);
# a flat base whose levels collapse to 1 cell on one axis
@pytest.mark.parametrize("dims,base,s0", [((32, 32, 32), (16, 16, 16), 1.0), ((30, 22, 26), (15, 11, 13), 1.0),
                                          ((32, 24, 20), (12, 9, 7), 1.0), ((32, 32, 32), (16, 16, 16), 1.5),
                                          ((40, 8, 24), (20, 4, 12), 2.0)])
def test_pyramid_levels_match_oracle(ctx, dims, base, s0):
    wl = scene.workload("cone", n=32, image=8)
    w, h, d = dims
    wl.volume = scene.synth_blobs(w, h, d, abi.CVR_U8, 8, seed=31, noise_max=20.0)
    wl.pyramid = dict(base_dims=base, sigma0=s0, n_levels=5)
    scene.prepare(ctx, wl)
    levels = ctx.pyramid()
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    assert len(levels) == orc.n_levels
    for l, lev in enumerate(levels):
        ref = orc.pyramid_level(l, 64)
        assert lev.shape == ref.shape
        err = np.abs(lev - ref) / np.maximum(np.abs(ref), 1e-3)
        assert err.max() <= 1e-4, (l, err.max())


def test_rays_missing_the_volume_are_zero(ctx):
    wl = scene.workload("plain", n=16, image=32)
    # camera beside the volume looking parallel to it: every slab test fails
    wl.cam = scene.camera((3.0, 0.0, 0.0), center=(3.0, 0.0, 5.0), fovy=10.0)
    scene.prepare(ctx, wl)
    img, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, 32, 32)
    assert (img == 0).all() and st.samples == 0


def test_box_behind_camera_matches_reference_quirk(ctx):
    """RayAABBIntersection tests tfar > tnear before clamping tnear to 0
    (ray_bbox_intersection.comp:44-46), so a box entirely behind the camera
    counts as hit and the ray marches |tfar| forward through clamp-to-edge
    samples.  The GPU path keeps that behaviour; it must agree with the oracle."""
    wl = scene.workload("plain", n=16, image=32)
    wl.cam = scene.camera((0.0, 0.0, 3.0), center=(0.0, 0.0, 6.0))  # looking away
    img, st, ref, total = run_both(ctx, wl)
    compare(img, ref, "box behind camera")
    assert st.samples == total > 0


def test_camera_inside_volume_and_tiny_images(ctx):
    wl = scene.workload("plain", n=24, image=8)
    wl.cam = scene.camera((0.05, -0.1, 0.12), center=(0.4, 0.3, -0.2), fovy=70.0)
    for w, h in [(1, 1), (7, 3), (37, 23)]:
        wl.width, wl.height = w, h
        img, st, ref, total = run_both(ctx, wl)
        compare(img, ref, f"inside camera {w}x{h}")


def test_single_voxel_and_flat_volumes(ctx):
    for shape in [(1, 1, 1), (1, 9, 13), (17, 1, 5)]:
        vol = (np.arange(np.prod(shape)) * 37 % 256).astype(np.uint8).reshape(shape)
        wl = scene.workload("plain", n=4, image=8)
        wl.volume = vol
        wl.spacing = (0.1, 0.1, 0.1)
        wl.params.step_size = 0.05
        wl.cam = scene.camera((1.0, 0.7, 2.0), fovy=30.0)
        wl.width, wl.height = 24, 24
        img, st, ref, total = run_both(ctx, wl)
        compare(img, ref, f"volume {shape}")


def test_errors_are_reported_not_crashing(ctx):
    import ctypes as C
    lib = abi.load()
    img = np.zeros((4, 4, 4), np.float32)
    p = abi.PlainParams()
    p.step_size = 0.0
    cam = scene.camera((0, 0, 3))
    scene.prepare(ctx, scene.workload("plain", n=8, image=4))
    r = lib.cvr_render_host(ctx.h, abi.PLAIN, C.byref(cam), None, C.byref(p), C.sizeof(p), abi.fptr(img), 4, 4, None)
    assert r == abi.CVR_ERR_INVALID_ARG
    p.step_size = 0.01
    r = lib.cvr_render_host(ctx.h, 99, C.byref(cam), None, C.byref(p), C.sizeof(p), abi.fptr(img), 4, 4, None)
    assert r == abi.CVR_ERR_INVALID_ARG
    # method tables missing -> NOT_READY, context stays usable
    fresh = scene.Context(0)
    fresh.set_volume(np.zeros((4, 4, 4), np.uint8))
    fresh.set_transfer_function(scene.BENCH_TF)
    ep = scene.ext_params(0.5, 7.0)
    r = lib.cvr_render_host(fresh.h, abi.EXTINCTION, C.byref(cam), None, C.byref(ep), C.sizeof(ep), abi.fptr(img),
                            4, 4, None)
    assert r == abi.CVR_ERR_NOT_READY
    r = lib.cvr_render_host(fresh.h, abi.PLAIN, C.byref(cam), None, C.byref(p), C.sizeof(p), abi.fptr(img), 4, 4, None)
    assert r == abi.CVR_OK
    fresh.close()
    empty = scene.Context(0)
    r = lib.cvr_render_host(empty.h, abi.PLAIN, C.byref(cam), None, C.byref(p), C.sizeof(p), abi.fptr(img), 4, 4, None)
    assert r == abi.CVR_ERR_NO_VOLUME
    empty.close()


@pytest.mark.parametrize("name,n,image", [("plain", 64, 128), ("extinction", 40, 96), ("cone", 40, 80),
                                          ("ground_truth", 32, 64)])
def test_texture_variant_parity(ctx, name, n, image):
    """The hardware-texture variant of the volume samples (8-bit filter
    weights) stays within 1/255 max-abs of the FP64 oracle, PSNR >= 45 dB;
    for the cone method 2/255: a ray whose opacity crosses the 0.99 cut one
    step earlier or later moves its pixel by up to 1% of its colour."""
    wl = scene.workload(name, n=n, image=image)
    ctx.set_sampling(abi.SAMPLING_TEX_FEATURES | abi.SAMPLING_TEX_VOLUME)
    try:
        img, st, ref, total = run_both(ctx, wl)
    finally:
        ctx.set_sampling(abi.SAMPLING_TEX_FEATURES)
    err = np.abs(img.astype(np.float64) - ref)
    p = psnr(img, ref)
    print(f"texture variant {name}: max abs {err.max():.2e}, PSNR {p:.1f} dB, samples {st.samples} vs {total}")
    assert np.isfinite(img).all()
    assert err.max() <= (2.0 / 255.0 if name == "cone" else MAX_ABS), err.max()
    assert p >= 45.0, p


@pytest.mark.parametrize("flags", [abi.SAMPLING_TEX_PYRAMID,
                                   abi.SAMPLING_TEX_PYRAMID | abi.SAMPLING_TEX_VOLUME | abi.SAMPLING_TEX_FEATURES])
def test_cone_texture_pyramid(ctx, flags):
    """The cone method's pyramid taps through the texture unit (FP16 levels,
    8-bit filter weights: the reference's own R16F / GL_LINEAR_MIPMAP_LINEAR
    sampling) against the FP64 oracle of the exact FP32 levels."""
    wl = scene.workload("cone", n=40, image=80)
    ctx.set_sampling(flags)
    try:
        img, st, ref, total = run_both(ctx, wl)
    finally:
        ctx.set_sampling(abi.SAMPLING_TEX_FEATURES)
    err = np.abs(img.astype(np.float64) - ref)
    p = psnr(img, ref)
    print(f"cone texture pyramid flags {flags}: max abs {err.max():.2e}, PSNR {p:.1f} dB")
    # measured on GB300: 2.7e-4 / 95 dB with the pyramid taps alone, 6.7e-3 / 83 dB
    # with the volume samples through the texture unit too (early-termination flips)
    assert np.isfinite(img).all()
    assert err.max() <= (MAX_ABS if flags == abi.SAMPLING_TEX_PYRAMID else 2.0 / 255.0), err.max()
    assert p >= 60.0, p


TILES = [(8, 8), (16, 8), (32, 4), (8, 16), (32, 8), (16, 16)]


@pytest.mark.parametrize("name,n,image", [("extinction", 48, 72), ("plain", 40, 56), ("cone", 40, 48),
                                          ("ground_truth", 24, 40), ("iso", 40, 48)])
def test_tuning_does_not_change_results(ctx, name, n, image):
    """Every tile shape / register variant / brick size renders the same bits."""
    import ctypes as C
    lib = abi.load()
    wl = scene.workload(name, n=n, image=image)
    scene.prepare(ctx, wl)
    images = []
    for tw, th in TILES:
        for v in ((0, 1, 2, 3) if name == "extinction" else ((0, 1, 2) if name == "cone" else (0,))):
            abi.check(lib.cvr_set_tuning(ctx.h, tw, th, v), ctx.h)
            img, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
            images.append(img)
    abi.check(lib.cvr_set_tuning(ctx.h, 16, 8, 0), ctx.h)
    for edge in (4, 8, 16, 32):
        abi.check(lib.cvr_set_brick_size(ctx.h, edge), ctx.h)
        assert lib.cvr_get_brick_size(ctx.h) == edge
        img, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
        images.append(img)
    abi.check(lib.cvr_set_brick_size(ctx.h, 0), ctx.h)
    abi.check(lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_QUADS), ctx.h)
    assert lib.cvr_get_volume_layout(ctx.h) == abi.LAYOUT_QUADS
    for tw, th in ((16, 8), (32, 8)):
        abi.check(lib.cvr_set_tuning(ctx.h, tw, th, 0), ctx.h)
        img, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
        images.append(img)
    abi.check(lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_PLAIN), ctx.h)
    for tw, th, ww in ((16, 8, 4), (16, 8, 16), (32, 4, 16), (8, 16, 4)):
        abi.check(lib.cvr_set_tuning(ctx.h, tw, th, 0), ctx.h)
        abi.check(lib.cvr_set_warp_shape(ctx.h, ww), ctx.h)
        img, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
        images.append(img)
    abi.check(lib.cvr_set_warp_shape(ctx.h, 8), ctx.h)
    abi.check(lib.cvr_set_tuning(ctx.h, 16, 8, 0), ctx.h)
    for k, im in enumerate(images[1:]):
        assert np.array_equal(im, images[0]), k + 1
    # the persistent ray-refill marchers (plain, extinction, cone, ground truth;
    # the iso caster keeps its tiles), every register variant, both layouts:
    # the same per-ray arithmetic in another kernel, where the compiler may
    # fuse a multiply-add differently, so equal to a few ulps, and within the
    # parity bar of the oracle
    refill = []
    for quads in (abi.LAYOUT_PLAIN, abi.LAYOUT_QUADS):
        abi.check(lib.cvr_set_volume_layout(ctx.h, quads), ctx.h)
        for v in (0, 1, 2):
            abi.check(lib.cvr_set_tuning(ctx.h, 16, 8, v), ctx.h)
            abi.check(lib.cvr_set_ray_refill(ctx.h, 1), ctx.h)
            assert lib.cvr_get_ray_refill(ctx.h) == 1
            img, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
            refill.append(img)
    abi.check(lib.cvr_set_ray_refill(ctx.h, 0), ctx.h)
    abi.check(lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_PLAIN), ctx.h)
    abi.check(lib.cvr_set_tuning(ctx.h, 16, 8, 0), ctx.h)
    if name == "plain":  # shared-memory brick staging (plain layout)
        abi.check(lib.cvr_set_brick_staging(ctx.h, 1), ctx.h)
        assert lib.cvr_get_brick_staging(ctx.h) == 1
        img, st = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
        refill.append(img)
        abi.check(lib.cvr_set_brick_staging(ctx.h, 0), ctx.h)
    for k, im in enumerate(refill):
        d = float(np.abs(im - images[0]).max())
        assert d <= 1e-5, (k, d)
    if name != "iso":
        orc = oracle.Oracle()
        oracle.prepare(orc, wl)
        ref, _, _ = orc.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height, precision=64)
        compare(refill[0], ref, f"{name} ray refill")
    assert lib.cvr_set_tuning(ctx.h, 24, 8, 0) == abi.CVR_ERR_INVALID_ARG  # 6 warps
    assert lib.cvr_set_tuning(ctx.h, 12, 8, 0) == abi.CVR_ERR_INVALID_ARG  # not whole warps
    assert lib.cvr_set_brick_size(ctx.h, 12) == abi.CVR_ERR_INVALID_ARG
    assert lib.cvr_set_volume_layout(ctx.h, 2) == abi.CVR_ERR_INVALID_ARG
    assert lib.cvr_set_warp_shape(ctx.h, 32) == abi.CVR_ERR_INVALID_ARG


def test_autotune_picks_a_valid_configuration(ctx):
    import ctypes as C
    lib = abi.load()
    wl = scene.workload("extinction", n=48, image=72)
    scene.prepare(ctx, wl)
    tw, th, v = C.c_int(), C.c_int(), C.c_int()
    ms = C.c_float()
    abi.check(lib.cvr_autotune(ctx.h, wl.method, C.byref(wl.cam), C.byref(wl.light), C.byref(wl.params),
                               C.sizeof(wl.params), wl.width, wl.height, 2, C.byref(tw), C.byref(th), C.byref(v),
                               C.byref(ms)), ctx.h)
    assert (tw.value, th.value) in TILES and v.value in (0, 1, 2) and ms.value > 0
    assert lib.cvr_get_brick_size(ctx.h) in (0, 8, 16, 32)
    assert lib.cvr_get_volume_layout(ctx.h) in (abi.LAYOUT_PLAIN, abi.LAYOUT_QUADS)
    assert lib.cvr_get_warp_shape(ctx.h) in (4, 8, 16)
    img, _ = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
    abi.check(lib.cvr_set_tuning(ctx.h, 16, 8, 0), ctx.h)
    abi.check(lib.cvr_set_brick_size(ctx.h, 0), ctx.h)
    abi.check(lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_PLAIN), ctx.h)
    abi.check(lib.cvr_set_warp_shape(ctx.h, 8), ctx.h)
    ref, _ = ctx.render(wl.method, wl.cam, wl.light, wl.params, wl.width, wl.height)
    assert np.array_equal(img, ref)


def test_directional_shadow_table_matches_per_sample_geometry(ctx):
    """The per-frame box table of a directional light equals the per-sample
    cone walk: render the same light once as directional (table) and compare
    with the oracle, which walks the cone per sample."""
    wl = scene.workload("extinction", n=40, image=64)
    for fwd in [(0.2, 0.3, 0.93), (-0.8, 0.1, 0.3), (0.1, -0.95, -0.2), (0.5, 0.5, 0.5)]:
        f, u, r = scene.light_frame(fwd)
        wl.light = scene.light(abi.LIGHT_DIRECTIONAL, forward=f, up=u, right=r)
        img, st, ref, total = run_both(ctx, wl)
        compare(img, ref, f"directional light {fwd}")
