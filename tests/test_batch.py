"""Batched rendering: resident volume slots and one graph-captured persistent
launch per method over many (volume, view, light) jobs.  Every image of a
batch must equal, bit for bit, the same job rendered alone by cvr_render with
the same tile configuration, and replays must repeat it."""
import ctypes as C

import numpy as np
import pytest

from cpp_volume_rendering_gb300 import abi, scene
from tests.devmem import DeviceMemory

pytestmark = pytest.mark.gpu


def small_network(ctx):
    ctx.mlp_init(5)
    p = ctx.mlp_params()
    p[abi.MLP_PARAMS - 2:] = 0.5
    p[64 * 48 + 64 + 64 * 64 + 64:abi.MLP_PARAMS - 2] *= 0.05
    ctx.mlp_set_params(p)


def test_volume_slots_keep_their_tables(ctx):
    a = scene.synth_blobs(24, 24, 24, abi.CVR_U8, 8, seed=5100)
    b = scene.synth_value_noise(20, 28, 16, abi.CVR_U16, seed=5101)
    wl_a = scene.workload("extinction", n=24, image=32)
    ctx.select_volume(3)
    assert ctx.lib.cvr_current_volume(ctx.h) == 3
    ctx.set_volume(a)
    ctx.set_transfer_function(scene.BENCH_TF)
    ctx.build_sat(scene.BENCH_TF.ext_per_value(abi.CVR_U8))
    img_a, _ = ctx.render(abi.EXTINCTION, wl_a.cam, wl_a.light, wl_a.params, 32, 32)
    ctx.select_volume(5)
    ctx.set_volume(b)
    ctx.build_sat(scene.BENCH_TF.ext_per_value(abi.CVR_U16))
    img_b, _ = ctx.render(abi.EXTINCTION, wl_a.cam, wl_a.light, wl_a.params, 32, 32)
    ctx.select_volume(3)
    again, _ = ctx.render(abi.EXTINCTION, wl_a.cam, wl_a.light, wl_a.params, 32, 32)
    assert np.array_equal(again, img_a) and not np.array_equal(img_a, img_b)
    assert ctx.lib.cvr_select_volume(ctx.h, abi.MAX_VOLUMES) == abi.CVR_ERR_INVALID_ARG
    ctx.select_volume(0)


@pytest.mark.parametrize("sampling,tile,variant,brick", [(abi.SAMPLING_TEX_FEATURES, (16, 8), 0, 0),
                                                         (0, (16, 8), 0, 0),
                                                         (abi.SAMPLING_TEX_FEATURES, (32, 8), 1, 8),
                                                         (abi.SAMPLING_TEX_FEATURES, (8, 8), 2, 16),
                                                         (abi.SAMPLING_TEX_FEATURES, (16, 8), 0, -1),
                                                         (abi.SAMPLING_TEX_FEATURES, (32, 8), 1, -16)])
def test_batch_equals_single_renders(ctx, sampling, tile, variant, brick):
    """brick -1: the x-y quad volume layout; -16: that layout with warps of
    16x2 pixels."""
    # batches read the int64 SAT; the single renders compared with them do too
    abi.check(ctx.lib.cvr_set_compact_sat(ctx.h, 0), ctx.h)
    ctx.set_sampling(sampling)
    abi.check(ctx.lib.cvr_set_tuning(ctx.h, tile[0], tile[1], variant), ctx.h)
    abi.check(ctx.lib.cvr_set_brick_size(ctx.h, max(brick, 0)), ctx.h)
    abi.check(ctx.lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_QUADS if brick < 0 else abi.LAYOUT_PLAIN), ctx.h)
    abi.check(ctx.lib.cvr_set_warp_shape(ctx.h, 16 if brick == -16 else 8), ctx.h)
    vols = scene.batch_volumes(0.5)  # 64^3 u8, 96x128x80 u16, 128^3 u8, 192^3 u16
    scene.prepare_batch_volumes(ctx, vols)
    small_network(ctx)
    W, H = 48, 40
    mem = DeviceMemory()
    try:
        probe = scene.batch_jobs(vols, n_views=2, lights=scene.BATCH_LIGHTS[:2], image=W)
        n = len(probe.jobs)
        outs = [mem.alloc(W * H * 16, fill=0) for _ in range(n)]
        b = scene.batch_jobs(vols, n_views=2, lights=scene.BATCH_LIGHTS[:2], image=W, out_ptrs=outs)
        for j in b.jobs:
            j.height = H
        arr = (abi.Job * n)(*b.jobs)
        bh = C.c_void_p()
        abi.check(ctx.lib.cvr_batch_create(ctx.h, arr, n, C.byref(bh)), ctx.h)
        try:
            abi.check(ctx.lib.cvr_batch_run(bh), ctx.h)
            abi.check(ctx.lib.cvr_sync(ctx.h), ctx.h)
            first = [mem.download(p, (H, W, 4)) for p in outs]
            stats = []
            for k in range(n):
                st = abi.FrameStats()
                abi.check(ctx.lib.cvr_batch_job_stats(bh, k, C.byref(st)), ctx.h)
                stats.append((st.samples, st.shaded_samples))
            abi.check(ctx.lib.cvr_batch_run(bh), ctx.h)  # graph replay
            abi.check(ctx.lib.cvr_sync(ctx.h), ctx.h)
            second = [mem.download(p, (H, W, 4)) for p in outs]
        finally:
            ctx.lib.cvr_batch_destroy(bh)
        mismatches = []
        for k, j in enumerate(b.jobs):
            assert np.array_equal(first[k], second[k]), f"job {k}: replay differs"
            ctx.select_volume(j.volume)
            params = b.params[k]
            img, st = ctx.render(j.method, j.camera, j.light, params, W, H)
            if not np.array_equal(img, first[k]):
                mismatches.append((k, j.method, float(np.abs(img - first[k]).max())))
            assert (st.samples, st.shaded_samples) == stats[k], (k, stats[k], st.samples)
            assert np.isfinite(img).all() and img[..., 3].max() > 0
        assert not mismatches, mismatches
    finally:
        abi.check(ctx.lib.cvr_set_compact_sat(ctx.h, 1), ctx.h)
        ctx.select_volume(0)
        ctx.set_sampling(abi.SAMPLING_TEX_FEATURES)
        abi.check(ctx.lib.cvr_set_tuning(ctx.h, 16, 8, 0), ctx.h)
        abi.check(ctx.lib.cvr_set_brick_size(ctx.h, 0), ctx.h)
        abi.check(ctx.lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_PLAIN), ctx.h)
        abi.check(ctx.lib.cvr_set_warp_shape(ctx.h, 8), ctx.h)
        mem.close()


def test_batch_rejects_other_methods(ctx):
    p = abi.PlainParams()
    p.step_size = 0.5
    j = abi.Job()
    j.volume, j.method, j.params, j.params_size = 0, abi.PLAIN, C.addressof(p), C.sizeof(p)
    j.width = j.height = 8
    bh = C.c_void_p()
    arr = (abi.Job * 1)(j)
    assert ctx.lib.cvr_batch_create(ctx.h, arr, 1, C.byref(bh)) == abi.CVR_ERR_INVALID_ARG


def test_batch_with_compact_sats(ctx):
    """With the compact SAT on (the default) a batch builds one compact table
    per volume at the largest region of its jobs; its images stay within 1/255
    of the single renders (which choose the fixed point per frame)."""
    vols = scene.batch_volumes(0.5)
    scene.prepare_batch_volumes(ctx, vols)
    small_network(ctx)
    W = H = 40
    mem = DeviceMemory()
    try:
        probe = scene.batch_jobs(vols, n_views=2, lights=scene.BATCH_LIGHTS[:2], image=W)
        n = len(probe.jobs)
        outs = [mem.alloc(W * H * 16, fill=0) for _ in range(n)]
        b = scene.batch_jobs(vols, n_views=2, lights=scene.BATCH_LIGHTS[:2], image=W, out_ptrs=outs)
        arr = (abi.Job * n)(*b.jobs)
        bh = C.c_void_p()
        abi.check(ctx.lib.cvr_batch_create(ctx.h, arr, n, C.byref(bh)), ctx.h)
        try:
            abi.check(ctx.lib.cvr_batch_run(bh), ctx.h)
            abi.check(ctx.lib.cvr_sync(ctx.h), ctx.h)
            got = [mem.download(p, (H, W, 4)) for p in outs]
        finally:
            ctx.lib.cvr_batch_destroy(bh)
        worst = 0.0
        for k, j in enumerate(b.jobs):
            if j.method != abi.EXTINCTION:
                continue
            ctx.select_volume(j.volume)
            img, _ = ctx.render(j.method, j.camera, j.light, b.params[k], W, H)
            worst = max(worst, float(np.abs(img - got[k]).max()))
        assert worst <= 1.0 / 255.0, worst
    finally:
        ctx.select_volume(0)
        mem.close()
