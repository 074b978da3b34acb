"""The learned occlusion / shadow surrogate: network inputs and ground-truth
labels of shading points against the CPU oracle, the fused tensor-core marcher
against the oracle's surrogate renderer, checkpoints, and the trained
network against the ground-truth integrator and the cone method.

Tolerances: with FP32 hand-written trilinear sampling, inputs within 2e-4
absolute of the FP64 restatement (FP32 taps and exponentials), surrogate
images within 1/255 max per channel and PSNR >= 50 dB of the FP64 oracle fed
the same network; with texture-unit sampling (8-bit interpolation weights,
the default) inputs within 3e-2 and images within 8/255, PSNR >= 40 dB.
Ground-truth labels within 2e-4; network outputs within 1e-2 of the
BF16-emulating FP64 forward (a BF16 operand that rounds the other way moves
an output by ~1e-3)."""
import math

import numpy as np
import pytest

import oracle
from cpp_volume_rendering_gb300 import abi, scene

pytestmark = pytest.mark.gpu


def small_scene(ctx, n=64, image=64, seed=4100):
    vol = scene.synth_blobs(n, n, n, abi.CVR_U8, 32, seed=seed, noise_max=20.0)
    wl = scene.surrogate_workload(vol, image)
    scene.prepare(ctx, wl)
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    return wl, orc


@pytest.mark.parametrize("sampling,tol", [(0, 2e-4), (abi.SAMPLING_TEX_FEATURES, 3e-2)])
def test_inputs_and_labels_match_oracle(ctx, sampling, tol):
    ctx.set_sampling(sampling)
    wl, orc = small_scene(ctx)
    ctx.clear_points()
    got = ctx.collect_points(wl.cam, 64, 64, wl.params.step_size, 0.05, 11, 4096)
    assert 50 < got <= 4096
    pts = ctx.points()
    assert pts.shape == (got, 6)
    # points lie inside the volume box on unit primary directions
    S = np.array(wl.dims, np.float32)
    assert (pts[:, :3] >= 0).all() and (pts[:, :3] <= S).all()
    assert np.allclose(np.linalg.norm(pts[:, 3:], axis=1), 1.0, atol=1e-5)
    for shadow_type, lt in ((0, wl.light), (2, scene.light(abi.LIGHT_DIRECTIONAL, forward=wl.light.forward[:],
                                                             up=wl.light.up[:], right=wl.light.right[:]))):
        gp = scene.gt_params(wl.params.step_size, wl.diagonal, occ_distance=32.0, light_step=1.0, gap=1.0,
                             shadow_type=shadow_type)
        x, t = ctx.label_points(lt, gp)
        xr = orc.sur_features(lt, gp, pts)
        err = np.abs(x - xr)
        print(f"inputs sampling={sampling} shadow_type={shadow_type}: max err {err.max():.2e} "
              f"(taps {err[:, :42].max():.2e}, gradient {err[:, 45:].max():.2e}), "
              f"labels {np.abs(t - orc.gt_points(lt, gp, pts)).max():.2e}")
        assert err.max() <= tol, (shadow_type, err.max(), np.unravel_index(err.argmax(), err.shape))
        assert (x[:, :42] >= 0).all() and (x[:, :42] < 1).all()
        assert np.allclose(np.linalg.norm(x[:, 42:45], axis=1), 1.0, atol=1e-4)
        tr = orc.gt_points(lt, gp, pts)
        assert np.abs(t - tr).max() <= 2e-4, np.abs(t - tr).max()
        assert (t >= 0).all() and (t <= 1 + 1e-6).all()
    ctx.set_sampling(abi.SAMPLING_TEX_FEATURES)


def test_network_outputs_on_points_match_oracle(ctx, lib):
    ctx.set_sampling(0)
    wl, orc = small_scene(ctx, seed=4101)
    ctx.mlp_init(21)
    ctx.clear_points()
    ctx.collect_points(wl.cam, 64, 64, wl.params.step_size, 0.05, 12, 2048)
    pts = ctx.points()
    x, _ = ctx.label_points(wl.light, wl.params)
    y = np.zeros((len(x), 2), np.float32)
    abi.check(lib.cvr_mlp_forward(ctx.h, abi.fptr(x), len(x), abi.fptr(y)), ctx.h)
    orc.set_mlp(ctx.mlp_params())
    _, yr = orc.sur_features(wl.light, wl.params, pts, with_outputs=True)
    scale = max(1.0, float(np.abs(yr).max()))
    print(f"network outputs: max err {np.abs(y - yr).max():.2e} (scale {scale:.2f})")
    ctx.set_sampling(abi.SAMPLING_TEX_FEATURES)
    assert np.abs(y - yr).max() <= 1e-2 * scale, np.abs(y - yr).max()


@pytest.mark.parametrize("n,image,shadow_type,sampling", [(64, 64, 0, 0), (64, 40, 2, 0), (64, 64, 0, 1)])
def test_surrogate_image_matches_oracle(ctx, n, image, shadow_type, sampling):
    vol = scene.synth_blobs(n, n, n, abi.CVR_U8, 32, seed=4102, noise_max=20.0)
    wl = scene.surrogate_workload(vol, image)
    if shadow_type == 2:
        f, u, r = scene.light_frame((0.3, 0.9, -0.2))
        wl.light = scene.light(abi.LIGHT_DIRECTIONAL, forward=f, up=u, right=r)
        wl.params.shadow_type = 2
    scene.prepare(ctx, wl)
    ctx.mlp_init(5)
    # a network whose outputs span [0, 1]: small random weights, biases 0.5
    p = ctx.mlp_params()
    p[abi.MLP_PARAMS - 2:] = 0.5
    p[64 * 48 + 64 + 64 * 64 + 64:abi.MLP_PARAMS - 2] *= 0.05
    ctx.mlp_set_params(p)
    ctx.set_sampling(sampling)
    img, st = ctx.render(abi.SURROGATE, wl.cam, wl.light, wl.params, image, image)
    ctx.set_sampling(abi.SAMPLING_TEX_FEATURES)
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    orc.set_mlp(p)
    ref, _, total = orc.render(abi.SURROGATE, wl.cam, wl.light, wl.params, image, image, precision=64)
    assert np.isfinite(img).all()
    err = np.abs(img.astype(np.float64) - ref)
    mse = float(np.mean(err ** 2))
    psnr = float("inf") if mse == 0 else 10 * math.log10(1.0 / mse)
    print(f"surrogate image n={n} {image}^2 sampling={sampling}: max err {err.max():.2e} psnr {psnr:.1f} dB")
    max_abs, min_psnr = (1.0 / 255.0, 50.0) if sampling == 0 else (8.0 / 255.0, 40.0)
    assert err.max() <= max_abs, err.max()
    assert psnr >= min_psnr, psnr
    assert abs(int(st.samples) - int(total)) <= max(2, total // 2000)
    assert st.shaded_samples > 0 and st.aux_fetches == 67 * st.shaded_samples  # pyramid taps per point


def test_surrogate_needs_network_and_pyramid(ctx, lib):
    vol = scene.synth_blobs(32, 32, 32, abi.CVR_U8, 8, seed=4103, noise_max=20.0)
    wl = scene.surrogate_workload(vol, 16)
    ctx.set_volume(wl.volume, wl.spacing)
    ctx.set_transfer_function(wl.tf)
    ctx.build_pyramid(base_dims=(16, 16, 16), sigma0=1.0, n_levels=4)  # too few levels
    ctx.mlp_init(1)
    out = np.zeros((16, 16, 4), np.float32)
    r = lib.cvr_render_host(ctx.h, abi.SURROGATE, abi.C.byref(wl.cam), abi.C.byref(wl.light),
                            abi.C.byref(wl.params), abi.C.sizeof(wl.params), abi.fptr(out), 16, 16, None)
    assert r == abi.CVR_ERR_NOT_READY


def test_checkpoint_roundtrip(ctx, tmp_path):
    ctx.mlp_init(77)
    p = ctx.mlp_params()
    path = str(tmp_path / "net.cvrmlp").encode()
    abi.check(ctx.lib.cvr_mlp_save(ctx.h, path), ctx.h)
    ctx.mlp_init(78)
    assert not np.array_equal(ctx.mlp_params(), p)
    abi.check(ctx.lib.cvr_mlp_load(ctx.h, path), ctx.h)
    assert np.array_equal(ctx.mlp_params(), p)
    bad = tmp_path / "bad.cvrmlp"
    bad.write_bytes(b"CVRMLP01" + b"\0" * 16)
    assert ctx.lib.cvr_mlp_load(ctx.h, str(bad).encode()) == abi.CVR_ERR_FORMAT


def test_trained_surrogate_beats_cone_and_runs_faster_than_gt(ctx):
    """Reduced-scale training run (6 volumes of 96^3, 300k points) that must
    already cut the occlusion error well below the cone method's and run far
    faster than the ground-truth integrator; the full-scale figure (20 volumes
    of 160^3 .. 448^3, up to 8M points, held-out 512^3 at 1024^2) is measured by
    the bench and bounded by test_heldout_rmse_within_bound."""
    ctx.mlp_init(3)
    ctx._ck(ctx.lib.cvr_mlp_set_training_data(ctx.h, None, None, 0))
    n0 = ctx.lib.cvr_mlp_training_size(ctx.h)
    assert n0 == 0
    added = scene.build_surrogate_training_set(ctx, n_volumes=6, size=96, points=300_000, views=4, image=160)
    assert added > 200_000
    assert ctx.lib.cvr_mlp_training_size(ctx.h) == n0 + added
    losses = scene.train_surrogate(ctx, batch=2048, schedule=((10, 2e-3), (5, 5e-4)))
    assert losses[-1] < 0.5 * losses[0], losses
    vol = scene.synth_blobs(128, 128, 128, abi.CVR_U8, 32, seed=4190, noise_max=20.0)
    wl = scene.surrogate_workload(vol, 256)
    scene.prepare(ctx, wl)
    r = scene.evaluate_surrogate(ctx, wl, points=200_000)
    print("reduced-scale surrogate:", {k: round(v, 5) for k, v in r.items()}, "final loss", losses[-1])
    assert r["points"] > 50_000
    assert r["rmse_ao"] < 0.5 * r["cone_rmse_ao"], r
    assert r["rmse_shadow"] < r["cone_rmse_shadow"], r
    # frame times: the surrogate frame against the GT frame of the same view
    img_s, st_s = ctx.render(abi.SURROGATE, wl.cam, wl.light, wl.params, 256, 256)
    img_g, st_g = ctx.render(abi.GROUND_TRUTH, wl.cam, wl.light, wl.params, 256, 256)
    assert st_s.samples == st_g.samples and st_s.shaded_samples == st_g.shaded_samples
    print(f"frame 256^2: GT {st_g.kernel_ms:.2f} ms, surrogate {st_s.kernel_ms:.2f} ms")
    assert st_g.kernel_ms > 5.0 * st_s.kernel_ms, (st_g.kernel_ms, st_s.kernel_ms)
    assert np.abs(img_s - img_g).max() < 0.25


def test_heldout_rmse_within_bound(ctx):
    """The surrogate's accuracy bound: trained from scratch with the benchmark's
    budget (up to 8M ground-truth-labelled shading points of 20 seeded blob
    volumes of 160^3 .. 448^3, the Adam schedule of scene.SURROGATE_SCHEDULE,
    about fifteen seconds on one GPU), its occlusion and shadow RMSE against the ground-truth
    integrator over 2M shading points of the held-out 512^3 volume at 1024^2
    are both at most 0.02, and well below the cone method's."""
    ctx.mlp_init(scene.SURROGATE_SEED)
    ctx._ck(ctx.lib.cvr_mlp_set_training_data(ctx.h, None, None, 0))
    added = scene.build_surrogate_training_set(ctx)
    assert added > 3_000_000
    losses = scene.train_surrogate(ctx)
    assert losses[-1] < 0.2 * losses[0], losses
    wl = scene.workload("surrogate")
    scene.prepare(ctx, wl)
    r = scene.evaluate_surrogate(ctx, wl)
    print("held-out surrogate:", {k: round(v, 5) for k, v in r.items()})
    assert r["points"] > 1_000_000
    assert r["rmse_ao"] <= 0.02, r
    assert r["rmse_shadow"] <= 0.02, r
    assert r["rmse_ao"] < 0.25 * r["cone_rmse_ao"], r
