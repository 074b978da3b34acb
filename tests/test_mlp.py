"""The tensor-core surrogate network against its FP64 reference
(oracle/mlp_ref.py): forward outputs, gradients of every parameter, and a
training run that must reduce the loss."""
import ctypes as C

import numpy as np
import pytest

from cpp_volume_rendering_gb300 import abi
from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def params(ctx, lib):
    p = np.zeros(abi.MLP_PARAMS, np.float32)
    abi.check(lib.cvr_mlp_get_params(ctx.h, abi.fptr(p), abi.MLP_PARAMS), ctx.h)
    return p


def test_forward_matches_reference(ctx):
    lib = abi.load()
    abi.check(lib.cvr_mlp_init(ctx.h, 7), ctx.h)
    rng = np.random.default_rng(1)
    for n in (1, 128, 300):
        X = rng.normal(0, 1, size=(n, 48)).astype(np.float32)
        Y = np.zeros((n, 2), np.float32)
        abi.check(lib.cvr_mlp_forward(ctx.h, abi.fptr(X), n, abi.fptr(Y)), ctx.h)
        ref, _ = mlp_ref.forward(params(ctx, lib), X, bf=True)
        scale = max(1.0, np.abs(ref).max())
        assert np.abs(Y - ref).max() <= 2e-3 * scale, (n, np.abs(Y - ref).max())


def test_gradients_match_reference(ctx):
    lib = abi.load()
    abi.check(lib.cvr_mlp_init(ctx.h, 11), ctx.h)
    rng = np.random.default_rng(2)
    n = 300  # three tiles, the last one partial
    X = rng.normal(0, 1, size=(n, 48)).astype(np.float32)
    T = rng.uniform(0, 1, size=(n, 2)).astype(np.float32)
    g = np.zeros(abi.MLP_PARAMS, np.float32)
    loss = C.c_float()
    abi.check(lib.cvr_mlp_gradients(ctx.h, abi.fptr(X), abi.fptr(T), n, abi.fptr(g), C.byref(loss)), ctx.h)
    p = params(ctx, lib)
    ref, ref_loss = mlp_ref.gradients(p, X, T, bf=True)
    exact, exact_loss = mlp_ref.gradients(p, X, T, bf=False)
    assert abs(loss.value - ref_loss) <= 1e-3 * ref_loss
    groups = {"W1": (0, 3072), "b1": (3072, 3136), "W2": (3136, 7232), "b2": (7232, 7296), "W3": (7296, 7424),
              "b3": (7424, 7426)}
    for name, (a, b) in groups.items():
        rel = np.linalg.norm(g[a:b] - ref[a:b]) / max(np.linalg.norm(ref[a:b]), 1e-12)
        assert rel <= 1e-2, (name, rel)
        rel_exact = np.linalg.norm(g[a:b] - exact[a:b]) / max(np.linalg.norm(exact[a:b]), 1e-12)
        assert rel_exact <= 5e-2, (name, rel_exact)


def test_training_reduces_loss(ctx):
    lib = abi.load()
    abi.check(lib.cvr_mlp_init(ctx.h, 3), ctx.h)
    rng = np.random.default_rng(5)
    n = 65536
    X = rng.normal(0, 1, size=(n, 48)).astype(np.float32)
    # a smooth target in [0, 1] of a few input features
    T = np.stack([1.0 / (1.0 + np.exp(-(X[:, 0] - 0.5 * X[:, 3]))), np.exp(-0.25 * X[:, 1] ** 2)], 1)
    T = T.astype(np.float32)
    abi.check(lib.cvr_mlp_set_training_data(ctx.h, abi.fptr(X), abi.fptr(T), n), ctx.h)
    assert lib.cvr_mlp_training_size(ctx.h) == n
    losses = np.zeros(20, np.float32)
    abi.check(lib.cvr_mlp_train(ctx.h, 20, 1024, 3e-3, 9, abi.fptr(losses)), ctx.h)
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.2 * losses[0], losses
    # the trained network predicts the held-out function
    Xv = rng.normal(0, 1, size=(512, 48)).astype(np.float32)
    Tv = np.stack([1.0 / (1.0 + np.exp(-(Xv[:, 0] - 0.5 * Xv[:, 3]))), np.exp(-0.25 * Xv[:, 1] ** 2)], 1)
    Yv = np.zeros((512, 2), np.float32)
    abi.check(lib.cvr_mlp_forward(ctx.h, abi.fptr(Xv), 512, abi.fptr(Yv)), ctx.h)
    rmse = float(np.sqrt(np.mean((Yv - Tv) ** 2)))
    baseline = float(np.sqrt(np.mean((Tv - T.mean(0)) ** 2)))  # predicting the training mean
    assert rmse < 0.35 * baseline, (rmse, baseline)
