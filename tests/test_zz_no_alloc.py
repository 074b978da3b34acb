"""cvr_mlp_gradients_noalloc: the network gradient from device buffers with the
scratch in a fixed device array (no allocation), against cvr_mlp_gradients
(same kernels, host buffers, allocated scratch).  Collected last so that it
also runs after everything else in the session; one case runs in a fresh
process.  Device buffers for the inputs come from the CUDA runtime through
ctypes (tests/devmem.py); free device memory is compared around the calls."""
import ctypes as C
import subprocess
import sys

import numpy as np
import pytest

from cpp_volume_rendering_gb300 import abi

pytestmark = pytest.mark.gpu


def device_memory():
    """The tests' own cudaMalloc'd buffers (tests/devmem.py), or a skip."""
    try:
        from tests.devmem import DeviceMemory
        return DeviceMemory()
    except (ImportError, RuntimeError) as e:
        pytest.skip(f"no CUDA runtime for test buffers: {e}")


def free_device_bytes(rt):
    free, total = C.c_size_t(), C.c_size_t()
    rt.cudaMemGetInfo.argtypes = [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def gradients_both(ctx, n, seed):
    lib = abi.load()
    rng = np.random.default_rng(seed)
    X = rng.normal(0, 1, size=(n, 48)).astype(np.float32)
    T = rng.uniform(0, 1, size=(n, 2)).astype(np.float32)
    g_ref = np.zeros(abi.MLP_PARAMS, np.float32)
    loss_ref = C.c_float()
    abi.check(lib.cvr_mlp_gradients(ctx.h, abi.fptr(X), abi.fptr(T), n, abi.fptr(g_ref), C.byref(loss_ref)), ctx.h)
    buf = device_memory()
    try:
        xd, td = buf.upload(X), buf.upload(T)
        gd, ld = buf.alloc(4 * abi.MLP_PARAMS), buf.alloc(4)
        # the first call on the device does the one-time set-up (and loads the kernels)
        abi.check(lib.cvr_mlp_gradients_noalloc(ctx.h, xd, td, n, gd, ld), ctx.h)
        abi.check(lib.cvr_mlp_check(ctx.h), ctx.h)
        free_before = free_device_bytes(buf.rt)
        out = []
        for _ in range(2):  # two calls in a row reuse the same scratch
            abi.check(lib.cvr_mlp_gradients_noalloc(ctx.h, xd, td, n, gd, ld), ctx.h)
            abi.check(lib.cvr_mlp_check(ctx.h), ctx.h)  # no tensor-core wait gave up
            out.append((buf.download(gd, abi.MLP_PARAMS), float(buf.download(ld, 1)[0])))
        # the property the entry point exists for: it allocated no device memory
        assert free_device_bytes(buf.rt) == free_before
    finally:
        buf.close()
    return g_ref, loss_ref.value, out


@pytest.mark.parametrize("n", [1, 300, abi.MLP_NOALLOC_MAX_POINTS])
def test_noalloc_gradients_match_allocating_entry_point(ctx, n):
    abi.check(abi.load().cvr_mlp_init(ctx.h, 17), ctx.h)
    g_ref, loss_ref, out = gradients_both(ctx, n, seed=n)
    scale = max(float(np.abs(g_ref).max()), 1e-12)
    for g, loss in out:
        # same kernels and reduction order: equal up to FP32 rounding
        assert np.abs(g - g_ref).max() <= 1e-6 * scale, np.abs(g - g_ref).max()
        assert abs(loss - loss_ref) <= 1e-6 * max(abs(loss_ref), 1e-12)


def test_noalloc_rejects_oversized_batches(ctx):
    lib = abi.load()
    abi.check(lib.cvr_mlp_init(ctx.h, 1), ctx.h)
    r = lib.cvr_mlp_gradients_noalloc(ctx.h, C.c_void_p(16), C.c_void_p(16), abi.MLP_NOALLOC_MAX_POINTS + 1,
                                      C.c_void_p(16), None)
    assert r == abi.CVR_ERR_INVALID_ARG
    assert b"CVR_MLP_NOALLOC_MAX_POINTS" in lib.cvr_last_error(ctx.h)


def test_noalloc_in_a_fresh_process():
    code = (
        "import numpy as np\n"
        "from cpp_volume_rendering_gb300 import scene\n"
        "from tests.test_zz_no_alloc import gradients_both\n"
        "from cpp_volume_rendering_gb300 import abi\n"
        "ctx = scene.Context(0)\n"
        "abi.check(abi.load().cvr_mlp_init(ctx.h, 5), ctx.h)\n"
        "g_ref, loss_ref, out = gradients_both(ctx, 777, seed=3)\n"
        "scale = max(float(np.abs(g_ref).max()), 1e-12)\n"
        "assert all(np.abs(g - g_ref).max() <= 1e-6 * scale for g, _ in out)\n"
        "ctx.close()\n"
        "print('ok')\n")
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    r = subprocess.run([sys.executable, "-c", code], cwd=str(root), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "ok" in r.stdout, r.stdout + r.stderr
