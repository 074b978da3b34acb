"""The headless RenderingManager driver (cvr_headless): data loading and error
reporting run on the host before any device call, so they are tested on CPU;
the rendering path is compared with the C ABI render on the GPU."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from cpp_volume_rendering_gb300 import abi, build, scene

TOOL = build.TOOL


@pytest.fixture(scope="module")
def data(tmp_path_factory, lib):
    d = tmp_path_factory.mktemp("headless")
    vol = scene.synth_blobs(24, 20, 16, abi.CVR_U8, 5, seed=21)
    vp = d / "blobs.1.24x20x16.raw"
    vol.tofile(vp)
    tp = d / "ramp.tf1d"
    tp.write_text("linear\n0\n4\n0.2 0.3 0.9 0\n0.3 0.8 0.4 80\n0.9 0.7 0.2 160\n1.0 0.95 0.9 255\n"
                  "4\n0.0 0\n0.05 80\n0.4 160\n0.9 255\n")
    cp = d / "cameras"
    cp.write_text("Front\nARCBALL\n 10.0 20.0 60.0\n 0.0 0.0 0.0\n 0.0 1.0 0.0\n"
                  "Side\nARCBALL\n-55.0 10.0 5.0\n 0.0 0.0 0.0\n 0.0 1.0 0.0\n")
    lp = d / "lights"
    lp.write_text("One light\n1\n-40.0 60.0 30.0\n-0.5 0.75 0.4\n0.0 1.0 0.0\n1.0 0.0 0.0\n20\n")
    return dict(vol=vol, vp=vp, tp=tp, cp=cp, lp=lp, dir=d)


def run(*args):
    return subprocess.run([str(TOOL), *map(str, args)], capture_output=True, text=True, timeout=300)


def test_usage_errors(data):
    assert run().returncode == 1
    assert run("--volume", data["vp"]).returncode == 1
    assert run("--bogus").returncode == 1
    assert run("--gradient", "laplace").returncode == 1
    assert run("--volume", data["vp"], "--tf", data["tp"], "--renderer", "s_1rc", "--multiscaling", "4").returncode == 1


def test_data_errors_before_any_device_call(data, tmp_path):
    r = run("--volume", tmp_path / "missing.1.4x4x4.raw", "--tf", data["tp"], "--renderer", "s_1rc")
    assert r.returncode == 2 and "opening .raw" in r.stderr
    short = tmp_path / "short.1.8x8x8.raw"
    short.write_bytes(b"\1" * 100)
    r = run("--volume", short, "--tf", data["tp"], "--renderer", "s_1rc")
    assert r.returncode == 2 and "short .raw" in r.stderr
    badtf = tmp_path / "bad.tf1d"
    badtf.write_text("linear\n0\n3\n1 1 1 0\n")
    r = run("--volume", data["vp"], "--tf", badtf, "--renderer", "s_1rc")
    assert r.returncode == 2 and "tf1d" in r.stderr
    r = run("--volume", data["vp"], "--tf", data["tp"], "--renderer", "s_1rc", "--cameras", data["cp"],
            "--camera-index", "7")
    assert r.returncode == 2 and "camera" in r.stderr
    badl = tmp_path / "lights"
    badl.write_text("Broken\n2\n1 2 3\n")
    r = run("--volume", data["vp"], "--tf", data["tp"], "--renderer", "s_1rc", "--lights", badl)
    assert r.returncode == 2 and "light" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("abbr,method", [("s_1rc", abi.PLAIN), ("s_1pebs", abi.EXTINCTION),
                                         ("s_1pdosct", abi.CONE_DOS), ("s_1pcrtgt", abi.GROUND_TRUTH),
                                         ("iso", abi.ISO)])
def test_headless_frames(data, abbr, method, tmp_path):
    out = tmp_path / f"{abbr}.pfm"
    # the ground-truth renderer starts with occlusion and shadows off (crtgtrenderer.cpp:40-46)
    extra = ["--occlusion", "1", "--shadow", "1"] if abbr == "s_1pcrtgt" else []
    r = run("--volume", data["vp"], "--tf", data["tp"], "--renderer", abbr, "--width", "40", "--height", "32",
            "--cameras", data["cp"], "--camera-index", "1", "--lights", data["lp"], "--out", out, *extra)
    assert r.returncode == 0, r.stderr
    assert f"renderer={abbr}" in r.stdout
    raw = out.read_bytes()
    header_end = raw.index(b"-1.0\n") + 5
    assert raw[:header_end].split()[:3] == [b"PF", b"40", b"32"]
    img = np.frombuffer(raw[header_end:], np.float32).reshape(32, 40, 3)
    assert np.isfinite(img).all() and img.max() > 0.0


@pytest.mark.gpu
def test_headless_surrogate_renderer(ctx, tmp_path):
    """The surrogate plugin (no reference counterpart) loads a network
    checkpoint and renders; without one it reports the missing network."""
    vol = scene.synth_blobs(64, 64, 64, abi.CVR_U8, 16, seed=22, noise_max=20.0)
    vp = tmp_path / "blobs.1.64x64x64.raw"
    vol.tofile(vp)
    tp = tmp_path / "ramp.tf1d"
    tp.write_text("linear\n0\n4\n0.2 0.3 0.9 0\n0.3 0.8 0.4 80\n0.9 0.7 0.2 160\n1.0 0.95 0.9 255\n"
                  "4\n0.0 0\n0.05 80\n0.4 160\n0.9 255\n")
    ckpt = tmp_path / "net.cvrmlp"
    ctx.mlp_init(9)
    abi.check(ctx.lib.cvr_mlp_save(ctx.h, str(ckpt).encode()), ctx.h)
    out = tmp_path / "surr.pfm"
    r = run("--volume", vp, "--tf", tp, "--renderer", "s_1psurr", "--width", "48", "--height", "40",
            "--occlusion", "1", "--shadow", "1", "--weights", ckpt, "--out", out)
    assert r.returncode == 0, r.stderr
    assert "renderer=s_1psurr" in r.stdout
    raw = out.read_bytes()
    img = np.frombuffer(raw[raw.index(b"-1.0\n") + 5:], np.float32).reshape(40, 48, 3)
    assert np.isfinite(img).all() and img.max() > 0.0
    r = run("--volume", vp, "--tf", tp, "--renderer", "s_1psurr", "--width", "16", "--height", "16")
    assert r.returncode != 0 and "network" in (r.stdout + r.stderr)


@pytest.mark.gpu
@pytest.mark.parametrize("abbr,model", [("s_1rc", "fd"), ("s_1pebs", "sobel"), ("s_1pdosct", "cs")])
def test_headless_gradient_shading(data, abbr, model, tmp_path):
    """--gradient picks DataManager's gradient model and --gradient-shading the
    renderers' "Apply Gradient Shading" switch: the frame changes, opacity does not.
    (With the cone renderer's default of no shadows the gradient branch only
    differs from the plain one where the gradient vanishes, so shadows are on.)"""
    illum = ["--occlusion", "1", "--shadow", "1"] if abbr == "s_1pdosct" else []

    def frame(*extra):
        out = tmp_path / f"{abbr}_{len(extra)}.pfm"
        r = run("--volume", data["vp"], "--tf", data["tp"], "--renderer", abbr, "--width", "40", "--height", "32",
                "--cameras", data["cp"], "--camera-index", "0", "--lights", data["lp"], "--out", out, *illum,
                *extra)
        assert r.returncode == 0, r.stderr
        raw = out.read_bytes()
        return np.frombuffer(raw[raw.index(b"-1.0\n") + 5:], np.float32).reshape(32, 40, 3)
    plain = frame()
    model_only = frame("--gradient", model)
    shaded = frame("--gradient", model, "--gradient-shading", "1")
    assert np.array_equal(plain, model_only)  # a gradient alone changes nothing
    assert np.isfinite(shaded).all() and not np.array_equal(shaded, plain)


@pytest.mark.gpu
@pytest.mark.parametrize("fixture", ["smooth_v3e_strip143.pvm", "wide_u16_v3_dds_skip2.pvm"])
def test_headless_reads_pvm(data, fixture, tmp_path):
    """A DDS-compressed .pvm goes through ReadStructuredVolume to a frame."""
    vol = Path(__file__).resolve().parent / "golden" / "pvm" / fixture
    out = tmp_path / "pvm.pfm"
    r = run("--volume", vol, "--tf", data["tp"], "--renderer", "s_1rc", "--width", "24", "--height", "24",
            "--eye", "0", "0", "40", "--out", out)
    assert r.returncode == 0, r.stderr
    assert out.stat().st_size > 24 * 24 * 12


@pytest.mark.gpu
def test_headless_multiscaling(data, tmp_path):
    """--multiscaling picks the extinction renderer's MULTISCALING mode (the
    others do not declare support, as in the reference): frames change with
    the mode and stay finite; the plain renderer ignores it."""
    def frame(abbr, *extra):
        out = tmp_path / f"{abbr}_{'_'.join(extra)}.pfm"
        r = run("--volume", data["vp"], "--tf", data["tp"], "--renderer", abbr, "--width", "40", "--height", "32",
                "--cameras", data["cp"], "--camera-index", "0", "--lights", data["lp"], "--out", out, *extra)
        assert r.returncode == 0, r.stderr
        raw = out.read_bytes()
        return np.frombuffer(raw[raw.index(b"-1.0\n") + 5:], np.float32).reshape(32, 40, 3)
    base = frame("s_1pebs")
    for mode in ("1", "2", "3"):
        img = frame("s_1pebs", "--multiscaling", mode, "--image-filter", "4")
        assert np.isfinite(img).all() and not np.array_equal(img, base), mode
    assert np.array_equal(frame("s_1rc", "--multiscaling", "2"), frame("s_1rc"))
