"""Benchmark of the GB300 volume ray caster (one JSON line on rank 0).

Default workload (the headline configuration): extinction-based shading of a
256^3 u16 value-noise volume (4 octaves, lacunarity 2, gain 0.5, 4 nested
shells) rendered at 1024^2 with SAT ambient occlusion (radii 2, 6, 16 voxels)
and a directional SAT cone shadow, step 0.5 voxel.  A step is one frame.

  value  : Msamples/s of the render kernel with inputs resident in HBM
           (primary-ray steps counted by the kernel / CUDA-event time), L2
           flushed between timed frames.
  e2e    : the same metric through the C ABI from host buffers: per step the
           volume is copied from pinned host memory (cvr_set_volume), the SAT
           is rebuilt (cvr_build_sat) and the frame is rendered and read back
           (cvr_render_host) — the Init() + Redraw() + readback sequence.
  roofline: the marcher is bound by the L1 load path (its volume and SAT
           quads are cache-resident): the bytes its 16-byte gathers request
           per launch / kernel time, against the L1 hit bandwidth of the same
           load instruction measured in this run (cvr_measure_l1_bandwidth);
           its DRAM traffic (ncu) against the measured HBM copy bandwidth is
           reported beside it.
  cpu_baseline: the FP32 CPU oracle (a restatement of the reference shaders)
           on all host cores over a band of rows of the same frame.

Output: one JSON line per section (renderers, surrogate, batch, gradient,
post-passes, tables) as each finishes, then the headline line LAST.

--impl reference times that CPU restatement alone (the reference's own GLSL
path needs OpenGL, which neither machine has); it builds its workload with
the oracle's own generators and tables and never loads libcvr.so.
With torchrun (N > 1) every rank renders its own frame on its own GPU
(replicas; the path needs no exchange), timing is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOAD_DESC = {
    "extinction": "extinction SAT shading: 256^3 u16 value-noise shells -> 1024^2, AO radii {2,6,16} + "
                  "directional SAT cone shadow, step 0.5 voxel",
    "plain": "plain ray casting: 64^3 u8 8-blob volume, unit cube -> 256^2, step 0.5 voxel",
    "plain_large": "plain ray casting: 256^3 u8 8-blob volume, unit cube -> 1024^2, step 0.5 voxel",
    "extinction_lightcache": "extinction shading with the 32^3 object-space light cache: 256^3 u16 value-noise "
                             "shells -> 1024^2, AO radii {2,6,16} + directional SAT cone shadow per cache cell",
    "iso": "adaptive-step isosurface caster: 256^3 u16 value-noise shells -> 1024^2, isovalue 0.5, steps "
           "0.05 / 1.0 voxels within / beyond 0.1 of it, opaque colour",
    "cone": "cone DOS shading: 256^3 u8 32 blobs + U[0,20] noise -> 512^2, 5-level extinction pyramid, "
            "occlusion + point-light shadow cones",
    "ground_truth": "ground truth: 256^3 u8 32 blobs + U[0,20] noise -> 512^2, 16 occlusion rays of 32 voxels + "
                    "1 shadow ray to a point light, 1-voxel light steps",
    "surrogate": "learned occlusion/shadow surrogate: MLP 48-64-64-2 (BF16 tcgen05) trained on up to 8M GT-labelled "
                 "points of 20 seeded blob volumes (160^3..448^3); held-out 512^3 u8 blobs -> 1024^2, point light",
}

MLP_FLOP_PER_SAMPLE = 2 * (48 * 64 + 64 * 64 + 64 * 2)  # 14,592
GRADIENT_BUILDERS = {1: "k_gradient_tiled", 2: "k_gradient", 3: "k_gradient_tma"}
ROOFLINE_NOTES = {
    "extinction": "algorithmic gather bytes (8 voxel texels per primary step + 64 four-byte SAT texels per box "
                  "query + image); the SAT and volume are L2-resident, so the effective gather rate can exceed the "
                  "HBM line; ncu shows the marcher bound by L1 throughput (88 % with 8x4-pixel warps, 73 % with 4x8) "
                  "with the integer pipe next (54-57 %), DRAM traffic about 1/2700 of the gathered bytes",
    "plain_large": "algorithmic gather bytes (8 voxel texels per primary step + image); ncu shows the marcher "
                   "instruction-issue bound (81 % issue active) with the gathers hitting L1 (91 %)",
}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier_max(values, ws):
    """Barrier + max over ranks (gloo on host tensors); identity for one rank."""
    if ws == 1:
        return values
    import torch
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def barrier_sum(values, ws):
    if ws == 1:
        return values
    import torch
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.tolist()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"cvr_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [l.split(",") for l in self.path.read_text().splitlines() if l.strip()]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def profile_traffic(workload):
    """Per-launch DRAM traffic of the marcher from the committed ncu summary."""
    for p in sorted((ROOT / "profiles").glob(f"*{workload}*.md")):
        m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", p.read_text())
        if m:
            return float(m.group(1)), p.name
    return None, None


def algorithmic_bytes(wl, st, abi):
    """Algorithmic bytes of one frame: 8 voxel texels per primary sample,
    plus per secondary fetch 64 four-byte SAT texels (extinction: the
    reference's R32F table, this library's compact table), 8 float32 pyramid
    texels (cone) or 8 voxel texels (ground truth), plus the image."""
    bvox = 1 if wl.dtype == abi.CVR_U8 else 2
    if wl.method == abi.SURROGATE:  # per shaded sample: 67 pyramid taps of 8 float32 texels
        return st.samples * 8 * bvox + st.shaded_samples * 67 * 8 * 4 + wl.width * wl.height * 16
    per_aux = {abi.PLAIN: 0, abi.EXTINCTION: 64 * 4, abi.CONE_DOS: 8 * 4, abi.GROUND_TRUTH: 8 * bvox,
               abi.ISO: 0}[wl.method]
    return st.samples * 8 * bvox + st.aux_fetches * per_aux + wl.width * wl.height * 16


def l1_request_bytes(wl, st, abi, walk):
    """Bytes the extinction marcher's loads request from L1 per frame: the
    volume's trilinear footprint per primary step, 16 sixteen-byte quads per
    AO box, per shadow box 16 quads or, from a walk table, 4 thirty-two-byte
    octs, and the image.  Other methods: their algorithmic bytes."""
    if wl.method != abi.EXTINCTION:
        return algorithmic_bytes(wl, st, abi)
    bvox = 1 if wl.dtype == abi.CVR_U8 else 2
    p = wl.params
    ao = st.shaded_samples * (p.ao_n_shells if p.apply_occlusion else 0)
    shadow = st.aux_fetches - ao
    return (st.samples * 8 * bvox + ao * 256 + shadow * (128 if walk else 256) + wl.width * wl.height * 16)


def cpu_baseline(wl, target_s=12.0, threads=None):
    """FP32 oracle on all host cores over a centred band of rows."""
    import oracle
    threads = threads or os.cpu_count() or 1
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    H = wl.height
    band = max(1, H // 128)
    mid = H // 2
    t0 = time.perf_counter()
    _, _, n0 = orc.render(wl.method, wl.cam, wl.light, wl.params, wl.width, H, precision=32,
                          rows=(mid - band // 2, mid - band // 2 + band), threads=threads)
    dt = time.perf_counter() - t0
    rows = int(min(H, max(band, band * target_s / max(dt, 1e-3))))
    y0 = max(0, mid - rows // 2)
    t0 = time.perf_counter()
    _, _, n = orc.render(wl.method, wl.cam, wl.light, wl.params, wl.width, H, precision=32, rows=(y0, y0 + rows),
                         threads=threads)
    dt = time.perf_counter() - t0
    return {"value": n / dt / 1e6, "unit": "Msamples/s", "cores": threads, "kind": "port",
            "sample": f"rows {y0}..{y0 + rows} of the {wl.width}x{H} frame ({n} samples, {dt:.1f} s, FP32 oracle, "
                      f"OpenMP over rows)"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from cpp_volume_rendering_gb300 import scene
    import oracle
    oracle.build_lib()
    # the same workload, volume and tables built by the oracle alone
    wl = scene.workload(args.workload, n=args.size, image=args.image, gen=oracle.GEN)
    threads = os.cpu_count() or 1
    orc = oracle.Oracle()
    oracle.prepare(orc, wl)
    H = wl.height
    band = max(1, H // 128)
    mid = H // 2
    # size each step's band of rows so the whole run stays within a few minutes
    t0 = time.perf_counter()
    orc.render(wl.method, wl.cam, wl.light, wl.params, wl.width, H, precision=32,
               rows=(mid - band // 2, mid - band // 2 + band), threads=threads)
    dt = time.perf_counter() - t0
    per_step_s = min(20.0, 150.0 / max(1, args.steps + args.warmup))
    rows = int(min(H, max(band, band * per_step_s / max(dt, 1e-3))))
    y0 = max(0, mid - rows // 2)
    for _ in range(args.warmup):
        orc.render(wl.method, wl.cam, wl.light, wl.params, wl.width, H, precision=32, rows=(y0, y0 + rows),
                   threads=threads)
    tot_n, tot_t = 0, 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, _, n = orc.render(wl.method, wl.cam, wl.light, wl.params, wl.width, H, precision=32,
                             rows=(y0, y0 + rows), threads=threads)
        tot_t += time.perf_counter() - t0
        tot_n += n
    value = tot_n / tot_t / 1e6
    sample = f"rows {y0}..{y0 + rows} of the {wl.width}x{H} frame per step, FP32 oracle on {threads} threads"
    libs = mapped_repo_libraries()
    if any("libcvr" in l for l in libs):
        raise RuntimeError(f"the reference arm loaded the product library: {libs}")
    print(json.dumps({
        "impl": "reference", "metric": "Msamples/s", "value": value, "unit": "Msamples/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * tot_t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD_DESC[args.workload], "image": [wl.width, wl.height], "volume": list(wl.dims)},
        "cpu_baseline": {"value": value, "unit": "Msamples/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "native_libraries": libs,
        "note": "the reference renders with GLSL compute shaders (OpenGL), unavailable on this box; its CPU "
                "restatement (the oracle, with its own tables and volume generator) is what is timed"}), flush=True)


def mapped_repo_libraries():
    """Shared libraries of this repository mapped into the process."""
    out = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if len(line.split()) >= 6 else ""
                if path.startswith(str(ROOT)) and ".so" in path:
                    out.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(out)


def emit(section, obj):
    """One JSON line per benchmark section (the headline line comes last)."""
    print(json.dumps({"section": section, **obj}), flush=True)


def time_frames(ctx, lib, wl, params, out_ptr, steps, warmup, flush=True):
    import ctypes as C
    from cpp_volume_rendering_gb300 import abi
    cam, lt = wl.cam, wl.light
    for _ in range(warmup):
        abi.check(lib.cvr_render(ctx.h, wl.method, C.byref(cam), C.byref(lt), C.byref(params), C.sizeof(params),
                                 out_ptr, wl.width, wl.height, None, None), ctx.h)
    abi.check(lib.cvr_sync(ctx.h), ctx.h)
    times = []
    ms = C.c_float()
    for _ in range(steps):
        if flush:
            abi.check(lib.cvr_flush_l2(ctx.h), ctx.h)
        abi.check(lib.cvr_timer_start(ctx.h), ctx.h)
        abi.check(lib.cvr_render(ctx.h, wl.method, C.byref(cam), C.byref(lt), C.byref(params), C.sizeof(params),
                                 out_ptr, wl.width, wl.height, None, None), ctx.h)
        abi.check(lib.cvr_timer_stop(ctx.h, C.byref(ms)), ctx.h)
        times.append(ms.value)
    return times


def tuned_frames(ctx, lib, w2):
    """One prepared frame autotuned (tile x registers x volume layout) and timed with
    FP32 volume samples and with the texture-unit variant."""
    import ctypes as C
    from cpp_volume_rendering_gb300 import abi
    o2 = C.POINTER(C.c_float)()
    abi.check(lib.cvr_get_frame_buffer(ctx.h, w2.width, w2.height, C.byref(o2)), ctx.h)
    entry = {}
    for key, flags in (("", abi.SAMPLING_TEX_FEATURES),
                       ("tex_", abi.SAMPLING_TEX_FEATURES | abi.SAMPLING_TEX_VOLUME | abi.SAMPLING_TEX_PYRAMID)):
        ctx.set_sampling(flags)
        tw, th, tv = C.c_int(), C.c_int(), C.c_int()
        abi.check(lib.cvr_autotune(ctx.h, w2.method, C.byref(w2.cam), C.byref(w2.light), C.byref(w2.params),
                                   C.sizeof(w2.params), w2.width, w2.height, 1, C.byref(tw), C.byref(th),
                                   C.byref(tv), None), ctx.h)
        s2 = abi.FrameStats()
        abi.check(lib.cvr_render(ctx.h, w2.method, C.byref(w2.cam), C.byref(w2.light), C.byref(w2.params),
                                 C.sizeof(w2.params), C.cast(o2, C.c_void_p), w2.width, w2.height, None,
                                 C.byref(s2)), ctx.h)
        tt = time_frames(ctx, lib, w2, w2.params, C.cast(o2, C.c_void_p), 3, 1)
        m = statistics.median(tt)
        if not key:
            # the tuned configuration with the persistent ray refill switched the other
            # way (and, for the plain caster, brick staging): both variants' times
            alt = {}
            knobs = [("refill", lib.cvr_set_ray_refill, lib.cvr_get_ray_refill)]
            if w2.method == abi.PLAIN:
                knobs.append(("staging", lib.cvr_set_brick_staging, lib.cvr_get_brick_staging))
            for name, setter, getter in knobs:
                was = getter(ctx.h)
                abi.check(setter(ctx.h, 1 - was), ctx.h)
                keep = (lib.cvr_get_brick_size(ctx.h), lib.cvr_get_volume_layout(ctx.h))
                if name == "staging" and not was:  # staging reads the plain layout
                    abi.check(lib.cvr_set_brick_size(ctx.h, 0), ctx.h)
                    abi.check(lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_PLAIN), ctx.h)
                t_alt = statistics.median(time_frames(ctx, lib, w2, w2.params, C.cast(o2, C.c_void_p), 3, 1))
                abi.check(setter(ctx.h, was), ctx.h)
                abi.check(lib.cvr_set_brick_size(ctx.h, keep[0]), ctx.h)
                abi.check(lib.cvr_set_volume_layout(ctx.h, keep[1]), ctx.h)
                alt[f"{name}_on_ms" if was else f"{name}_off_ms"] = m
                alt[f"{name}_off_ms" if was else f"{name}_on_ms"] = t_alt
            entry["variants"] = alt
        entry.update({key + "ms": m, key + "fps": 1000.0 / m, key + "msamples_s": s2.samples / (m / 1000.0) / 1e6,
                      key + "roofline_achieved_gbs": algorithmic_bytes(w2, s2, abi) / (m / 1000.0) / 1e9,
                      key + "tuning": {"tile": [tw.value, th.value], "variant": tv.value,
                                       "brick": lib.cvr_get_brick_size(ctx.h),
                  "quads": lib.cvr_get_volume_layout(ctx.h), "warp_w": lib.cvr_get_warp_shape(ctx.h),
              "refill": lib.cvr_get_ray_refill(ctx.h), "staging": lib.cvr_get_brick_staging(ctx.h)}})
    ctx.set_sampling(abi.SAMPLING_TEX_FEATURES)
    return entry


def gradient_section(ctx, lib, args, log=print):
    """Gradient Blinn-Phong: the device gradient builders (HBM-bound: each
    voxel read once from L1/L2-cached neighbourhoods, 8 bytes written) against
    the measured copy bandwidth and the FP64 CPU restatement of the
    reference's builders, then shaded frames of the plain and extinction
    workloads with the finite-difference gradient and the reference's default
    Blinn-Phong terms (ka 0.5, kd 0.5, ks 0.8, shininess 30)."""
    import ctypes as C

    import numpy as np

    import oracle
    from cpp_volume_rendering_gb300 import abi, scene
    peak, peak_src = measured_peak_hbm()
    out = {"build": {}, "frames": {}}
    vols = {"512^3 u8 blobs": scene.synth_blobs(512, 512, 512, abi.CVR_U8, 32, seed=4020, noise_max=20.0),
            "256^3 u16 value noise": scene.synth_value_noise(256, 256, 256, abi.CVR_U16, seed=2000)}
    ms = C.c_float()
    for vname, vol in vols.items():
        ctx.set_volume(vol, (1.0, 1.0, 1.0))
        nvox = vol.size
        for mname, model in (("finite_differences", abi.GRADIENT_FINITE_DIFFERENCES),
                             ("sobel_feldman", abi.GRADIENT_SOBEL_FELDMAN)):
            gp = abi.GradientParams(model, 1, 0, 1)
            # the default builder (tensor-memory-accelerator plane streaming
            # where the row pitch allows) and the shared-memory ring builder
            for suffix, kern in (("", abi.GRADIENT_KERNEL_AUTO), (" tiled", abi.GRADIENT_KERNEL_TILED)):
                abi.check(lib.cvr_set_gradient_kernel(ctx.h, kern), ctx.h)
                for _ in range(2):
                    abi.check(lib.cvr_build_gradient(ctx.h, C.byref(gp)), ctx.h)
                times = []
                for _ in range(5):
                    abi.check(lib.cvr_flush_l2(ctx.h), ctx.h)
                    abi.check(lib.cvr_timer_start(ctx.h), ctx.h)
                    abi.check(lib.cvr_build_gradient(ctx.h, C.byref(gp)), ctx.h)
                    abi.check(lib.cvr_timer_stop(ctx.h, C.byref(ms)), ctx.h)
                    times.append(ms.value)
                m = statistics.median(times)
                algo = nvox * (vol.itemsize + 8)
                out["build"][f"{vname} {mname}{suffix}"] = {
                    "ms": m, "gvoxels_s": nvox / (m / 1000.0) / 1e9,
                    "builder": GRADIENT_BUILDERS.get(lib.cvr_get_gradient_kernel(ctx.h), "?"),
                    "roofline": {"bound": "hbm", "achieved": algo / (m / 1000.0) / 1e9, "peak": peak, "unit": "GB/s",
                                 "frac": algo / (m / 1000.0) / 1e9 / peak, "peak_source": peak_src,
                                 "algorithmic_bytes": algo}}
            abi.check(lib.cvr_set_gradient_kernel(ctx.h, abi.GRADIENT_KERNEL_AUTO), ctx.h)
    # CPU: the FP64 restatement of GenerateGradientTexture (the reference's own
    # loop, single-threaded like it) on a 128^3 sample of the u8 volume
    sample = np.ascontiguousarray(vols["512^3 u8 blobs"][192:320, 192:320, 192:320])
    orc = oracle.Oracle()
    orc.set_volume(sample, (1.0, 1.0, 1.0))
    t0 = time.perf_counter()
    orc.build_gradient(abi.GRADIENT_FINITE_DIFFERENCES)
    dt = time.perf_counter() - t0
    out["build"]["cpu_baseline"] = {"value": sample.size / dt / 1e9, "unit": "Gvoxels/s", "cores": 1, "kind": "port",
                                    "sample": f"finite differences on a 128^3 crop of the 512^3 u8 volume, FP64, "
                                              f"{dt:.2f} s"}
    ctx.build_gradient(abi.GRADIENT_NONE)
    for name in ("plain_large", "extinction"):
        w2 = scene.workload(name)
        if name == "plain_large":
            w2.light = scene.light(abi.LIGHT_POINT, position=(1.5, 2.5, 1.0))
        scene.prepare(ctx, w2)
        ctx.build_gradient(abi.GRADIENT_FINITE_DIFFERENCES)
        ctx.set_blinn_phong(True)
        try:
            out["frames"][name] = {"workload": WORKLOAD_DESC[name] + ", gradient Blinn-Phong (finite differences)",
                                   **tuned_frames(ctx, lib, w2)}
        finally:
            ctx.set_blinn_phong(False)
            ctx.build_gradient(abi.GRADIENT_NONE)
        log(f"gradient frame {name}: {out['frames'][name]['ms']:.3f} ms")
    return out


def postpass_section(ctx, lib, args, log=print):
    """Pixel multiscaling (BaseVolumeRenderer's MULTISCALING modes and
    RenderFrameToScreen's image kernels) as device post-passes.  Each pass
    alone on a 1024^2 output: multisample and down-scale from a rendered
    2048^2 frame, up-scale from a rendered 512^2 frame (the cardinal B-spline
    and o-MOMS up-scales include their digital prefilter of the source); HBM
    roofline on 16 bytes read per source pixel + 16 written per output pixel.
    Against the FP64 restatement of the passes on a 64^2 output.  Then whole
    multiscaled plain frames (256^3 u8 -> 1024^2) against the single-scale frame."""
    import ctypes as C

    import numpy as np

    from cpp_volume_rendering_gb300 import abi, scene
    from oracle import postpass as pp
    peak, peak_src = measured_peak_hbm()
    W = 1024
    fb_w = 32768
    buf = C.POINTER(C.c_float)()
    abi.check(lib.cvr_get_frame_buffer(ctx.h, fb_w, (2048 * 2048 + W * W + fb_w - 1) // fb_w, C.byref(buf)), ctx.h)
    base = C.cast(buf, C.c_void_p).value
    src, dst = C.c_void_p(base), C.c_void_p(base + 2048 * 2048 * 16)
    wl = scene.workload("plain_large")
    scene.prepare(ctx, wl)
    ms = C.c_float()

    def render_into(ptr, w, h):
        abi.check(lib.cvr_render(ctx.h, wl.method, C.byref(wl.cam), C.byref(wl.light), C.byref(wl.params),
                                 C.sizeof(wl.params), ptr, w, h, None, None), ctx.h)

    def timed(fn, reps=10):
        for _ in range(2):
            fn()
        ts = []
        for _ in range(reps):
            abi.check(lib.cvr_flush_l2(ctx.h), ctx.h)
            abi.check(lib.cvr_timer_start(ctx.h), ctx.h)
            fn()
            abi.check(lib.cvr_timer_stop(ctx.h, C.byref(ms)), ctx.h)
            ts.append(ms.value)
        return statistics.median(ts)

    names = ["box", "hat", "catmull_rom", "mitchell_netravali", "cardinal_bspline3", "cardinal_omoms3"]
    cases = [("multisample", abi.MULTISCALE_MULTISAMPLE, abi.FILTER_HAT, 2048)]
    cases += [("downscale", abi.MULTISCALE_DOWNSCALE, k, 2048) for k in range(6)]
    cases += [("upscale", abi.MULTISCALE_UPSCALE, k, 512) for k in range(6)]
    out = {"passes": {}, "frames": {}}
    rng = np.random.default_rng(5)
    rendered = None
    for mode_name, mode, k, sw in cases:
        if rendered != sw:
            render_into(src, sw, sw)
            rendered = sw
        m = timed(lambda: abi.check(lib.cvr_rescale_frame(ctx.h, mode, k, src, sw, sw, dst, W, W), ctx.h))
        algo = (sw * sw + W * W) * 16
        # the FP64 restatement on a 64^2 output (its sources scaled alike)
        ssw = 128 if sw > W else 32
        small = rng.uniform(0.0, 1.0, size=(ssw, ssw, 4))
        t0 = time.perf_counter()
        pp.rescale(small, mode, k, 64, 64)
        cpu_s = time.perf_counter() - t0
        out["passes"][f"{mode_name} {names[k]} {sw}^2 -> {W}^2"] = {
            "ms": m, "mpixels_s": W * W / (m / 1000.0) / 1e6,
            "roofline": {"bound": "hbm", "achieved": algo / (m / 1000.0) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": algo / (m / 1000.0) / 1e9 / peak, "peak_source": peak_src,
                         "algorithmic_bytes": algo},
            "cpu_baseline": {"value": 64 * 64 / cpu_s / 1e6, "unit": "Mpixels/s", "cores": 1, "kind": "port",
                             "sample": f"a 64^2 output from a {ssw}^2 source, FP64 restatement"}}
    # whole multiscaled frames through cvr_render
    out_ptr = dst
    single = statistics.median(time_frames(ctx, lib, wl, wl.params, out_ptr, 5, 2))
    out["frames"]["single 1024^2"] = {"ms": single}
    for label, mode, k in (("multisample hat (2048^2 generated)", abi.MULTISCALE_MULTISAMPLE, abi.FILTER_HAT),
                           ("downscale cardinal_omoms3 (2048^2 generated)", abi.MULTISCALE_DOWNSCALE,
                            abi.FILTER_CARDINAL_OMOMS3),
                           ("upscale catmull_rom (512^2 generated)", abi.MULTISCALE_UPSCALE, abi.FILTER_CATMULL_ROM),
                           ("upscale cardinal_bspline3 (512^2 generated)", abi.MULTISCALE_UPSCALE,
                            abi.FILTER_CARDINAL_BSPLINE3)):
        ctx.set_multiscaling(mode, k)
        try:
            t = statistics.median(time_frames(ctx, lib, wl, wl.params, out_ptr, 5, 2))
        finally:
            ctx.set_multiscaling(abi.MULTISCALE_SINGLE)
        out["frames"][label] = {"ms": t, "vs_single": t / single}
    out["workload"] = WORKLOAD_DESC["plain_large"]
    return out


def tables_section(ctx, lib, wl, log=print):
    """The table builders of the headline workload: the GPU extinction SAT
    (int64, HBM streaming: N^3 voxels read + (N+2)^3 8-byte cells written in the
    single-pass ideal) against the FP64 restatement of the reference's
    single-threaded SummedAreaTable3D::BuildSAT on the host, and the Gaussian
    extinction pyramid of the cone workload on the GPU."""
    import ctypes as C

    import oracle
    from cpp_volume_rendering_gb300 import abi, scene
    peak, peak_src = measured_peak_hbm()
    out = {}
    ext = wl.tf.ext_per_value(wl.dtype)
    ctx.set_volume(wl.volume, wl.spacing)
    ctx.set_transfer_function(wl.tf)
    ms = C.c_float()
    times = []
    for r in range(6):
        abi.check(lib.cvr_flush_l2(ctx.h), ctx.h)
        abi.check(lib.cvr_timer_start(ctx.h), ctx.h)
        abi.check(lib.cvr_build_sat(ctx.h, abi.dptr(ext), len(ext)), ctx.h)
        abi.check(lib.cvr_prepare_sat(ctx.h), ctx.h)
        abi.check(lib.cvr_timer_stop(ctx.h, C.byref(ms)), ctx.h)
        if r:
            times.append(ms.value)
    m = statistics.median(times)
    d, h, w = wl.volume.shape
    cells = (w + 2) * (h + 2) * (d + 2)
    algo = wl.volume.nbytes + cells * 8
    orc = oracle.Oracle()
    orc.set_volume(wl.volume, wl.spacing)
    t0 = time.perf_counter()
    orc.build_sat(ext)
    cpu_s = time.perf_counter() - t0
    out["sat"] = {"volume": [w, h, d], "gpu_ms": m, "gcells_s": cells / (m / 1000.0) / 1e9,
                  "roofline": {"bound": "hbm", "achieved": algo / (m / 1000.0) / 1e9, "peak": peak, "unit": "GB/s",
                               "frac": algo / (m / 1000.0) / 1e9 / peak, "peak_source": peak_src,
                               "algorithmic_bytes": algo},
                  "includes": "cvr_build_sat + cvr_prepare_sat: fixed-point table of the 65536 values + upload + "
                              "x-y plane prefixes + z pass (CUDA events)",
                  "cpu_baseline": {"value": cpu_s * 1000.0, "unit": "ms", "cores": 1, "kind": "port",
                                   "sample": f"the whole {w + 2}x{h + 2}x{d + 2} FP64 SAT, single-threaded "
                                             "(the reference's BuildSAT recurrence)"}}
    wc = scene.workload("cone")
    ctx.set_volume(wc.volume, wc.spacing)
    ctx.set_transfer_function(wc.tf)
    pyr_ms = {}
    for label, layout in (("plain", abi.LAYOUT_PLAIN), ("quads", abi.LAYOUT_QUADS)):
        # the base level's volume taps read the marchers' layout (same values)
        abi.check(lib.cvr_set_volume_layout(ctx.h, layout), ctx.h)
        times = []
        for r in range(4):
            abi.check(lib.cvr_flush_l2(ctx.h), ctx.h)
            abi.check(lib.cvr_timer_start(ctx.h), ctx.h)
            ctx.build_pyramid(**wc.pyramid)
            abi.check(lib.cvr_timer_stop(ctx.h, C.byref(ms)), ctx.h)
            if r:
                times.append(ms.value)
        pyr_ms[label] = statistics.median(times)
    abi.check(lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_PLAIN), ctx.h)
    out["pyramid"] = {"volume": list(wc.dims), "base": list(wc.pyramid["base_dims"]),
                      "levels": wc.pyramid["n_levels"], "gpu_ms": min(pyr_ms.values()),
                      "gpu_ms_by_layout": pyr_ms,
                      "note": "the 7x7x7 Gaussian of gen_extcoefvol_anysize / _mmlevel per level as one lattice "
                              "pass (the trilinear samples the 343 taps share) and three 7-tap passes, then the "
                              "opacity -> extinction pass"}
    log(f"tables: SAT {m:.3f} ms GPU vs {cpu_s * 1000:.0f} ms CPU, pyramid {out['pyramid']['gpu_ms']:.3f} ms")
    return out


def measured_peak_bf16():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["bf16_tflops"]), "measured"
        except Exception:
            pass
    return 1900.0, "fallback"


def surrogate_section(ctx, lib, args, log=print):
    """Trains the surrogate from scratch (cfg: up to 8M GT-labelled points of
    20 seeded blob volumes of 160^3..448^3, 60 epochs), then on the held-out 512^3 volume at 1024^2
    measures its RMSE and the cone method's against the ground-truth
    integrator, and the GT and surrogate frame times.  Leaves the surrogate
    workload prepared on ctx."""
    import ctypes as C
    from cpp_volume_rendering_gb300 import abi, scene
    t0 = time.perf_counter()
    ctx.mlp_init(scene.SURROGATE_SEED)
    abi.check(lib.cvr_mlp_set_training_data(ctx.h, None, None, 0), ctx.h)
    pts = scene.build_surrogate_training_set(ctx, points=args.surrogate_points)
    own = args.workload == "surrogate"
    t_data = time.perf_counter() - t0
    t0 = time.perf_counter()
    losses = scene.train_surrogate(ctx)
    t_train = time.perf_counter() - t0
    wl = scene.workload("surrogate", n=args.size if own else None, image=args.image if own else None)
    scene.prepare(ctx, wl)
    err = scene.evaluate_surrogate(ctx, wl)
    out = C.POINTER(C.c_float)()
    abi.check(lib.cvr_get_frame_buffer(ctx.h, wl.width, wl.height, C.byref(out)), ctx.h)
    optr = C.cast(out, C.c_void_p)
    # Both renderers tuned before timing, each over the sampling modes (FP32
    # volume samples, or texture-unit samples) and the autotuner's space (tile x
    # registers x brick for the ground truth on a 256^2 frame of the same view;
    # CTAs per SM x brick for the surrogate, whose persistent launch ignores the
    # tile, on a 512^2 frame).  The fastest configuration of each is timed.
    def tuned(method, size, flags_list):
        best = None
        for flags in flags_list:
            ctx.set_sampling(flags)
            tw, th, tv = C.c_int(), C.c_int(), C.c_int()
            abi.check(lib.cvr_autotune(ctx.h, method, C.byref(wl.cam), C.byref(wl.light), C.byref(wl.params),
                                       C.sizeof(wl.params), size, size, 1, C.byref(tw), C.byref(th), C.byref(tv),
                                       None), ctx.h)
            cfg = {"sampling": flags, "tile": [tw.value, th.value], "variant": tv.value,
                   "brick": lib.cvr_get_brick_size(ctx.h),
                  "quads": lib.cvr_get_volume_layout(ctx.h), "warp_w": lib.cvr_get_warp_shape(ctx.h),
              "refill": lib.cvr_get_ray_refill(ctx.h), "staging": lib.cvr_get_brick_staging(ctx.h)}
            wl.method = method
            reps = 2 if method == abi.GROUND_TRUTH else 3
            t = time_frames(ctx, lib, wl, wl.params, optr, reps, 1)
            if method != abi.SURROGATE:
                # the tuner ran on a smaller frame, where the ray refill's shorter
                # tail counts for more: its choice is checked again at full size
                abi.check(lib.cvr_set_ray_refill(ctx.h, 1 - cfg["refill"]), ctx.h)
                t2 = time_frames(ctx, lib, wl, wl.params, optr, reps, 1)
                if statistics.median(t2) < statistics.median(t):
                    t, cfg["refill"] = t2, 1 - cfg["refill"]
                abi.check(lib.cvr_set_ray_refill(ctx.h, cfg["refill"]), ctx.h)
            if best is None or statistics.median(t) < statistics.median(best[1]):
                best = (cfg, t)
        cfg = best[0]
        ctx.set_sampling(cfg["sampling"])
        abi.check(lib.cvr_set_tuning(ctx.h, cfg["tile"][0], cfg["tile"][1], cfg["variant"]), ctx.h)
        abi.check(lib.cvr_set_brick_size(ctx.h, cfg["brick"]), ctx.h)
        abi.check(lib.cvr_set_volume_layout(ctx.h, cfg["quads"]), ctx.h)
        abi.check(lib.cvr_set_warp_shape(ctx.h, cfg["warp_w"]), ctx.h)
        abi.check(lib.cvr_set_ray_refill(ctx.h, cfg["refill"]), ctx.h)
        abi.check(lib.cvr_set_brick_staging(ctx.h, cfg["staging"]), ctx.h)
        return best
    sampling_modes = (abi.SAMPLING_TEX_FEATURES, abi.SAMPLING_TEX_FEATURES | abi.SAMPLING_TEX_VOLUME)
    gt_tuning, tg = tuned(abi.GROUND_TRUTH, 256, sampling_modes)
    st_s, st_g = abi.FrameStats(), abi.FrameStats()
    abi.check(lib.cvr_render(ctx.h, abi.GROUND_TRUTH, C.byref(wl.cam), C.byref(wl.light), C.byref(wl.params),
                             C.sizeof(wl.params), optr, wl.width, wl.height, None, C.byref(st_g)), ctx.h)
    # the exact (FP32 volume samples) ground truth at its best tuning, for reference
    ctx.set_sampling(abi.SAMPLING_TEX_FEATURES)
    gt_fp32_tuning, tg32 = tuned(abi.GROUND_TRUTH, 256, (abi.SAMPLING_TEX_FEATURES,))
    sur_tuning, ts = tuned(abi.SURROGATE, 512, sampling_modes)
    abi.check(lib.cvr_render(ctx.h, abi.SURROGATE, C.byref(wl.cam), C.byref(wl.light), C.byref(wl.params),
                             C.sizeof(wl.params), optr, wl.width, wl.height, None, C.byref(st_s)), ctx.h)
    wl.method = abi.SURROGATE
    ms_s, ms_g = statistics.median(ts), statistics.median(tg)
    peak, src = measured_peak_bf16()
    tflops = st_s.shaded_samples * MLP_FLOP_PER_SAMPLE / (ms_s / 1000.0) / 1e12
    return {
        "workload": WORKLOAD_DESC["surrogate"], "volume": list(wl.dims), "image": [wl.width, wl.height],
        "training": {"points": pts, "volumes": scene.SURROGATE_VOLUMES, "epochs": len(losses),
                     "schedule": [list(x) for x in scene.SURROGATE_SCHEDULE], "batch": 4096,
                     "final_loss": losses[-1], "first_loss": losses[0], "data_s": t_data, "train_s": t_train},
        "heldout": {k: err[k] for k in ("rmse_ao", "rmse_shadow", "cone_rmse_ao", "cone_rmse_shadow", "points",
                                        "mean_ao", "mean_shadow", "max_err_ao", "shaded_samples")},
        "gt_ms": ms_g, "surrogate_ms": ms_s, "speedup_vs_gt": ms_g / ms_s,
        "gt_tuning": gt_tuning, "surrogate_tuning": sur_tuning,
        "gt_fp32_ms": statistics.median(tg32), "gt_fp32_tuning": gt_fp32_tuning,
        "speedup_vs_gt_fp32": statistics.median(tg32) / ms_s,
        "surrogate_fps": 1000.0 / ms_s, "surrogate_msamples_s": st_s.samples / (ms_s / 1000.0) / 1e6,
        "gt_msamples_s": st_g.samples / (ms_g / 1000.0) / 1e6,
        "mlp_tensor": {"achieved_tflops": tflops, "peak_tflops": peak, "frac": tflops / peak,
                       "peak_source": f"{src} (MEASURED_PEAKS.json bf16_tflops)",
                       "flop_per_inference": MLP_FLOP_PER_SAMPLE,
                       "note": "network FLOPs of the fused frame / frame time; the marcher is gather-bound, "
                               "the tensor pipe is far from its roofline by design"},
        "frame": {"samples": st_s.samples, "shaded_samples": st_s.shaded_samples},
    }


def apply_tuning(lib, ctx, tuning):
    """--tuning tile_w,tile_h,variant,warp_w,layout,refill[,brick edge] on ctx; returns the fields."""
    from cpp_volume_rendering_gb300 import abi
    t = [int(v) for v in tuning.split(",")]
    abi.check(lib.cvr_set_tuning(ctx.h, t[0], t[1], t[2]), ctx.h)
    abi.check(lib.cvr_set_warp_shape(ctx.h, t[3]), ctx.h)
    abi.check(lib.cvr_set_volume_layout(ctx.h, t[4]), ctx.h)
    abi.check(lib.cvr_set_ray_refill(ctx.h, t[5]), ctx.h)
    abi.check(lib.cvr_set_brick_size(ctx.h, t[6] if len(t) > 6 else 0), ctx.h)
    return t


def batch_section(ctx, lib, args, log=print):
    """The batched workload: 4 volumes of uneven size x 16 views (--batch-views)
    x 4 directional lights at 512^2, extinction and surrogate shading (512
    images), one CUDA graph of persistent launches; against the same jobs as
    512 cvr_render calls.  Uses the network on ctx (trained by the surrogate
    section when it ran).  --tuning fixes the marchers' configuration instead
    of tuning it on the largest extinction job."""
    import ctypes as C
    from cpp_volume_rendering_gb300 import abi, scene
    t0 = time.perf_counter()
    vols = scene.batch_volumes(args.batch_scale)
    scene.prepare_batch_volumes(ctx, vols)
    t_prep = time.perf_counter() - t0
    if not ctx.lib.cvr_mlp_training_size(ctx.h):  # no trained network on ctx: timing only
        ctx.mlp_init(7)
    W = 512
    views = args.batch_views
    probe = scene.batch_jobs(vols, n_views=views, image=W)
    n = len(probe.jobs)
    frames = C.POINTER(C.c_float)()
    fb_w = 32768  # one library-owned buffer holding all n frames
    abi.check(lib.cvr_get_frame_buffer(ctx.h, fb_w, (n * W * W + fb_w - 1) // fb_w, C.byref(frames)), ctx.h)
    base = C.cast(frames, C.c_void_p).value
    outs = [C.c_void_p(base + k * W * W * 16) for k in range(n)]
    b = scene.batch_jobs(vols, n_views=views, image=W, out_ptrs=outs)
    tw, th, tv, tms = C.c_int(), C.c_int(), C.c_int(), C.c_float()
    if args.tuning:
        apply_tuning(lib, ctx, args.tuning)
        abi.check(lib.cvr_get_tuning(ctx.h, C.byref(tw), C.byref(th), C.byref(tv)), ctx.h)
    else:
        # tuner: tile shape x register variant on the largest volume's first extinction job
        big = max(range(n), key=lambda k: (b.jobs[k].method == abi.EXTINCTION, vols[b.jobs[k].volume].size))
        jb = b.jobs[big]
        ctx.select_volume(jb.volume)
        abi.check(lib.cvr_autotune(ctx.h, jb.method, C.byref(jb.camera), C.byref(jb.light), C.c_void_p(jb.params),
                                   jb.params_size, W, W, 2, C.byref(tw), C.byref(th), C.byref(tv), C.byref(tms)),
                  ctx.h)
        ctx.select_volume(0)
    ms = C.c_float()

    def run_batch(idx):
        """Median device time of 3 replays of a batch of the jobs idx, and its samples."""
        arr = (abi.Job * len(idx))(*[b.jobs[k] for k in idx])
        bh = C.c_void_p()
        abi.check(lib.cvr_batch_create(ctx.h, arr, len(idx), C.byref(bh)), ctx.h)
        try:
            for _ in range(2):
                abi.check(lib.cvr_batch_run(bh), ctx.h)
            abi.check(lib.cvr_sync(ctx.h), ctx.h)
            times = []
            for _ in range(3):
                abi.check(lib.cvr_flush_l2(ctx.h), ctx.h)
                abi.check(lib.cvr_timer_start(ctx.h), ctx.h)
                abi.check(lib.cvr_batch_run(bh), ctx.h)
                abi.check(lib.cvr_timer_stop(ctx.h, C.byref(ms)), ctx.h)
                times.append(ms.value)
            smp = 0
            for k in range(len(idx)):
                st = abi.FrameStats()
                abi.check(lib.cvr_batch_job_stats(bh, k, C.byref(st)), ctx.h)
                smp += st.samples
        finally:
            lib.cvr_batch_destroy(bh)
        return statistics.median(times), smp

    def run_sequential(idx):
        """The same jobs as single cvr_render calls (one pass, device-timed as a whole)."""
        abi.check(lib.cvr_flush_l2(ctx.h), ctx.h)
        abi.check(lib.cvr_timer_start(ctx.h), ctx.h)
        for k in idx:
            j = b.jobs[k]
            abi.check(lib.cvr_select_volume(ctx.h, j.volume), ctx.h)
            abi.check(lib.cvr_render(ctx.h, j.method, C.byref(j.camera), C.byref(j.light), C.c_void_p(j.params),
                                     j.params_size, outs[k], W, W, None, None), ctx.h)
        abi.check(lib.cvr_timer_stop(ctx.h, C.byref(ms)), ctx.h)
        abi.check(lib.cvr_select_volume(ctx.h, 0), ctx.h)
        return ms.value

    every = list(range(n))
    med, tot = run_batch(every)
    seq_ms = run_sequential(every)
    per_method = {}
    for name, m in (("extinction", abi.EXTINCTION), ("surrogate", abi.SURROGATE)):
        idx = [k for k in every if b.jobs[k].method == m]
        bm, smp = run_batch(idx)
        sm = run_sequential(idx)
        per_method[name] = {"jobs": len(idx), "batch_ms": bm, "msamples_s": smp / (bm / 1000.0) / 1e6,
                            "sequential_ms": sm, "sequential_msamples_s": smp / (sm / 1000.0) / 1e6,
                            "speedup_vs_sequential": sm / bm}
    dims = ", ".join("x".join(str(e) for e in v.shape[::-1]) for v in vols)
    return {"workload": f"4 volumes ({dims}; u8, u16, u8, u16 value noise) x {views} views x "
                        f"4 directional lights x {{extinction, surrogate}} = {n} images of 512^2",
            "jobs": n, "batch_ms": med, "images_per_s": n / (med / 1000.0),
            "msamples_s": tot / (med / 1000.0) / 1e6, "by_method": per_method,
            "sequential_ms": seq_ms, "speedup_vs_sequential": seq_ms / med,
            "tuning": {"tile": [tw.value, th.value], "variant": tv.value, "brick": lib.cvr_get_brick_size(ctx.h),
                       "quads": lib.cvr_get_volume_layout(ctx.h), "warp_w": lib.cvr_get_warp_shape(ctx.h),
                       "refill": lib.cvr_get_ray_refill(ctx.h), "staging": lib.cvr_get_brick_staging(ctx.h)},
            "prepare_s": t_prep,
            "launch": "one CUDA graph: 2 memsets + the persistent extinction launch + persistent surrogate launches "
                      "of up to 32 jobs each (their descriptors as kernel parameters)"}


def run_ours(args):
    import ctypes as C

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    from cpp_volume_rendering_gb300 import abi, build, scene
    build.build()
    lib = abi.load()
    ctx = scene.Context(local)
    if args.batch_only:
        if rank == 0:
            emit("batch", batch_section(ctx, lib, args))
        ctx.close()
        return
    surrogate = None
    if args.workload == "surrogate" and args.no_surrogate:
        # profiling the frame alone: an untrained network of the same shape (the
        # network scales the samples' colour; opacity, and so every ray's
        # samples and the frame's work, come from the transfer function)
        ctx.mlp_init(7)
    elif args.workload == "surrogate":
        surrogate = surrogate_section(ctx, lib, args)
    wl = scene.workload(args.workload, n=args.size, image=args.image)
    scene.prepare(ctx, wl)
    out = C.POINTER(C.c_float)()
    abi.check(lib.cvr_get_frame_buffer(ctx.h, wl.width, wl.height, C.byref(out)), ctx.h)
    out_ptr = C.cast(out, C.c_void_p)
    params = wl.params
    # autotuner (part of set-up, outside the timed region): tile shape x register variant
    # x warp shape x layout x ray refill; --tuning fixes a configuration instead (profiling)
    tw, th, tv, tms = C.c_int(), C.c_int(), C.c_int(), C.c_float()
    if args.tuning:
        t = apply_tuning(lib, ctx, args.tuning)
        tw.value, th.value, tv.value = t[0], t[1], t[2]
    else:
        abi.check(lib.cvr_autotune(ctx.h, wl.method, C.byref(wl.cam), C.byref(wl.light), C.byref(params),
                                   C.sizeof(params), wl.width, wl.height, 3, C.byref(tw), C.byref(th),
                                   C.byref(tv), C.byref(tms)), ctx.h)
    tuning = {"tile": [tw.value, th.value], "variant": tv.value, "brick": lib.cvr_get_brick_size(ctx.h),
              "quads": lib.cvr_get_volume_layout(ctx.h), "warp_w": lib.cvr_get_warp_shape(ctx.h),
              "refill": lib.cvr_get_ray_refill(ctx.h), "staging": lib.cvr_get_brick_staging(ctx.h)}
    if not args.tuning:
        tuning["autotune_ms"] = round(tms.value, 4)  # the winner's time as the tuner measured it
    # one stats frame: sample counts are deterministic for a fixed frame
    st = abi.FrameStats()
    abi.check(lib.cvr_render(ctx.h, wl.method, C.byref(wl.cam), C.byref(wl.light), C.byref(params), C.sizeof(params),
                             out_ptr, wl.width, wl.height, None, C.byref(st)), ctx.h)
    # the roofline's denominator: L1 hit bandwidth of the marchers' 16-byte loads
    l1 = C.c_float()
    abi.check(lib.cvr_measure_l1_bandwidth(ctx.h, C.byref(l1)), ctx.h)
    barrier_max([0.0], ws)
    with ClockSampler(local) as clk:
        times = time_frames(ctx, lib, wl, params, out_ptr, args.steps, args.warmup)
    clocks = clk.summary()
    total_ms = sum(times)
    total_ms, = barrier_max([total_ms], ws)
    samples_all, = barrier_sum([float(st.samples * args.steps)], ws)
    value = samples_all / (total_ms / 1000.0) / 1e6
    ms_per_step = total_ms / args.steps
    # roofline of the dominant kernel (the marcher is the only launch per frame)
    alg = algorithmic_bytes(wl, st, abi)
    walk = bool(lib.cvr_get_walk_tables(ctx.h)) and wl.method == abi.EXTINCTION and wl.params.shadow_type == 1
    req = l1_request_bytes(wl, st, abi, walk)
    med_ms = statistics.median(times)
    achieved = req / (med_ms / 1000.0) / 1e9
    peak_hbm, peak_src = measured_peak_hbm()
    traffic, traffic_src = profile_traffic(args.workload)
    roofline = {"bound": "l1", "achieved": round(achieved, 1), "peak": round(l1.value, 1), "unit": "GB/s",
                "frac": round(achieved / l1.value, 4), "traffic": traffic,
                "peak_source": "measured in this run: cvr_measure_l1_bandwidth (coalesced 16-byte L1 hits)",
                "bytes_per_launch": req, "kernel_ms": round(med_ms, 4),
                "effective_gather_gbs": round(alg / (med_ms / 1000.0) / 1e9, 1),
                "note": "achieved = bytes the marcher's loads request from L1 per launch (walk-table shadow boxes: "
                        "4 x 32 B) / CUDA-event time; effective_gather_gbs counts the reference's 64 SAT texels "
                        "of 4 B per box query"}
    if traffic:
        roofline["hbm"] = {"achieved": round(traffic / (med_ms / 1000.0) / 1e9, 2), "peak": peak_hbm,
                           "frac": round(traffic / (med_ms / 1000.0) / 1e9 / peak_hbm, 5),
                           "peak_source": f"{peak_src} MEASURED_PEAKS.json hbm_gbs",
                           "traffic_source": f"profiles/{traffic_src}"}
    # end to end through the C ABI with host buffers
    vol = wl.volume
    nbytes = vol.nbytes
    pinned = C.c_void_p()
    abi.check(lib.cvr_host_alloc_pinned(nbytes, C.byref(pinned)))
    img_pinned = C.c_void_p()
    abi.check(lib.cvr_host_alloc_pinned(wl.width * wl.height * 16, C.byref(img_pinned)))
    C.memmove(pinned, vol.ctypes.data, nbytes)
    ext = wl.tf.ext_per_value(wl.dtype)
    d, h, w = vol.shape
    e2e_times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        abi.check(lib.cvr_set_volume(ctx.h, pinned, w, h, d, wl.dtype, *wl.spacing), ctx.h)
        if wl.method == abi.EXTINCTION:
            abi.check(lib.cvr_build_sat(ctx.h, abi.dptr(ext), len(ext)), ctx.h)
        if wl.method in (abi.CONE_DOS, abi.SURROGATE):
            ctx.build_pyramid(**wl.pyramid)
        abi.check(lib.cvr_render_host(ctx.h, wl.method, C.byref(wl.cam), C.byref(wl.light), C.byref(params),
                                      C.sizeof(params), C.cast(img_pinned, C.POINTER(C.c_float)), wl.width,
                                      wl.height, None), ctx.h)
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
    lib.cvr_host_free_pinned(pinned)
    lib.cvr_host_free_pinned(img_pinned)
    e2e_total, = barrier_max([sum(e2e_times)], ws)
    e2e = {"value": samples_all / e2e_total / 1e6, "unit": "Msamples/s",
           "h2d_bytes_per_step": int(nbytes + (ext.nbytes if wl.method == abi.EXTINCTION else 0)),
           "d2h_bytes_per_step": int(wl.width * wl.height * 16),
           "ms_per_step": round(1000.0 * e2e_total / args.steps, 3),
           "includes": "cvr_set_volume from pinned host memory + the table build (SAT or pyramid) + "
                       "cvr_render_host readback"}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl, target_s=args.cpu_seconds)
    if not args.quick:
        def reset_tuning():
            ctx.set_sampling(abi.SAMPLING_TEX_FEATURES)
            abi.check(lib.cvr_set_tuning(ctx.h, 16, 8, 0), ctx.h)
            abi.check(lib.cvr_set_brick_size(ctx.h, 0), ctx.h)
            abi.check(lib.cvr_set_volume_layout(ctx.h, abi.LAYOUT_PLAIN), ctx.h)
            abi.check(lib.cvr_set_warp_shape(ctx.h, 8), ctx.h)
            abi.check(lib.cvr_set_ray_refill(ctx.h, 0), ctx.h)
            abi.check(lib.cvr_set_brick_staging(ctx.h, 0), ctx.h)
        emit_here = rank == 0
        # the headline frame at its tuned configuration against the alternatives:
        # the persistent ray refill switched the other way, and (extinction) the
        # directional shadow's boxes through the equal-fraction query instead of
        # the walk table
        hv = {"workload": WORKLOAD_DESC[args.workload], "tuned_ms": med_ms, "tuning": tuning}
        was = lib.cvr_get_ray_refill(ctx.h)
        abi.check(lib.cvr_set_ray_refill(ctx.h, 1 - was), ctx.h)
        hv["refill_off_ms" if was else "refill_on_ms"] = statistics.median(
            time_frames(ctx, lib, wl, params, out_ptr, 3, 1))
        abi.check(lib.cvr_set_ray_refill(ctx.h, was), ctx.h)
        if walk:
            abi.check(lib.cvr_set_walk_tables(ctx.h, 0), ctx.h)
            hv["walk_tables_off_ms"] = statistics.median(time_frames(ctx, lib, wl, params, out_ptr, 3, 1))
            abi.check(lib.cvr_set_walk_tables(ctx.h, 1), ctx.h)
        if emit_here:
            emit("headline variants", hv)
        if surrogate is None and not args.no_surrogate:
            surrogate = surrogate_section(ctx, lib, args)
        if surrogate is not None and emit_here:
            emit("surrogate", surrogate)
        reset_tuning()
        if not args.no_batch:
            batch = batch_section(ctx, lib, args)
            if emit_here:
                emit("batch", batch)
        reset_tuning()
        # every renderer tuned on its own frame (tile x registers x brick), with
        # FP32 volume samples and with the texture-unit variant
        for name in ("plain", "plain_large", "cone", "ground_truth", "extinction_lightcache", "iso"):
            if name == args.workload:
                continue
            w2 = scene.workload("extinction" if name == "extinction_lightcache" else name)
            scene.prepare(ctx, w2)
            abi.check(lib.cvr_set_light_cache(ctx.h, *((32, 32, 32) if name == "extinction_lightcache" else (0, 0, 0))),
                      ctx.h)
            r = {"workload": WORKLOAD_DESC[name], **tuned_frames(ctx, lib, w2)}
            abi.check(lib.cvr_set_light_cache(ctx.h, 0, 0, 0), ctx.h)
            if rank == 0 and not args.no_cpu_baseline and name != "extinction_lightcache":
                # the FP32 oracle on the host cores, a few seconds of rows of the same frame
                r["cpu_baseline"] = cpu_baseline(w2, target_s=args.cpu_seconds / 3.0)
            if emit_here:
                emit(f"renderer {name}", r)
        reset_tuning()
        if not args.no_gradient:
            g = gradient_section(ctx, lib, args)
            if emit_here:
                emit("gradient", g)
        reset_tuning()
        if not args.no_postpass:
            pp = postpass_section(ctx, lib, args)
            if emit_here:
                emit("postpass", pp)
        reset_tuning()
        t = tables_section(ctx, lib, wl)
        if emit_here:
            emit("tables", t)
    ctx.close()
    if rank != 0:
        return
    # the headline: the LAST stdout line, compact
    if cpu is not None:
        cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    print(json.dumps({
        "metric": "Msamples/s", "value": round(value, 2), "unit": "Msamples/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded value noise / Gaussian blobs)",
        "config": {"workload": WORKLOAD_DESC[args.workload], "image": [wl.width, wl.height],
                   "volume": list(wl.dims), "l2": "flushed between timed steps (outside the events)",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU", "tuning": tuning},
        "fps": round(1000.0 / ms_per_step, 2),
        "frame": {"samples": st.samples, "shaded_samples": st.shaded_samples, "box_queries": st.aux_fetches},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": args.steps,
        "clocks": clocks}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="extinction", choices=list(WORKLOAD_DESC))
    ap.add_argument("--quick", action="store_true", help="skip the per-renderer table")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true",
                    help="skip training / evaluating the surrogate (with --workload surrogate: time the frame "
                         "with an untrained network)")
    ap.add_argument("--surrogate-points", type=int, default=8_000_000)
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-rendering section")
    ap.add_argument("--batch-views", type=int, default=16, help="views per volume and light of the batch")
    ap.add_argument("--batch-scale", type=float, default=1.0, help="edge scale of the batch's volumes (profiling)")
    ap.add_argument("--batch-only", action="store_true",
                    help="run the batched-rendering section alone (profiling; no headline line)")
    ap.add_argument("--no-gradient", action="store_true", help="skip the gradient Blinn-Phong section")
    ap.add_argument("--no-postpass", action="store_true", help="skip the pixel-multiscaling section")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--size", type=int, default=None, help="volume side override (profiling / small cases)")
    ap.add_argument("--image", type=int, default=None, help="image side override (profiling / small cases)")
    ap.add_argument("--tuning", default=None,
                    help="tile_w,tile_h,variant,warp_w,layout,refill[,brick edge]: skip the autotuner (profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
