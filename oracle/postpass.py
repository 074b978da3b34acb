"""TEST INFRASTRUCTURE ONLY — FP64 NumPy restatement of the pixel
multiscaling post-passes (vis::RenderFrameToScreen,
libs/vis_utils/renderoutputframe.cpp:265-539, and the compute shaders of
libs/vis_utils/shader/renderoutputframe/), the checker of csrc/postpass.cu.

Images are (h, w, 4) arrays, row 0 first.  texelFetch outside the frame
reads 0 (undefined in GL; zero under robust access).  The kernels and the
digital filters are pinned against the reference's CPU filter classes
(libs/vis_utils/filters/*.hpp, compiled by oracle/build_ref.py).
"""
from __future__ import annotations

import math

import numpy as np

BOX, HAT, CATMULL_ROM, MITCHELL_NETRAVALI, CARDINAL_BSPLINE3, CARDINAL_OMOMS3 = range(6)
MULTISAMPLE, DOWNSCALE, UPSCALE = 1, 2, 3

# Pre-factored LU decompositions of the digital filters (cbs_digital_filter.comp,
# comoms_digital_filter.comp; filters/bspline3.hpp:22-23, omoms3.hpp:30-32).
LU = {
    CARDINAL_BSPLINE3: [.2, .26315789, .26760563, .26792453, .26794742, .26794907, .26794918, .26794919],
    CARDINAL_OMOMS3: [.23529412, .33170732, .34266611, .34395774, .34411062, .34412872, .34413087, .34413112,
                      .34413115],
}


def support(k: int) -> float:
    return 1.0 if k == BOX else (2.0 if k == HAT else 4.0)


def weight(k: int, x: float) -> float:
    """kernel_weight of renderoutputframe/*_filter.comp."""
    if k == BOX:
        return 0.0 if (x <= -0.5 or x > 0.5) else 1.0
    x = abs(x)
    if k == HAT:
        return 0.0 if x > 1.0 else 1.0 - x
    if x > 2.0:
        return 0.0
    outer = x > 1.0
    u = 2.0 - x if outer else 1.0 - x
    if k == CATMULL_ROM:
        return ((.5 * u - .5) * u) * u if outer else ((-1.5 * u + 2.0) * u + .5) * u
    if k == MITCHELL_NETRAVALI:
        return (((7 / 18.0) * u - 1 / 3.0) * u) * u if outer else (((-7 / 6.0) * u + 1.5) * u + 0.5) * u + 1 / 18.0
    if k == CARDINAL_BSPLINE3:
        return (u * u) * u if outer else ((-3.0 * u + 3.0) * u + 3.0) * u + 1.0
    return ((.875 * u) * u + .125) * u if outer else ((-2.625 * u + 2.625) * u + 2.25) * u + 1.0


def _fetch(img, x, y):
    h, w = img.shape[:2]
    if x < 0 or y < 0 or x >= w or y >= h:
        return np.zeros(4)
    return img[y, x]


def multisample(src, w, h):
    """multisample_filter.comp: texture() (GL_LINEAR, clamp-to-edge) at the pixel centres."""
    sh, sw = src.shape[:2]
    out = np.zeros((h, w, 4))

    def tap(u, n):
        f = math.floor(u)
        return min(max(f, 0), n - 1), min(max(f + 1, 0), n - 1), u - f

    for y in range(h):
        b0, b1, tb = tap((y + 0.5) / h * sh - 0.5, sh)
        for x in range(w):
            a0, a1, ta = tap((x + 0.5) / w * sw - 0.5, sw)
            c0 = src[b0, a0] + ta * (src[b0, a1] - src[b0, a0])
            c1 = src[b1, a0] + ta * (src[b1, a1] - src[b1, a0])
            out[y, x] = c0 + tb * (c1 - c0)
    return out


def downscale(src, w, h, k):
    """downscaling_filter.comp main()."""
    sh, sw = src.shape[:2]
    out = np.zeros((h, w, 4))
    s = (h / sh) * (w / sw)
    kr = 0.5 * support(k)
    for jr in range(h):
        xr = (jr + 0.5) / h
        rows = range(math.ceil((xr - kr / h) * sh - 0.5), math.floor((xr + kr / h) * sh - 0.5) + 1)
        for jc in range(w):
            xc = (jc + 0.5) / w
            cols = range(math.ceil((xc - kr / w) * sw - 0.5), math.floor((xc + kr / w) * sw - 0.5) + 1)
            acc = np.zeros(4)
            for ir in rows:
                wr = weight(k, (xr - (ir + 0.5) / sh) * h)
                for ic in cols:
                    acc += wr * weight(k, (xc - (ic + 0.5) / sw) * w) * _fetch(src, ic, ir)
            out[jr, jc] = acc * s
    return out


def upscale(src, w, h, k):
    """upscaling_filter.comp main()."""
    sh, sw = src.shape[:2]
    out = np.zeros((h, w, 4))
    kr = 0.5 * support(k)
    for jr in range(h):
        xir = (jr + 0.5) / h * sh - 0.5
        for jc in range(w):
            xic = (jc + 0.5) / w * sw - 0.5
            acc = np.zeros(4)
            for ir in range(math.ceil(xir - kr), math.floor(xir + kr) + 1):
                wr = weight(k, xir - ir)
                for ic in range(math.ceil(xic - kr), math.floor(xic + kr) + 1):
                    acc += wr * weight(k, xic - ic) * _fetch(src, ic, ir)
            out[jr, jc] = acc
    return out


def linear_solve(L, f):
    """The digital filter along one line (the shaders' in-place LU solve with
    p_inv = 1); lines shorter than the table are returned unchanged."""
    f = np.array(f, dtype=np.float64)
    m, n = len(L), len(f)
    if n < m:
        return f
    L_inf = L[m - 1]
    v_inv = L_inf / (1.0 + L_inf)
    for i in range(1, n):
        f[i] -= (L[i - 1] if i < m else L_inf) * f[i - 1]
    f[n - 1] *= v_inv
    for i in range(n - 2, -1, -1):
        f[i] = (L_inf if i >= m - 1 else L[i]) * (f[i] - f[i + 1])
    return f


def digital_filter(img, k):
    """Rows (FilterDirection 0) then columns (1)."""
    if k not in LU:
        return img
    out = np.array(img, dtype=np.float64)
    for y in range(out.shape[0]):
        out[y] = linear_solve(LU[k], out[y])
    for x in range(out.shape[1]):
        out[:, x] = linear_solve(LU[k], out[:, x])
    return out


def rescale(src, mode, k, w, h):
    """The post-pass of a multiscaling mode: generated frame src -> (h, w, 4)."""
    src = np.asarray(src, np.float64)
    if mode == MULTISAMPLE:
        return multisample(src, w, h)
    if mode == DOWNSCALE:
        return digital_filter(downscale(src, w, h, k), k)
    return upscale(digital_filter(src, k), w, h, k)


def generated_size(mode, fw, fh, w, h):
    return (w // fw, h // fh) if mode == UPSCALE else (w * fw, h * fh)
