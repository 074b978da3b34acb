"""The x-y quad layout's lookup rule, restated on the CPU: a GL_LINEAR
clamp-to-edge trilinear lookup equals the lookup that raises the x and y
texel coordinates to 0, reads the four x-y taps of a plane from one cell of
the quad copy (successors clamped at the high faces) and the two planes from
two cells.  The device kernels (sample_volume, pyr_sample_level) implement
this rule; the GPU tests check their frames bit for bit against the plain
layout."""
import numpy as np


def _tap(u, n):
    fl = np.floor(u)
    i = int(fl)
    return min(max(i, 0), n - 1), min(max(i + 1, 0), n - 1), u - fl


def _lerp(t, a, b):
    return t * (b - a) + a


def trilinear_plain(v, u):
    d, h, w = v.shape
    x0, x1, tx = _tap(u[0], w)
    y0, y1, ty = _tap(u[1], h)
    z0, z1, tz = _tap(u[2], d)
    c = [[_lerp(tx, v[z, y, x0], v[z, y, x1]) for y in (y0, y1)] for z in (z0, z1)]
    return _lerp(tz, _lerp(ty, c[0][0], c[0][1]), _lerp(ty, c[1][0], c[1][1]))


def quad_copy(v):
    d, h, w = v.shape
    xs = np.minimum(np.arange(w) + 1, w - 1)
    ys = np.minimum(np.arange(h) + 1, h - 1)
    return np.stack([v, v[:, :, xs], v[:, ys, :], v[:, ys][:, :, xs]], axis=-1)


def trilinear_quads(q, u):
    d, h, w, _ = q.shape
    x0, _, tx = _tap(max(u[0], 0.0), w)
    y0, _, ty = _tap(max(u[1], 0.0), h)
    z0, z1, tz = _tap(u[2], d)
    a, b = q[z0, y0, x0], q[z1, y0, x0]
    c0 = _lerp(ty, _lerp(tx, a[0], a[1]), _lerp(tx, a[2], a[3]))
    c1 = _lerp(ty, _lerp(tx, b[0], b[1]), _lerp(tx, b[2], b[3]))
    return _lerp(tz, c0, c1)


def test_quad_lookup_equals_clamp_to_edge_lookup():
    rng = np.random.default_rng(2)
    for shape in ((5, 7, 9), (1, 3, 2), (4, 1, 1), (2, 2, 6)):
        v = rng.integers(0, 65536, size=shape).astype(np.float64)
        q = quad_copy(v)
        d, h, w = shape
        # texel coordinates inside, on the faces and beyond them on every side
        for _ in range(400):
            u = rng.uniform(-2.0, 1.0, 3) + rng.uniform(0.0, 1.0, 3) * np.array([w + 2, h + 2, d + 2])
            assert trilinear_quads(q, u) == trilinear_plain(v, u), (shape, u)
        for u in ([-0.5, -0.5, -0.5], [0.0, 0.0, 0.0], [w - 1.0, h - 1.0, d - 1.0], [w - 0.5, h - 0.5, d - 0.5]):
            u = np.array(u)
            assert trilinear_quads(q, u) == trilinear_plain(v, u), (shape, u)
