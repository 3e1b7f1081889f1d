"""The float-float primary-ray arithmetic of the wave engine, restated in numpy.

`primary_ray` (beamcast-gx-v1.0-beta-_gb300/csrc/render.cu) computes the camera
ray in float-float arithmetic on the fp32 pipe: Knuth's TwoSum, the FMA form of
Dekker's TwoProduct and Dekker's add2, from hi + lo pairs of the host's fp64
basis and sample tables. This test runs the same operation sequence in numpy
float32 (an fp32 FMA is emulated exactly enough through float64, which holds
every product of two fp32 values exactly) and compares it with the reference's
fp64 camera arithmetic (adaptivePixel, renderer.go:1940-1950, as the oracle
restates it): the float-float direction must lie within 2^-40 of the fp64 one,
relative to the camera vectors, and its fp32 rounding must equal the fp64
direction's on all but a vanishing share of components, never by more than one
unit in the last place.
"""
import numpy as np
import pytest

from bcgx import scenes
from bcgx.settings import Camera

f32, f64 = np.float32, np.float64


def _two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def _fast_two_sum(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def _add(a, b):
    s_hi, s_lo = _two_sum(a[0], b[0])
    return _fast_two_sum(s_hi, f32(s_lo + f32(a[1] + b[1])))


def _fma(a, b, c):
    return f32(f64(a) * f64(b) + f64(c))


def _mul(a, b):
    p = f32(a[0] * b[0])
    e = _fma(a[0], b[0], -p)
    e = _fma(a[0], b[1], e)
    e = _fma(a[1], b[0], e)
    return _fast_two_sum(p, e)


def _split(v):
    hi = f32(v)
    return hi, f32(f64(v) - f64(hi))


def _ulp_diff(a, b):
    ia = a.astype(np.float32).view(np.int32).astype(np.int64)
    ib = b.astype(np.float32).view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return np.abs(ia - ib)


@pytest.mark.parametrize("W,H,seed", [(2560, 1440, 1), (320, 240, 2), (1921, 1079, 3)])
def test_float_float_primary_rays_match_fp64(orc, W, H, seed):
    rng = np.random.default_rng(seed)
    cam = Camera(tuple(rng.uniform(-50, 50, 3)), tuple(rng.uniform(-5, 5, 3)), (0.0, 1.0, 0.0),
                 float(rng.uniform(20, 90)))
    origin, lower, horiz, vert = orc.camera_basis(cam, W / H)
    X, Y = orc.sample_sequence(1, 256)  # Halton
    n = 200_000
    x = rng.integers(0, W, n)
    y = rng.integers(0, H, n)
    s = rng.integers(0, len(X), n)
    rot = np.array([orc.pixel_sample_rotation(int(a), int(b)) for a, b in zip(x[:4096], y[:4096])])
    rot = np.concatenate([rot] * (n // 4096 + 1))[:n]
    x, y = x[:n], y[:n]  # pixels beyond the first 4096 reuse their rotations: the arithmetic is what is tested

    # fp64, in the reference's operation order
    a = X[s] + rot[:, 0]
    b = Y[s] + rot[:, 1]
    jx64, jy64 = a - np.floor(a), b - np.floor(b)
    u64 = (x + jx64) / max(W - 1, 1)
    v64 = ((H - 1 - y) + jy64) / max(H - 1, 1)
    d64 = lower[None, :] + horiz[None, :] * u64[:, None] + vert[None, :] * v64[:, None] - origin[None, :]

    # float-float, in primary_ray's operation order
    h1 = np.round(rot[:, 0] * 2.0 ** 32).astype(np.uint64)
    h2 = np.round(rot[:, 1] * 2.0 ** 32).astype(np.uint64)
    rx = (f32((h1 >> 8).astype(np.float64) * 2.0 ** -24), f32((h1 & 255).astype(np.float64) * 2.0 ** -32))
    ry = (f32((h2 >> 8).astype(np.float64) * 2.0 ** -24), f32((h2 & 255).astype(np.float64) * 2.0 ** -32))
    qx, qy = _split(X[s]), _split(Y[s])

    def wrap(t):
        ge = (t[0] > 1) | ((t[0] == 1) & (t[1] >= 0))
        w = _fast_two_sum(f32(t[0] - f32(1)), t[1])
        return np.where(ge, w[0], t[0]), np.where(ge, w[1], t[1])

    jx, jy = wrap(_add(qx, rx)), wrap(_add(qy, ry))
    zero = np.zeros(n, np.float32)
    u = _mul(_add((x.astype(np.float32), zero), jx), _split(np.full(n, 1.0 / max(W - 1, 1))))
    v = _mul(_add(((H - 1 - y).astype(np.float32), zero), jy), _split(np.full(n, 1.0 / max(H - 1, 1))))
    d_ff = np.empty((n, 3))
    d_hi = np.empty((n, 3), np.float32)
    for k in range(3):
        base = _split(np.full(n, lower[k] - origin[k]))
        su, sv = _split(np.full(n, horiz[k])), _split(np.full(n, vert[k]))
        t = _add(_add(base, _mul(su, u)), _mul(sv, v))
        d_hi[:, k] = t[0]
        d_ff[:, k] = f64(t[0]) + f64(t[1])

    scale = np.abs(lower - origin) + np.abs(horiz) + np.abs(vert)
    err = np.abs(d_ff - d64) / scale[None, :]
    assert err.max() < 2.0 ** -40, err.max()
    ulps = _ulp_diff(d_hi, d64.astype(np.float32))
    assert ulps.max() <= 1, ulps.max()
    assert np.mean(ulps > 0) < 1e-4, np.mean(ulps > 0)
