"""Per-pixel statistical parity between two Monte Carlo renders.

Each side gives per-pixel means m and mean squares q of n samples. Pixels are
pooled into pool x pool blocks: a block's mean is the mean of its pixel means,
and the variance of that mean is the sum of the pixels' sample variances over
(pool^4 n). Per (block, channel), z = (mean_a - mean_b) / sqrt(var_a + var_b).
At a few hundred samples per pixel, pooled over four pixels, the block means
are close to Gaussian, so under the null hypothesis a fraction of about
P(|z| > 3) = 0.27% of the z values exceed 3; the bound allows that fraction
plus four binomial standard deviations of it at the number of blocks tested.
Blocks with (numerically) zero variance on both sides must agree outright.
"""
import math

import numpy as np

P3 = 0.0027  # P(|z| > 3) for a standard normal


def _var(m, q, n):
    return np.maximum(q - m * m, 0.0) * n / max(n - 1, 1)


def _pool(a, p):
    H, W = a.shape[:2]
    H, W = H - H % p, W - W % p
    return a[:H, :W].reshape(H // p, p, W // p, p, -1)


def pooled_z(m_a, q_a, n_a, m_b, q_b, n_b, pool=2):
    """Returns (fraction of |z| > 3, number of z values, all-deterministic-agree,
    global z of the image means, z array)."""
    m_a, q_a, m_b, q_b = (np.asarray(x, np.float64) for x in (m_a, q_a, m_b, q_b))
    v_a, v_b = _var(m_a, q_a, n_a), _var(m_b, q_b, n_b)
    P = pool * pool
    ba, bb = _pool(m_a, pool).mean(axis=(1, 3)), _pool(m_b, pool).mean(axis=(1, 3))
    sa = _pool(v_a, pool).sum(axis=(1, 3)) / (P * P * n_a)
    sb = _pool(v_b, pool).sum(axis=(1, 3)) / (P * P * n_b)
    se = np.sqrt(sa + sb)
    det = se < 1e-7 * (1.0 + np.abs(bb))
    z = np.zeros_like(ba)
    z[~det] = (ba[~det] - bb[~det]) / se[~det]
    n = int((~det).sum())
    frac = float(np.mean(np.abs(z[~det]) > 3)) if n else 0.0
    det_ok = bool(np.all(np.abs(ba[det] - bb[det]) <= 1e-4 * (1 + np.abs(bb[det]))))
    g_se = math.sqrt(v_a.mean() / (n_a * m_a.size) + v_b.mean() / (n_b * m_b.size))
    gz = (m_a.mean() - m_b.mean()) / max(g_se, 1e-12)
    return frac, n, det_ok, gz, z


def bound(n):
    """Allowed fraction of |z| > 3 among n z values: 0.27% + 4 binomial sigma."""
    return P3 + 4.0 * math.sqrt(P3 * (1 - P3) / max(n, 1))


def assert_parity(name, m_a, q_a, n_a, m_b, q_b, n_b, pool=2, global_z=4.0):
    frac, n, det_ok, gz, _ = pooled_z(m_a, q_a, n_a, m_b, q_b, n_b, pool)
    print(f"ZSTAT {name}: {frac:.5f} of {n} block channels beyond 3 sigma (bound {bound(n):.5f}), "
          f"global z {gz:.2f}")
    assert det_ok, f"{name}: zero-variance blocks disagree"
    assert n > 0, f"{name}: nothing to test"
    assert frac <= bound(n), f"{name}: {frac:.5f} of {n} beyond 3 sigma (bound {bound(n):.5f})"
    assert abs(gz) < global_z, f"{name}: global mean z = {gz:.2f}"
    return frac, n, gz
