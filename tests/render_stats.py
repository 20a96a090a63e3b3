"""Statistical comparison of Monte-Carlo renders at equal sample counts.

Two independent renders of the same estimator at the same spp differ only by noise; a
third render `x` is accepted as coming from the same estimator as the reference renders
`a` and `b` when
  * its per-value RMSE against `a` is no more than 1.3x the RMSE between `a` and `b`
    (a biased estimator adds its bias to this error), and
  * its image mean agrees with `a`'s within 3 standard deviations of the mean of the
    a-b difference plus 0.5 %.
"""
import numpy as np


def rmse(x, y):
    return float(np.sqrt(np.mean((np.asarray(x, np.float64) - np.asarray(y, np.float64)) ** 2)))


def rel_rmse(x, y, eps=1e-2):
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    return float(np.sqrt(np.mean(((x - y) / (y + eps)) ** 2)))


def assert_same_distribution(x, a, b, factor=1.3):
    floor = rmse(a, b)
    err = rmse(x, a)
    assert np.isfinite(x).all(), "non-finite pixels"
    assert err <= factor * floor + 1e-6, f"rmse vs reference {err:.5f} > {factor} x noise floor {floor:.5f}"
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    sd_mean = d.std() / np.sqrt(d.size)
    mx, ma = float(np.mean(x)), float(np.mean(a))
    assert abs(mx - ma) <= 3 * sd_mean * np.sqrt(2) + 5e-3 * abs(ma), f"image mean {mx:.5f} vs {ma:.5f}"
