"""Binning error estimate for correlated series (test-side; the product's own estimator
is nmmc_binning)."""
import numpy as np


def binned_error(x, min_bins=32):
    x = np.asarray(x, float)
    best = x.std(ddof=1) / np.sqrt(len(x))
    while len(x) >= 2 * min_bins:
        x = 0.5 * (x[: len(x) // 2 * 2 : 2] + x[1 : len(x) // 2 * 2 : 2])
        best = max(best, x.std(ddof=1) / np.sqrt(len(x)))
    return best
