"""Two-sample bands for the ensemble parity tests.

A cell is one (output, voxel[, species]) of an ensemble.  Each side is
summarised by (mean, variance with ddof=1, fourth central moment, n); the
difference of means is compared with its standard error
sqrt(v_a/n_a + v_b/n_b), the difference of variances with
sqrt(Var(s2_a) + Var(s2_b)), Var(s2) = (m4 - v^2 (n-3)/(n-1)) / n.
"""
import numpy as np


def moments_from_samples(x):
    """x [n, ...] -> (mean, var, m4, n) over the first axis."""
    x = np.asarray(x, np.float64)
    n = x.shape[0]
    mu = x.mean(0)
    d = x - mu
    return mu, (d * d).sum(0) / (n - 1), (d ** 4).mean(0), n


def moments_from_sums(s1, s2, s3, s4, n):
    """Raw sums of x, x^2, x^3, x^4 over n samples -> (mean, var, m4, n)."""
    mu = np.asarray(s1, np.float64) / n
    e2, e3, e4 = (np.asarray(a, np.float64) / n for a in (s2, s3, s4))
    var = (e2 - mu * mu) * n / (n - 1)
    m4 = e4 - 4 * mu * e3 + 6 * mu * mu * e2 - 3 * mu ** 4
    return mu, var, m4, n


def var_of_var(var, m4, n):
    return np.maximum(m4 - var * var * (n - 3) / (n - 1), 0.0) / n


def band_fractions(a, b, z=2.576, min_count=0.0):
    """Fractions of live cells whose mean and variance differences lie within
    z standard errors, and the number of live cells.  A cell is live when
    either side varies and, with min_count > 0, when the pooled mean times
    the smaller sample size reaches min_count (near-empty cells are
    discrete, and the normal bands do not hold there).  b's fourth moment
    may be None: a's then stands for both (the two ensembles share one
    distribution under the hypothesis tested)."""
    ma, va, qa, na = a
    mb, vb, qb, nb = b
    if qb is None:
        qb = qa
    live = (va > 0) | (vb > 0)
    if min_count > 0:
        live &= (ma * na + mb * nb) / (na + nb) * min(na, nb) >= min_count
    se_m = np.sqrt(va / na + vb / nb)
    se_v = np.sqrt(var_of_var(va, qa, na) + var_of_var(vb, qb, nb))
    fm = float(np.mean(np.abs(ma - mb)[live] <= z * se_m[live]))
    fv = float(np.mean(np.abs(va - vb)[live] <= z * se_v[live]))
    return fm, fv, int(live.sum())
