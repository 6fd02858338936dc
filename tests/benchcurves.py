"""Comparison of simulated fields with the benchmark curves carried in the
reference's Su-Olson and Marshak-wave decks (tests/golden/benchmark_curves.npz,
written by tests/golden/make_benchmark_curves.py), shared by the oracle tests
and the GPU tests.

Tolerances, stated once:

* Su-Olson E_r(x) at t = 1 at the 12 XBENCH points: |mean - bench| <=
  3 sigma_mean + 2 % of bench + 0.002.  sigma_mean is the ensemble's standard
  error, interpolated like the mean; the 2 % covers the deck's own space and
  time discretisation (DX = 0.01, DT = 0.002) against the analytic curve, and
  0.002 the tail values near zero.
* Marshak T(x) at t = 2 at the 300 XBENCH points.  The curve is itself a
  Monte Carlo run (its cold tail scatters +-12 % around the initial 0.01), so:
  where the curve is above 0.75 (behind the front), |mean - bench| <=
  3 sigma_mean + 2 % of bench; the front (where T first falls below 0.3)
  within 0.0025 (5 cells) of the curve's; ahead of the front (curve below
  0.02, from 5 cells past the curve's front on), the mean temperature within
  5 % of the curve's mean there.
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CURVES = os.path.join(HERE, "golden", "benchmark_curves.npz")
ORACLE = os.path.join(HERE, "golden", "benchmark_oracle_fp64.npz")


def curve(name):
    c = np.load(CURVES)
    return c[name + "_x"], c[name + "_y"]


def _at(x, centers, values):
    return np.interp(x, centers, values)


def suolson_violations(centers, mean, sem):
    """XBENCH points where the E_r ensemble mean misses the curve."""
    xb, yb = curve("suolson")
    m, s = _at(xb, centers, mean), _at(xb, centers, sem)
    tol = 3.0 * s + 0.02 * yb + 0.002
    bad = np.abs(m - yb) > tol
    return [(float(a), float(b), float(c), float(d)) for a, b, c, d in zip(xb[bad], yb[bad], m[bad], tol[bad])]


def front(x, T, level=0.3):
    """First x at which T falls below `level` (linear interpolation)."""
    j = int(np.argmax(T < level))
    if j == 0:
        return float(x[0])
    return float(x[j - 1] + (x[j] - x[j - 1]) * (T[j - 1] - level) / (T[j - 1] - T[j]))


def marshak_violations(centers, mean, sem):
    """Where the T ensemble mean misses the Marshak curve (list of strings)."""
    xb, yb = curve("marshak")
    m, s = _at(xb, centers, mean), _at(xb, centers, sem)
    out = []
    hot = yb > 0.75
    bad = hot & (np.abs(m - yb) > 3.0 * s + 0.02 * yb)
    out += ["hot x=%.5f bench %.4f got %.4f" % (a, b, c) for a, b, c in zip(xb[bad], yb[bad], m[bad])]
    fb, fm = front(xb, yb), front(centers, mean)
    if abs(fb - fm) > 0.0025:
        out.append("front bench %.5f got %.5f" % (fb, fm))
    cold = (yb < 0.02) & (xb > fb + 0.0025)
    if abs(m[cold].mean() / yb[cold].mean() - 1.0) > 0.05:
        out.append("cold mean bench %.5f got %.5f" % (yb[cold].mean(), m[cold].mean()))
    return out


def oracle_z(name, mean_gpu, std_gpu, n_gpu, live):
    """Per-cell z-scores of an ensemble mean against the FP64 oracle
    ensemble of the same deck, over the cells selected by `live`."""
    o = np.load(ORACLE)
    mo, so, no = o[name + "_mean"], o[name + "_std"], len(o[name + "_seeds"])
    sel = live & ((so > 0) | (std_gpu > 0))
    return (mean_gpu - mo)[sel] / np.sqrt(std_gpu[sel] ** 2 / n_gpu + so[sel] ** 2 / no)
