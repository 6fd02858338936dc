"""CPU checks of the surrogate's oracle (oracle/surrogate.py, orc_surr_walk):
its gradient against finite differences, BF16 rounding, the quantile
sampler, known answers of the in-cell walk, and the shared constants."""
import os
import re

import numpy as np

import oracle
import surrogate as S
from conftest import REPO


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    P = rng.normal(0.0, 0.3, S.N_PARAMS)
    n = 40
    x = rng.uniform(0.0, 1.0, (n, 4))
    x[:, 2] = rng.uniform(-1.0, 1.0, n)
    cls = rng.integers(0, 3, n)
    tgt = rng.normal(0.0, 1.0, (n, 2))
    _, g = S.loss_and_grad(P, x, cls, tgt)
    eps = 1e-6
    for i in rng.choice(S.N_PARAMS, 120, replace=False):
        Pp, Pm = P.copy(), P.copy()
        Pp[i] += eps
        Pm[i] -= eps
        fd = (S.loss_and_grad(Pp, x, cls, tgt)[0] - S.loss_and_grad(Pm, x, cls, tgt)[0]) / (2 * eps)
        assert abs(fd - g[i]) < 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -8 + 2.0 ** -20, -2.5, 0.0], np.float32)
    want = np.array([1.0, 1.0, 1.0 + 2.0 ** -6, 1.0 + 2.0 ** -7, -2.5, 0.0], np.float32)
    assert np.array_equal(S.bf16(v), want)


def test_knots_are_monotone_and_sampler_covers_the_extended_range():
    rng = np.random.default_rng(1)
    for _ in range(50):
        h = rng.normal(0.0, 3.0, 12)
        q = S.knots(h)
        assert np.all(np.diff(q) > 0.0)
        lo, hi = q[0] - 0.5 * (q[1] - q[0]), q[-1] + 0.5 * (q[-1] - q[-2])
        for u in rng.uniform(0.0, 1.0, 20):
            y = S.inv_cdf(q, u)
            assert lo <= y <= hi
        assert np.isclose(S.inv_cdf(q, 0.0), lo) and np.isclose(S.inv_cdf(q, 1.0), hi)
    # the median knot pair brackets u = 0.5
    q = S.knots(np.array([0.0, 0.5, 0.5, 0.5]))
    assert q[1] <= S.inv_cdf(q, 0.5) <= q[2]


def test_outcome_sampler_follows_softmax():
    out = np.zeros(64)
    out[:3] = [0.0, np.log(2.0), np.log(3.0)]  # p = 1/6, 2/6, 3/6
    us = (np.arange(6000) + 0.5) / 6000
    cls = [S.sample_outcome(out, u, 0.5, 0.5)[0] for u in us]
    assert np.allclose(np.bincount(cls, minlength=3) / 6000, [1 / 6, 2 / 6, 3 / 6], atol=1e-3)


def test_walk_without_reachable_faces_is_a_free_random_walk():
    """Faces beyond reach: every walk is truncated at lmax, and the
    displacement of an isotropic 1D-projected walk of path L has variance
    2L/3 (E[(mu s)^2] = E[mu^2] E[s^2] = 1/3 * 2 per unit mean free path)."""
    L, n = 400.0, 20000
    st = np.tile([1e6, 1e6, 0.5, L], (n, 1))
    _, c, t = oracle.surr_walk(7, st)
    assert np.all(c == S.TRUNC)
    disp = t[:, 0].astype(np.float64) * np.sqrt(L)
    var = disp.var()
    assert abs(var / (2.0 * L / 3.0) - 1.0) < 0.05, var
    assert abs(disp.mean() - 0.5) < 4.0 * np.sqrt(var / n)
    assert np.all(np.abs(t[:, 1]) <= 1.0)


def test_walk_exits_are_geometric():
    """Exit paths are at least the straight-line distance to the face and at
    most lmax; a face entry into a thick slab mostly comes back out."""
    rng = np.random.default_rng(2)
    n = 4000
    L = 10.0 ** rng.uniform(1.5, 4.0, n)
    dn = rng.uniform(0.0, 1.0, n) * L
    df = dn + rng.uniform(0.0, 1.0, n) * L
    mu = rng.uniform(-1.0, 1.0, n)
    st = np.stack([dn, df, mu, L], 1)
    _, c, t = oracle.surr_walk(3, st)
    path = np.exp(t[:, 0].astype(np.float64)) * L
    near, far = c == S.NEAR, c == S.FAR
    assert np.all(path[near] >= dn[near] * (1 - 1e-4))
    assert np.all(path[far] >= df[far] * (1 - 1e-4))
    assert np.all(path[near | far] <= L[near | far] * (1 + 1e-5))
    _, c2, _ = oracle.surr_walk(4, np.tile([0.0, 1e6, 0.7, 400.0], (20000, 1)))
    p_refl = np.mean(c2 == S.NEAR)
    assert 0.85 < p_refl < 0.98, p_refl


def test_constants_agree_with_the_cuda_header():
    hdr = open(os.path.join(REPO, "mixedprecisionimc.jl_gb300", "csrc", "imc_surrogate.cuh")).read()

    def const(name):
        return re.search(r"constexpr (?:int|float) %s = ([^;]+);" % name, hdr).group(1)
    assert const("kIn") == "4" and const("kHid") == "64" and const("kOut") == "64"
    assert re.search(r"kQL = 12, kQM = 6, kQP = 6", hdr)
    assert const("kNearL") == str(S.NEAR_L)
    imc_h = open(os.path.join(REPO, "include", "imc.h")).read()
    assert re.search(r"#define IMC_SURROGATE_PARAMS %d" % S.N_PARAMS, imc_h)
