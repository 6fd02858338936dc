"""GPU checks of the learned surrogate against its oracle: the in-cell walk
that makes the training data, the FP32 training gradient, the BF16 tensor-
core forward pass, the inverse-transform sampler, and a trained network's
outcome statistics against analog walks."""
import numpy as np
import pytest

import oracle
import surrogate as S

pytestmark = pytest.mark.gpu


def _states(rng, n, lo=1.5, hi=4.0):
    L = 10.0 ** rng.uniform(lo, hi, n)
    dn = rng.uniform(0.0, 1.25, n) * L
    dn[: n // 3] = 0.0
    df = dn + rng.uniform(0.0, 1.25, n) * L
    mu = rng.uniform(-1.0, 1.0, n)
    mu[: n // 3] = rng.uniform(0.01, 1.0, n // 3)
    return np.stack([dn, df, mu, L], 1).astype(np.float32)


def test_walk_matches_oracle(gpu_lib):
    """Same Philox variates, same FP32 operations: the outcome agrees walk by
    walk (a last-bit difference of a logarithm may flip a rare tie), and the
    targets agree to FP32 rounding where the outcome does."""
    from mpimc import surrogate as G
    st = _states(np.random.default_rng(10), 3000)
    x, c, t = G.walk(123, st)
    xo, co, to = oracle.surr_walk(123, st)
    same = c == co
    assert same.mean() >= 0.995, same.mean()
    assert np.allclose(x, xo, rtol=1e-6, atol=1e-6)
    d = np.abs(t[same] - to[same])
    assert np.median(d) < 1e-6 and np.mean(d < 1e-3) >= 0.99, (np.median(d), np.mean(d < 1e-3))


def test_training_states_cover_the_domain(gpu_lib):
    from mpimc import surrogate as G
    x, c, t = G.walk(5, None, 200000)
    assert np.all((x[:, :2] >= 0.0) & (x[:, :2] <= 1.0))
    assert np.all(np.abs(x[:, 2]) <= 1.0) and np.all(x[:, 2] != 0.0)
    # lmax on [40, 1.2e4]: (log10 lmax - 2)/2 on [-0.199, 1.040]
    assert x[:, 3].min() < -0.19 and x[:, 3].max() > 1.03
    frac = np.bincount(c, minlength=3) / len(c)
    assert np.all(frac > 0.05), frac
    assert np.all(np.isfinite(t))


def test_gradient_matches_oracle(gpu_lib):
    """The FP32 per-slice forward/backward with the block-order reduction
    equals the FP64 oracle gradient to FP32 accuracy (relative L2 < 1e-4)."""
    from mpimc import surrogate as G
    rng = np.random.default_rng(11)
    x, c, t = G.walk(77, None, 1000)
    P = np.zeros(S.N_PARAMS)
    for (wo, bo, fan) in ((S.W1, S.B1, 4), (S.W2, S.B2, 64), (S.W3, S.B3, 64), (S.W4, S.B4, 64)):
        P[wo:bo] = rng.uniform(-1.0, 1.0, bo - wo) * np.sqrt(6.0 / fan)
        P[bo:bo + 64] = rng.normal(0.0, 0.1, 64)
    P = P.astype(np.float32)
    loss, g = G.grad(P, x, c, t)
    lo, go = S.loss_and_grad(P.astype(np.float64), x, c, t)
    assert abs(loss - lo) < 1e-5 * abs(lo), (loss, lo)
    rel = np.linalg.norm(g - go) / np.linalg.norm(go)
    assert rel < 1e-4, rel
    for name, a, b in (("W1", S.W1, S.B1), ("W2", S.W2, S.B2), ("W4", S.W4, S.B4), ("b4", S.B4, S.N_PARAMS)):
        r = np.linalg.norm(g[a:b] - go[a:b]) / max(np.linalg.norm(go[a:b]), 1e-30)
        assert r < 1e-3, (name, r)


def test_forward_matches_bf16_oracle(gpu_lib):
    """The warp-level m16n8k16 BF16 pass equals the BF16-rounded oracle up to
    FP32 summation order, and the FP64 network to BF16 accuracy; ragged n."""
    from mpimc import surrogate as G
    P = G.train(seed=3, n_samples=1 << 16, batch=1024, iterations=200)
    rng = np.random.default_rng(12)
    x = np.concatenate([G.walk(9, None, 1000)[0], rng.uniform(-1.0, 1.0, (37, 4)).astype(np.float32)])
    out = G.forward(P, x)
    ob = S.forward_bf16(P, x)
    of = S.forward(P, x)
    scale = np.abs(of).max()
    assert np.max(np.abs(out - ob)) < 2e-3 * scale, np.max(np.abs(out - ob)) / scale
    assert np.max(np.abs(out - of)) < 5e-2 * scale, np.max(np.abs(out - of)) / scale
    assert np.array_equal(G.forward(P, x[:5]), out[:5])


def test_sampler_matches_oracle(gpu_lib):
    """k_surr_sample draws the same outcome and targets as the oracle's
    sampler fed with the network outputs and the same Philox uniforms."""
    from mpimc import surrogate as G
    P = G.train(seed=4, n_samples=1 << 16, batch=1024, iterations=200)
    st = _states(np.random.default_rng(13), 500)
    c, y0, y1 = G.sample(P, 99, st)
    out = G.forward(P, S.features(st).astype(np.float32))
    agree = 0
    for r in range(len(st)):
        u = oracle.philox_uniforms(99, 0, r, 4, 3)
        co, a, b = S.sample_outcome(out[r].astype(np.float64), *u)
        if co == c[r]:
            agree += 1
            assert abs(a - y0[r]) < 1e-4 * (1 + abs(a)) and abs(b - y1[r]) < 1e-4 * (1 + abs(b)), (r, a, y0[r], b, y1[r])
    assert agree >= len(st) - 2


def test_training_converges(surrogate_params):
    P, loss = surrogate_params
    assert np.all(np.isfinite(loss)) and np.all(np.isfinite(P))
    first, last = loss[:100].mean(), loss[-500:].mean()
    assert last < 0.6 * first, (first, last)


def test_trained_outcomes_match_analog_walks(surrogate_params):
    """At fixed states across the domain, the sampled outcome probabilities
    agree with 20,000 analog walks each to 0.03; the exit path to 10 % in
    the median and 20 % in the mean (the quantile heads end half a knot
    spacing beyond the last knot, which trims the heavy tail of long returns);
    the truncation displacement to 0.1 sqrt(lmax) + 10 %."""
    from mpimc import surrogate as G
    P, _ = surrogate_params
    n = 20000
    cases = [(5.0, 300.0, 0.6, 200.0), (20.0, 2000.0, 0.3, 5000.0), (15.0, 25.0, -0.2, 100.0),
             (30.0, 100.0, 0.9, 100.0), (800.0, 900.0, 0.1, 1000.0), (6.0, 12.0, 0.5, 64.0)]
    for k, case in enumerate(cases):
        st = np.tile(np.array(case, np.float32), (n, 1))
        cw, tw = G.walk(1000 + k, st)[1:]
        cs, y0, y1 = G.sample(P, 2000 + k, st)
        pw = np.bincount(cw, minlength=3) / n
        ps = np.bincount(cs, minlength=3) / n
        assert np.max(np.abs(pw - ps)) < 0.03, (case, pw, ps)
        for cl in (S.NEAR, S.FAR):
            if pw[cl] > 0.1 and ps[cl] > 0.1:
                lw, ls = np.exp(tw[cw == cl, 0]), np.exp(y0[cs == cl])
                assert abs(np.median(lw) - np.median(ls)) < 0.10 * np.median(lw), (case, cl, np.median(lw), np.median(ls))
                assert abs(lw.mean() - ls.mean()) < 0.20 * lw.mean(), (case, cl, lw.mean(), ls.mean())
        if pw[S.TRUNC] > 0.1 and ps[S.TRUNC] > 0.1:
            dw = tw[cw == S.TRUNC, 0].mean()
            ds = y0[cs == S.TRUNC].mean()
            assert abs(dw - ds) < 0.1 + 0.1 * abs(dw), (case, dw, ds)


@pytest.mark.parametrize("dn,mup", [(6.0, 0.4), (15.0, -0.7), (2.0, 0.9)])
def test_walk_generator_equals_transport_kernel_walks(gpu_lib, dn, mup):
    """The training walks (imc_surrogate_walk) are the plain transport kernel's
    in-cell walks: 200,000 histories started in one state inside a thick cell
    (tests/golden/decks/walk_cell.txt: 40 mean free paths of effective scatter,
    lmax = the census path, 399 mean free paths) and moved by the FP32
    transport kernel, against 200,000 generator walks from the same
    (d_n, d_f, mu', lmax).  A history that leaves the cell reaches census in
    the transparent buffer on its side, so the census cell gives the exit
    face and the census direction the exit |mu|.  Outcome fractions agree
    within 4 binomial sigma, mean exit |mu| and mean ln(exit path / lmax)
    within 4 sigma."""
    import mpimc
    from mpimc import surrogate as G
    from conftest import load_deck
    inputs, mesh = load_deck("walk_cell", NMAX="400000")
    e = mpimc.Engine(inputs, mesh)
    e.update()
    f, sa = e.field("fleck")[1], e.field("sigma_a")[1]
    seff = sa * (1.0 - f)
    W = 0.05 * seff
    lmax = 0.5 * seff  # c dt seff, from t = 0; the cut-off path is ~4.6x longer
    n = 200000
    e.set_particles({"t": np.zeros(n), "x": np.full(n, dn / seff), "mu": np.full(n, mup), "E": np.ones(n),
                     "E0": np.ones(n), "cell": np.ones(n, np.int32)})
    e.transport()
    p = e.particles()
    e.close()
    alive = p["E0"] >= 0
    assert alive.all()  # every history reaches census (in the cell or a buffer)
    cell, mu, x = p["cell"], p["mu"], p["x"]
    cls_t = np.where(cell == 1, 2, np.where(cell == 0, 0, 1))  # near face is the left one (dn < W / 2)
    # exit time from the distance streamed in the buffer (no collisions there)
    dx0 = 0.6
    left = cell == 0
    t_exit_l = 0.5 - (dx0 - x[left]) / np.abs(mu[left])
    lpath_t = np.log(t_exit_l * seff / lmax)
    st = np.tile(np.array([[dn, W - dn, mup, lmax]], np.float32), (n, 1))
    xw, cls_w, tgt_w = G.walk(4242, st)
    for k in range(3):
        pt, pw = np.mean(cls_t == k), np.mean(cls_w == k)
        sd = np.sqrt(max(pt * (1 - pt), pw * (1 - pw), 1e-6) * 2.0 / n)
        assert abs(pt - pw) < 4 * sd, (k, pt, pw)
    mu_t, mu_w = np.abs(mu[left]), tgt_w[cls_w == 0, 1]
    assert abs(mu_t.mean() - mu_w.mean()) < 4 * np.sqrt(mu_t.var() / len(mu_t) + mu_w.var() / len(mu_w))
    lw = tgt_w[cls_w == 0, 0]
    assert abs(lpath_t.mean() - lw.mean()) < 4 * np.sqrt(lpath_t.var() / len(lpath_t) + lw.var() / len(lw))
