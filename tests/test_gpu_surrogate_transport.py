"""GPU tests of transport with the learned thick-cell surrogate: exact
fallback to the analog path, reproducibility, temperatures against the analog
ensemble on the thick-slab deck, and the work it saves there."""
import numpy as np
import pytest

from conftest import load_deck

pytestmark = pytest.mark.gpu


def _run(deck, seed, params=None, **ov):
    import mpimc
    inputs, mesh = load_deck(deck, SEED=str(seed), **ov)
    e = mpimc.Engine(inputs, mesh)
    if params is not None:
        e.set_surrogate(params)
    steps, _ = e.run()
    out = dict(temp=e.field("temp"), rad=e.field("radenergydens"), steps=steps,
               segments=sum(s["segments"] for s in steps), calls=sum(s["surrogate_calls"] for s in steps))
    e.close()
    return out


def test_surrogate_needs_1d_and_fp32_or_fp16(surrogate_params):
    import mpimc
    P, _ = surrogate_params
    for deck, ov in (("tiny_2d", {"precision": 1}), ("thick_slab", {"precision": 0, "scale_select_precision": 0})):
        inputs, mesh = load_deck(deck)
        e = mpimc.Engine(inputs, mesh, ov)
        with pytest.raises(mpimc.ImcError):
            e.set_surrogate(P)
        assert not e.surrogate_active()
        e.close()
    inputs, mesh = load_deck("thick_slab")
    e = mpimc.Engine(inputs, mesh)
    with pytest.raises(mpimc.ImcError):
        e.set_surrogate(P[:100])
    e.set_surrogate(P)
    assert e.surrogate_active()
    e.set_surrogate(None)
    assert not e.surrogate_active()
    e.close()


def test_surrogate_off_is_the_analog_path(surrogate_params):
    """Turning the surrogate on and off again leaves the analog kernels,
    bit for bit."""
    import mpimc
    P, _ = surrogate_params
    a = _run("thick_slab", 11, NINPUT="20000", NMAX="200000")
    inputs, mesh = load_deck("thick_slab", SEED="11", NINPUT="20000", NMAX="200000")
    e = mpimc.Engine(inputs, mesh)
    e.set_surrogate(P)
    e.set_surrogate(None)
    e.run()
    assert np.array_equal(e.field("temp"), a["temp"])
    e.close()


def test_surrogate_transport_is_reproducible(surrogate_params):
    P, _ = surrogate_params
    a = _run("thick_slab", 12, P, NINPUT="20000", NMAX="200000")
    b = _run("thick_slab", 12, P, NINPUT="20000", NMAX="200000")
    assert a["calls"] > 0
    assert np.array_equal(a["temp"], b["temp"]) and np.array_equal(a["rad"], b["rad"])
    assert a["segments"] == b["segments"] and a["calls"] == b["calls"]
    for s in a["steps"][:-1]:
        assert abs(s["energy_error"]) < 1e-5 and s["error_flags"] == 0


def test_surrogate_gain_on_thick_slab(surrogate_params):
    """Thick slab (40 mean free paths per cell, ~400 collisions per history
    per step): with the surrogate the analog segments fall at least 2-fold,
    and the ensemble-mean temperature agrees with the analog ensemble --
    per cell within 4 sigma, within 3 sigma on average (rms z < 1.6), and
    within 0.3 % over the source region."""
    P, _ = surrogate_params
    A = [_run("thick_slab", 700 + i) for i in range(8)]
    S = [_run("thick_slab", 800 + i, P) for i in range(8)]
    seg_a = np.mean([r["segments"] for r in A])
    seg_s = np.mean([r["segments"] for r in S])
    assert seg_a / seg_s > 2.0, (seg_a, seg_s)
    assert np.mean([r["calls"] for r in S]) > 1e6
    Ta = np.array([r["temp"] for r in A])
    Ts = np.array([r["temp"] for r in S])
    live = Ta.mean(0) > 0.02
    se = np.sqrt(Ta.var(0, ddof=1) / len(Ta) + Ts.var(0, ddof=1) / len(Ts))[live]
    z = (Ts.mean(0) - Ta.mean(0))[live] / se
    assert np.all(np.abs(z) < 4.0), np.round(z, 1)
    assert np.sqrt(np.mean(z ** 2)) < 1.6, np.round(z, 1)
    src = slice(0, 10)  # RADSOURCE on [0, 0.5]: cells 0-9
    assert abs(Ts.mean(0)[src].mean() / Ta.mean(0)[src].mean() - 1.0) < 3e-3


def test_main_with_randomwalk_uses_the_surrogate(tmp_path, surrogate_params):
    """RANDOMWALK = TRUE (src/MixedPrecisionIMC.jl:127,140: Transport.MC_RW)
    runs main(args) with the learned surrogate."""
    import os
    import mpimc
    from mpimc import surrogate
    from conftest import deck_path
    surrogate._CACHE["P"] = surrogate_params[0]
    text = open(deck_path("thick_slab")).read()
    text = text.replace("RANDOMWALK = FALSE", "RANDOMWALK = TRUE").replace("NINPUT = 200000", "NINPUT = 20000")
    text = text.replace("NMAX = 2000000", "NMAX = 200000")
    p = os.path.join(str(tmp_path), "thick_rw.txt")
    open(p, "w").write(text)
    res = mpimc.main([p], verbose=False)
    assert sum(s["surrogate_calls"] for s in res.steps) > 0
    plain = mpimc.main([deck_path("thick_slab")], verbose=False)
    assert sum(s["surrogate_calls"] for s in plain.steps) == 0


def test_surrogate_with_fp16_state(surrogate_params):
    """FP16 particle state with the surrogate: runs, conserves energy to the
    FP32 arithmetic's level, queries the network, and is reproducible."""
    import mpimc
    P, _ = surrogate_params
    out = []
    for _ in range(2):
        inputs, mesh = load_deck("thick_slab", SEED="31", NINPUT="20000", NMAX="200000")
        e = mpimc.Engine(inputs, mesh, {"precision": 2, "scale_select_precision": 2})
        e.set_surrogate(P)
        steps, _ = e.run()
        out.append(e.field("temp"))
        assert sum(s["surrogate_calls"] for s in steps) > 0
        for s in steps[:-1]:
            assert abs(s["energy_error"]) < 1e-4 and s["error_flags"] == 0
        e.close()
    assert np.array_equal(out[0], out[1])


def test_learned_on_heated_thick_slab_matches_oracle_and_saves(surrogate_params):
    """The heated thick slab (30 cells of 40 mean free paths, a source in
    every cell), where every arm's per-run temperature error is ~0.15 %:
    8 learned + FP32 runs against the 32-seed FP64 oracle ensemble of the deck
    (tests/golden/oracle_fp64_ensembles.npz) and against 8 plain FP32 runs of
    the same seeds.  The network is an approximation of the walk, so its
    ensemble is held to a bias bound, not to statistical identity: per-run
    RMS error below 1 % (the target), the learned ensemble mean within 0.2 %
    RMS of the oracle mean (measured ~0.1 %), and the cells within 3 sigma of
    the oracle for the most part; the network removes over half of the analog
    segments and the runs are faster."""
    import os
    from conftest import REPO
    P, _ = surrogate_params
    g = np.load(os.path.join(REPO, "tests", "golden", "oracle_fp64_ensembles.npz"))
    ref, ref_sd, n_o = g["thick_temp"], g["thick_temp_std"], len(g["thick_seeds"])
    import mpimc
    L, F = [], []
    for sd in range(8):
        for params, out in ((P, L), (None, F)):
            inputs, mesh = load_deck("thick_heated", SEED=str(7100 + sd))
            e = mpimc.Engine(inputs, mesh)
            if params is not None:
                e.set_surrogate(params)
            steps, ms = e.run()
            out.append((e.field("temp"), ms, sum(s["segments"] for s in steps), sum(s["surrogate_calls"] for s in steps)))
            e.close()
    TL = np.array([r[0] for r in L])
    rel = np.sqrt(np.mean(((TL - ref) / ref) ** 2, axis=1))
    assert rel.max() < 0.01, rel
    bias = np.sqrt(np.mean(((TL.mean(0) - ref) / ref) ** 2))
    assert bias < 0.002, bias
    z = (TL.mean(0) - ref) / np.sqrt(TL.std(0, ddof=1) ** 2 / len(TL) + ref_sd ** 2 / n_o)
    assert np.mean(np.abs(z) < 3.0) >= 0.85, z
    assert sum(r[3] for r in L) > 0
    assert sum(r[2] for r in L) < 0.5 * sum(r[2] for r in F)
    assert sum(r[1] for r in L) < sum(r[1] for r in F)
