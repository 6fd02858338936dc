"""GPU tests of the batched ensemble (imc_run_batch, imc_run_batch_fused):
decks run side by side, or stepped together with one transport launch per
step, give exactly the fields they give alone, and a failing or unsuitable
deck is named."""
import os
import sys

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(REPO, "tests", "golden"))


def test_batch_equals_one_by_one(gpu_lib):
    import mpimc
    from c5_decks import c5_decks
    decks = c5_decks(12, particle_scale=0.01)
    alone = []
    for inputs, mesh in decks:
        e = mpimc.Engine(inputs, mesh)
        steps, _ = e.run()
        alone.append((len(steps), e.field("temp"), e.field("radenergydens")))
        e.close()
    engines = [mpimc.Engine(i, m) for i, m in decks]
    steps, wall = mpimc.run_batch(engines, threads=6)
    assert wall > 0.0
    for e, s, (n, T, R) in zip(engines, steps, alone):
        assert s == n
        assert np.array_equal(e.field("temp"), T)
        assert np.array_equal(e.field("radenergydens"), R)
        e.close()


def test_batch_with_surrogate_and_max_steps(gpu_lib, surrogate_params):
    import mpimc
    from c5_decks import c5_decks
    decks = c5_decks(6, particle_scale=0.01)
    engines = [mpimc.Engine(i, m) for i, m in decks]
    for e in engines:
        e.set_surrogate(surrogate_params[0])
    steps, _ = mpimc.run_batch(engines, max_steps=5, threads=3)
    assert steps == [5] * 6
    for e in engines:
        t, dt, s = e.time()
        assert s == 5
        e.close()


def test_batch_rejects_repeated_handles(gpu_lib):
    import mpimc
    from c5_decks import c5_decks
    (inputs, mesh), = c5_decks(1, particle_scale=0.01)
    e = mpimc.Engine(inputs, mesh)
    with pytest.raises(mpimc.ImcError):
        mpimc.run_batch([e, e])
    e.close()


def _alone(decks, overrides=None):
    import mpimc
    out = []
    for inputs, mesh in decks:
        e = mpimc.Engine(inputs, mesh, overrides)
        steps, _ = e.run()
        out.append((len(steps), e.field("temp"), e.field("radenergydens"), e.totals()))
        e.close()
    return out


def _fused_equals_alone(decks, overrides=None):
    import mpimc
    alone = _alone(decks, overrides)
    engines = [mpimc.Engine(i, m, overrides) for i, m in decks]
    steps, wall = mpimc.run_batch(engines, fused=True)
    assert wall > 0.0
    for e, s, (n, T, R, tot) in zip(engines, steps, alone):
        assert s == n
        assert np.array_equal(e.field("temp"), T)
        assert np.array_equal(e.field("radenergydens"), R)
        assert e.totals() == tot
        e.close()


def test_fused_batch_equals_one_by_one(gpu_lib):
    """One transport launch per step over every deck: each deck's fields and
    segment count equal its own run's, bit for bit (FP32 state)."""
    from c5_decks import c5_decks
    _fused_equals_alone(c5_decks(12, particle_scale=0.01))


def test_fused_batch_fp64_equals_one_by_one(gpu_lib):
    """FP64 state (512-thread blocks of the FP64 kernel)."""
    from c5_decks import c5_decks
    _fused_equals_alone(c5_decks(4, particle_scale=0.01), {"precision": 0, "scale_select_precision": 0})


def test_fused_batch_fp16_equals_one_by_one(gpu_lib):
    """FP16 state: the small slab (101 steps) and the nine-scale deck (its
    sorter falls back across scales; 3 steps) stepped together."""
    from conftest import load_deck
    decks = [load_deck("c1_slab", PRECISION=np.float16, SEED=str(s)) for s in (11, 12, 13)]
    decks += [load_deck("multiscale_1d", SEED=str(s)) for s in (5, 6)]
    _fused_equals_alone(decks)


def test_fused_batch_clocks_growth_and_max_steps(gpu_lib):
    """Decks whose clocks end at different times leave the group (the step
    graph is rebuilt), a deck whose buffers must grow mid-run grows, and
    max_steps stops every deck; each deck still equals its own run."""
    import mpimc
    from c5_decks import c5_decks
    decks = c5_decks(5, particle_scale=0.01)
    decks[1][0]["ENDTIME"] = "0.3"
    decks[3][0]["ENDTIME"] = "0.6"
    decks[2][0]["CAPACITY"] = "2500"
    alone = _alone(decks)
    engines = [mpimc.Engine(i, m) for i, m in decks]
    steps, _ = mpimc.run_batch(engines, fused=True)
    assert steps[1] < steps[3] < steps[0]
    for e, s, (n, T, R, tot) in zip(engines, steps, alone):
        assert s == n
        assert np.array_equal(e.field("temp"), T)
        assert np.array_equal(e.field("radenergydens"), R)
        e.close()
    engines = [mpimc.Engine(i, m) for i, m in decks]
    steps, _ = mpimc.run_batch(engines, max_steps=7, fused=True)
    assert steps == [7] * 5
    for e in engines:
        assert e.time()[2] == 7
        e.close()


def test_fused_batch_rejects_unsuitable_decks(gpu_lib, surrogate_params):
    import mpimc
    from c5_decks import c5_decks
    from conftest import load_deck
    decks = c5_decks(2, particle_scale=0.01)
    engines = [mpimc.Engine(i, m) for i, m in decks]
    engines[1].set_surrogate(surrogate_params[0])
    with pytest.raises(mpimc.ImcError):
        mpimc.run_batch(engines, fused=True)
    with pytest.raises(mpimc.ImcError):
        mpimc.run_batch([engines[0], engines[0]], fused=True)
    e2d = mpimc.Engine(*load_deck("tiny_2d"))
    with pytest.raises(mpimc.ImcError):
        mpimc.run_batch([engines[0], e2d], fused=True)
    for e in engines + [e2d]:
        e.close()
