"""GPU tests of the batched ensemble (imc_run_batch): decks run side by side
give exactly the fields they give alone, and a failing deck is named."""
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
