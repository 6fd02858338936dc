"""The batched-ensemble workload (tests/golden/c5_decks.py), on the CPU: the
256 decks are rebuilt identically, follow their stated distributions, and all
qualify for the fused batch (imc_run_batch_fused: 1D, one state precision, one
energy scale, both tallies of the transport in shared memory)."""
import os
import sys

import numpy as np

from conftest import REPO

sys.path.insert(0, os.path.join(REPO, "tests", "golden"))

# the transport's shared-memory budget for block-private tallies (bytes) and
# its per-cell use in 1D: a 32-byte table row plus 2 x 24-byte tally slots
# per energy scale
SMEM_BUDGET = 200 * 1024


def test_ensemble_is_reproducible_and_in_range():
    from c5_decks import c5_params
    a, b = c5_params(256), c5_params(256)
    assert a == b
    cells = np.array([p["cells"] for p in a])
    sig = np.array([p["sigma_a"] for p in a])
    nin = np.array([p["ninput"] for p in a])
    assert cells.min() >= 50 and cells.max() <= 2000
    assert sig.min() >= 0.1 and sig.max() <= 1000.0
    assert nin.min() >= 1e4 and nin.max() <= 1e6
    assert set(p["power"] for p in a) == {0.0, -3.0}
    assert [p["seed"] for p in a] == list(range(256))


def test_every_deck_qualifies_for_the_fused_batch():
    import mpimc
    from c5_decks import c5_decks
    for inputs, mesh in c5_decks(256, particle_scale=0.01):
        d, _ = mpimc.build_deck(inputs, mesh)
        assert d.geometry == 1 and d.precision == 1 and d.n_scales == 1
        assert 32 * d.nx + 48 * d.n_scales * d.nx <= SMEM_BUDGET, d.nx
