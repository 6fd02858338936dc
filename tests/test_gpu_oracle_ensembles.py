"""GPU ensembles of the slab (C2), heat-wave (C3) and channel (C4) decks at
reduced particle counts against FP64 oracle ensembles of the same reduced decks
(tests/golden/oracle_fp64_ensembles.npz, tests/golden/make_oracle_ensembles.py):
per cell, the 32-seed GPU mean of the final temperature and radiation energy
density within 3 sigma of the 32-seed oracle mean, for FP64, FP32 and FP16
particle state (FP64 and FP32 on the 2D channel; FP16 against the oracle's
FP16-state ensemble).  The mesh, physics and
clock are the full configurations' -- C3 keeps its sigma = 10 T^-3 opacity
with the TEMP_FLOOR clamp, RAMP timestepping and left surface source -- so
these tests tie the GPU's full-size runs, whose FP64 means are the error
references of the benchmark, to the oracle."""
import os
import sys

import numpy as np
import pytest

from conftest import REPO

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(REPO, "tests", "golden")
GOLD = os.path.join(GOLDEN, "oracle_fp64_ensembles.npz")
# particle-state precision as an engine override: the deck keeps its own
# PRECISION for parsing (binary16 would round DX = 0.005 and the mesh with it)
PREC = {"fp64": 0, "fp32": 1, "fp16": 2}


def _have(name):
    return os.path.exists(GOLD) and (name + "_temp") in np.load(GOLD)


def _ensemble(name, prec, seeds):
    import mpimc
    sys.path.insert(0, GOLDEN)
    from make_oracle_ensembles import reduced_inputs
    T, R = [], []
    for sd in seeds:
        inputs = reduced_inputs(name, sd)
        mesh = mpimc.Mesh.mesh_generation(inputs)
        e = mpimc.Engine(inputs, mesh, {"precision": PREC[prec], "scale_select_precision": PREC[prec]})
        steps, _ = e.run()
        assert all(s["error_flags"] == 0 for s in steps)
        T.append(e.field("temp"))
        R.append(e.field("radenergydens"))
        e.close()
    return np.array(T), np.array(R)


# The heat wave is an FP32-state configuration: its opacity 10 T^-3 reaches 1e7
# at T_init = 0.01, past binary16, and its sourcing products overflow there
# (the oracle gives the same non-finite source energy).
CASES = [("c2", p) for p in ("fp64", "fp32", "fp16")] + [("c3", "fp64"), ("c3", "fp32"), ("c4", "fp64"), ("c4", "fp32")]


@pytest.mark.parametrize("name,prec", CASES)
def test_reduced_ensemble_within_3_sigma_of_oracle(gpu_lib, name, prec):
    if not _have(name):
        pytest.skip("oracle ensemble of %s not generated" % name)
    g = np.load(GOLD)
    # binary16 state is compared with the oracle's binary16-state ensemble:
    # the storage shifts both alike (~0.6 sigma, mean T +0.18 % on the slab)
    ref = name + "_fp16" if prec == "fp16" else name
    if ref + "_temp" not in g.files:
        pytest.skip("oracle ensemble %s not generated" % ref)
    n_o = len(g[ref + "_seeds"])
    T, R = _ensemble(name, prec, [600000 + i for i in range(32)])
    for field, arr in (("temp", T), ("rad", R)):
        mo, so = g["%s_%s" % (ref, field)], g["%s_%s_std" % (ref, field)]
        sg = arr.std(0, ddof=1)
        live = (so > 0) | (sg > 0)
        z = (arr.mean(0) - mo)[live] / np.sqrt(sg[live] ** 2 / len(arr) + so[live] ** 2 / n_o)
        # hundreds to thousands of cells: allow the odd 3-sigma excursion,
        # bound the mean square and a shift of the whole profile
        z2_max = 1.0 + 6.0 * np.sqrt(2.0 / live.sum()) + 0.2
        assert np.mean(np.abs(z) < 3.0) >= 0.95, (field, np.sort(np.abs(z))[-8:])
        assert np.mean(z ** 2) < z2_max, (field, np.mean(z ** 2))
        assert abs(np.mean(z)) < 0.5, (field, np.mean(z))
