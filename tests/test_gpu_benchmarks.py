"""The GPU engine on the reference's benchmark decks, against the decks' own
benchmark curves and against the FP64 oracle ensembles of the same decks
(tests/golden/benchmark_oracle_fp64.npz), in every particle-state precision.

* Su-Olson (src/inputs/SuOlson.txt) to t = 1, 32 seeds each in FP64, FP32
  and the deck's own FLOAT16 (with its ENERGYSCALES = [32768]): E_r at the
  XBENCH points on the curve (tolerance in tests/benchcurves.py), and per cell
  within 3 sigma of the oracle ensemble.
* Marshak wave (src/inputs/MarshakWave.txt, the deck's FLOAT64, and FP32) to
  its ENDTIME 2: T on the curve behind the front, the front position and the
  cold tail, and per cell within 3 sigma of the oracle ensemble.
"""
import os
import sys

import numpy as np
import pytest

from benchcurves import ORACLE, marshak_violations, oracle_z, suolson_violations
from conftest import REPO

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(REPO, "tests", "golden")
PREC = {"fp64": np.float64, "fp32": np.float32, "fp16": np.float16}
FIELD = {"suolson": "radenergydens", "marshak": "temp"}


def _ensemble(name, prec, seeds):
    import mpimc
    sys.path.insert(0, GOLDEN)
    from make_benchmark_curves import load_inputs
    vals, flags = [], 0
    for sd in seeds:
        inputs = load_inputs(name, sd)
        inputs["PRECISION"] = PREC[prec]
        mesh = mpimc.Mesh.mesh_generation(inputs)
        e = mpimc.Engine(inputs, mesh)
        steps, _ = e.run()
        flags |= max(s["error_flags"] for s in steps)
        vals.append(e.field(FIELD[name]))
        centers = np.asarray(mesh.centers)
        e.close()
    assert flags == 0
    return centers, np.array(vals)


def _check_oracle(name, v, live):
    z = oracle_z(name, v.mean(0), v.std(0, ddof=1), len(v), live)
    assert np.mean(np.abs(z) < 3.0) >= 0.97, np.sort(np.abs(z))[-8:]
    assert np.mean(z ** 2) < 1.0 + 6.0 * np.sqrt(2.0 / len(z)), np.mean(z ** 2)


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp16"])
def test_suolson_on_curve_and_oracle(gpu_lib, prec):
    x, v = _ensemble("suolson", prec, [7000 + i for i in range(32)])
    bad = suolson_violations(x, v.mean(0), v.std(0, ddof=1) / np.sqrt(len(v)))
    assert not bad, bad
    # the wave front is at x = 1.5 at t = 1: compare where either side has energy
    _check_oracle("suolson", v, x < 1.6)


@pytest.mark.skipif("marshak_mean" not in np.load(ORACLE), reason="Marshak oracle ensemble not generated")
@pytest.mark.parametrize("prec,n", [("fp64", 8), ("fp32", 32)])
def test_marshak_on_curve_and_oracle(gpu_lib, prec, n):
    x, v = _ensemble("marshak", prec, [8000 + i for i in range(n)])
    bad = marshak_violations(x, v.mean(0), v.std(0, ddof=1) / np.sqrt(len(v)))
    assert not bad, bad
    _check_oracle("marshak", v, np.ones(len(x), bool))
