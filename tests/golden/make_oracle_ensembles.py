"""FP64 oracle ensembles of the slab, heat-wave and channel decks at reduced
particle counts, and of the heated thick slab at full size:
tests/golden/oracle_fp64_ensembles.npz.

The CPU oracle (the restatement of the reference path) runs each deck with its
mesh, physics and clock unchanged -- the 2000-cell slab to t = 3 (602 steps),
the nonlinear heat wave with sigma = 10 T^-3 clamped at TEMP_FLOOR, RAMP
timestepping and the left surface source (src/imc_update.jl:12-56,
src/MixedPrecisionIMC.jl:199-218), the 140 x 40 channel to t = 1 -- and only
NINPUT / NMAX scaled down (REDUCED below), 32 seeds each, FP64 particle state.
The GPU tests (tests/test_gpu_oracle_ensembles.py) run the same reduced decks
in every state precision and compare their ensemble means with these per cell.

"c2_fp16" is the reduced slab with binary16 particle state (the oracle's
restatement of the kernels' FP16 state): binary16 storage shifts the
ensemble by ~0.6 sigma (mean temperature +0.18 %) against FP64 state, in the
oracle as on the GPU, so the GPU's FP16 runs are compared with this one.

The heated thick slab (tests/golden/decks/thick_heated.txt: 30 cells of 40
mean free paths, a source in every cell, vacuum on the right) runs as
written; its mean is the error reference of the learned surrogate's
comparison in bench.py, where every arm reaches an error below 1 %.

Run from the repository root:  python tests/golden/make_oracle_ensembles.py [c2 c3 c4 thick c2_fp16]
"""
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "oracle_fp64_ensembles.npz")
# deck file and the particle counts of the reduced run
REDUCED = {
    "c2": ("c2_slab_fine", {"NINPUT": "20000", "NMAX": "200000"}),
    "c3": ("c3_heatwave", {"NINPUT": "20000", "NMAX": "200000"}),
    "c4": ("c4_channel2d", {"NINPUT": "10000", "NMAX": "50000"}),
    "thick": ("thick_heated", {}),
    "c2_fp16": ("c2_slab_fine", {"NINPUT": "20000", "NMAX": "200000"}),
}
# particle-state precision of each ensemble (IMC_FP64 unless listed)
STATE = {"c2_fp16": 2}
SEEDS = [500000 + i for i in range(32)]


def reduced_inputs(name, seed):
    """The reduced deck as parsed inputs (shared with the GPU tests)."""
    if os.path.join(REPO, "mixedprecisionimc.jl_gb300") not in sys.path:
        sys.path.insert(0, os.path.join(REPO, "mixedprecisionimc.jl_gb300"))
    import mpimc
    deck, over = REDUCED[name]
    inputs = mpimc.Input.readInputs(os.path.join(HERE, "decks", deck + ".txt"))
    inputs.update(over)
    inputs["SEED"] = str(seed)
    return inputs


def one(args):
    name, seed = args
    sys.path[:0] = [os.path.join(REPO, "mixedprecisionimc.jl_gb300"), os.path.join(REPO, "oracle")]
    import mpimc
    import oracle
    inputs = reduced_inputs(name, seed)
    prec = STATE.get(name, 0)
    if prec == 0:
        inputs["PRECISION"] = np.float64  # FP64 state, constants in FP64
    mesh = mpimc.Mesh.mesh_generation(inputs)
    o = oracle.Oracle(inputs, mesh, {"precision": prec, "scale_select_precision": prec} if prec else None)
    t0 = time.time()
    steps = o.run()
    return (o.field("temp"), o.field("radenergydens"), time.time() - t0, len(steps),
            max(abs(s["energy_error"]) for s in steps[:-1]))


def main():
    names = [a for a in sys.argv[1:] if a in REDUCED] or ["c2", "c3", "c4"]
    out = dict(np.load(OUT)) if os.path.exists(OUT) else {}
    with mp.get_context("spawn").Pool(min(8, os.cpu_count() or 1)) as pool:
        for name in names:
            res = pool.map(one, [(name, s) for s in SEEDS])
            T = np.array([r[0] for r in res])
            R = np.array([r[1] for r in res])
            out.update({name + "_temp": T.mean(0), name + "_temp_std": T.std(0, ddof=1),
                        name + "_rad": R.mean(0), name + "_rad_std": R.std(0, ddof=1),
                        name + "_seeds": np.array(SEEDS), name + "_steps": res[0][3],
                        name + "_energy_error_max": max(r[4] for r in res)})
            print(name, "s/run %.1f" % np.mean([r[2] for r in res]), "steps", res[0][3],
                  "energy error (before the last step) %.2e" % max(r[4] for r in res), flush=True)
            np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
