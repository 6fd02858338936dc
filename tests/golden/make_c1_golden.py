"""Generates tests/golden/c1_oracle_fp64_32seeds.npz: the FP64 oracle (CPU
restatement of the reference path) on the C1 linearized-slab deck
(tests/golden/decks/c1_slab.txt) for 32 seeds, the ensemble the statistical
GPU tests compare against (mean and standard deviation per cell of the final
temperature, radiation and material energy density).

Run from the repository root:  python tests/golden/make_c1_golden.py
"""
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
SEEDS = [500 + i for i in range(32)]


def one(seed):
    sys.path[:0] = [os.path.join(REPO, "mixedprecisionimc.jl_gb300"), os.path.join(REPO, "oracle")]
    import mpimc
    import oracle
    inputs = mpimc.Input.readInputs(os.path.join(HERE, "decks", "c1_slab.txt"))
    inputs["SEED"] = str(seed)
    mesh = mpimc.Mesh.mesh_generation(inputs)
    o = oracle.Oracle(inputs, mesh)
    steps = o.run()
    return (o.field("temp"), o.field("radenergydens"), o.field("matenergydens"),
            max(abs(s["energy_error"]) for s in steps), len(steps))


def main():
    with mp.get_context("spawn").Pool(min(8, os.cpu_count() or 1)) as pool:
        res = pool.map(one, SEEDS)
    T = np.array([r[0] for r in res])
    R = np.array([r[1] for r in res])
    M = np.array([r[2] for r in res])
    out = os.path.join(HERE, "c1_oracle_fp64_32seeds.npz")
    np.savez_compressed(out, seeds=np.array(SEEDS), temp_mean=T.mean(0), temp_std=T.std(0, ddof=1),
                        rad_mean=R.mean(0), rad_std=R.std(0, ddof=1), mat_mean=M.mean(0), mat_std=M.std(0, ddof=1),
                        energy_error_max=max(r[3] for r in res), steps=res[0][4])
    print("wrote", out, "steps", res[0][4], "max |energy error|", max(r[3] for r in res))


if __name__ == "__main__":
    main()
