"""Generates tests/golden/c2_fp64_mean.npz on a GPU: the ensemble mean (32
seeds) of the final cell fields of the fine linearized slab deck
(tests/golden/decks/c2_slab_fine.txt: 2000 cells, dt = 0.005 to t = 3,
NINPUT 2e6, NMAX 2e7) run with FP64 particle state and FP64 sorter scale
selection -- the plain FP64 path, which the parity tests tie history by history
to the FP64 CPU oracle.  bench.py measures the relative temperature error of
its runs against this mean.  A full FP64 CPU ensemble at this size (about
2.5e10 segments per seed) is out of reach, hence the GPU FP64 path.

Run from the repository root on a GPU machine:
    python tests/golden/make_c2_reference.py [n_seeds]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(REPO, "mixedprecisionimc.jl_gb300")]


def main():
    import mpimc
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 32
    seeds = [900000 + i for i in range(n)]
    T, R, M = [], [], []
    t0 = time.time()
    for sd in seeds:
        inputs = mpimc.Input.readInputs(os.path.join(HERE, "decks", "c2_slab_fine.txt"))
        inputs["SEED"] = str(sd)
        mesh = mpimc.Mesh.mesh_generation(inputs)
        e = mpimc.Engine(inputs, mesh, {"precision": 0, "scale_select_precision": 0})
        steps, ms = e.run()
        T.append(e.field("temp"))
        R.append(e.field("radenergydens"))
        M.append(e.field("matenergydens"))
        e.close()
        print("seed", sd, "steps", len(steps), "%.1f ms" % ms, flush=True)
    T, R, M = np.array(T), np.array(R), np.array(M)
    out = os.path.join(HERE, "c2_fp64_mean.npz")
    np.savez_compressed(out, seeds=np.array(seeds), temp=T.mean(0), temp_std=T.std(0, ddof=1),
                        rad=R.mean(0), rad_std=R.std(0, ddof=1), mat=M.mean(0), mat_std=M.std(0, ddof=1))
    print("wrote", out, "in %.0f s" % (time.time() - t0))


if __name__ == "__main__":
    main()
