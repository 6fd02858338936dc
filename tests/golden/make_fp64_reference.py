"""Generates the FP64 ensemble mean of a test deck on a GPU:
tests/golden/<name>_fp64_mean.npz with the mean and standard deviation over
n seeds (900000 + i) of the final cell fields, run with FP64 particle state
and FP64 sorter scale selection -- the plain FP64 path, which the parity tests
tie history by history to the FP64 CPU oracle.  bench.py measures the
relative temperature error of its runs against these means.

    python tests/golden/make_fp64_reference.py c3_heatwave c3 [n_seeds]
    python tests/golden/make_fp64_reference.py thick_slab thick [n_seeds]
    python tests/golden/make_fp64_reference.py c4_channel2d c4 8

(c4_fp64_mean.npz: 8 seeds of the full 140 x 40 channel, 112 s on one GB300;
the GPU FP64 channel is tied to the oracle by the reduced-channel ensemble
test.)

(deck file tests/golden/decks/<deck>.txt; output <name>_fp64_mean.npz)
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
    deck, name = sys.argv[1], sys.argv[2]
    n = int(sys.argv[3]) if len(sys.argv) > 3 else 32
    seeds = [900000 + i for i in range(n)]
    T, R, M = [], [], []
    t0 = time.time()
    for sd in seeds:
        inputs = mpimc.Input.readInputs(os.path.join(HERE, "decks", deck + ".txt"))
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
    out = os.path.join(HERE, name + "_fp64_mean.npz")
    np.savez_compressed(out, seeds=np.array(seeds), temp=T.mean(0), temp_std=T.std(0, ddof=1),
                        rad=R.mean(0), rad_std=R.std(0, ddof=1), mat=M.mean(0), mat_std=M.std(0, ddof=1))
    print("wrote", out, "in %.0f s" % (time.time() - t0))


if __name__ == "__main__":
    main()
