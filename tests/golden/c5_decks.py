"""The batched-ensemble workload (256 independent 1D decks), drawn with
seeded numpy (seed 0) from these distributions:

  cells          log-uniform 50-2000 on x in [0, 1] (uniform mesh)
  sigma_a        log-uniform 0.1-1000, temperature power 0 or -3 (even odds;
                 the opacity sees T clamped at >= 1e-3), sigma_s = 0
  heat capacity  uniform 0.05-1
  surfaces       left T uniform 0.2-1, right vacuum; T_init 0.01
  particles      NINPUT log-uniform 1e4-1e6, NMAX = 10 NINPUT
  clock          RAMP dt0 1e-4, K 1.1, DTMAX 1e-2 to t = 1
  seeds          0-255; FP32 particle state

Physical constants are the nonlinear heat-wave deck's (PHYS_C 299.70,
PHYS_A 0.01372016), as are every keyword not listed.  Nothing is read from
outside this repository, so the decks are rebuilt identically wherever the
bench runs.
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TEMPLATE = os.path.join(HERE, "decks", "c3_heatwave.txt")


def c5_params(n=256):
    rng = np.random.default_rng(0)
    cells = np.round(10.0 ** rng.uniform(np.log10(50), np.log10(2000), n)).astype(int)
    sig = 10.0 ** rng.uniform(-1.0, 3.0, n)
    power = np.where(rng.uniform(size=n) < 0.5, 0.0, -3.0)
    bee = rng.uniform(0.05, 1.0, n)
    tleft = rng.uniform(0.2, 1.0, n)
    ninput = np.round(10.0 ** rng.uniform(4.0, 6.0, n)).astype(int)
    return [dict(cells=int(cells[i]), sigma_a=float(sig[i]), power=float(power[i]), bee=float(bee[i]),
                 t_left=float(tleft[i]), ninput=int(ninput[i]), seed=i) for i in range(n)]


def c5_decks(n=256, seed_offset=0, particle_scale=1.0):
    """(inputs, mesh) of the first n decks; particle_scale shrinks NINPUT and
    NMAX (for tests), seed_offset shifts every deck's seed."""
    import mpimc
    out = []
    for p in c5_params(256)[:n]:
        inputs = mpimc.Input.readInputs(TEMPLATE)
        nin = max(1000, int(round(p["ninput"] * particle_scale)))
        inputs.update({
            "NAME": "Batched ensemble deck %d" % p["seed"],
            "DX": repr(1.0 / p["cells"]),
            "SIGMA_A_VALS": [repr(p["sigma_a"])],
            "SIGMA_A_POWERS": [repr(p["power"])],
            "BEE_VALS": [repr(p["bee"])],
            "T_SURFACE_VALS": [np.float32(p["t_left"]), np.float32(0.0)],
            "NINPUT": str(nin),
            "NMAX": str(10 * nin),
            "SEED": str(p["seed"] + seed_offset),
        })
        out.append((inputs, mpimc.Mesh.mesh_generation(inputs)))
    return out
