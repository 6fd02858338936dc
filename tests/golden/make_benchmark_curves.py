"""Fixtures that pin the oracle to the only numbers the reference holds: the
benchmark curves carried in two of its decks.

* ``src/inputs/SuOlson.txt``: radiation energy density E_r(x) at the XBENCH
  points (YBENCH, lines 71-72).  The curve is the Su-Olson transport solution
  at tau = c*t = 1 (its support ends at x = 0.5 + tau = 1.5); the deck runs to
  ENDTIME 10, where its field is ~3x the curve and reaches past x = 3, so the
  comparison is made at t = 1 with every other keyword unchanged.
* ``src/inputs/MarshakWave.txt``: temperature T(x) at the XBENCH points
  (YBENCH, lines 74-109), a run of the deck to its ENDTIME (2.0) with the
  ``MARSHAK WAVE`` opacity sigma = sigma_0 / T^3 (src/imc_update.jl:32-34).

Written here:

* ``decks/suolson.txt``, ``decks/marshak.txt``: the two decks' keywords as in
  the reference files (comments and the XBENCH / YBENCH / BENCHMARK lines
  dropped), so the tests run them without the reference checkout;
* ``benchmark_curves.npz``: both curves as float64 (parsed from the deck text,
  not in the decks' FLOAT16 precision);
* ``benchmark_oracle_fp64.npz`` (``--oracle``): FP64 oracle ensembles of both
  decks (Su-Olson at t = 1: 32 seeds; Marshak at t = 2: 16 seeds), mean and
  standard deviation per cell -- the CPU side of the pin, against which the
  GPU runs are compared.

Run from the repository root with the reference checkout at IMC_REFERENCE:
    IMC_REFERENCE=<checkout> python tests/golden/make_benchmark_curves.py --decks
    python tests/golden/make_benchmark_curves.py --oracle [suolson] [marshak]
"""
import multiprocessing as mp
import os
import re
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
DECKS = {"suolson": "src/inputs/SuOlson.txt", "marshak": "src/inputs/MarshakWave.txt"}
DROP = ("XBENCH", "YBENCH", "BENCHMARK")
# the comparison time of each curve (see above) and the oracle ensemble size
ENDTIME = {"suolson": "1.0", "marshak": None}
SEEDS = {"suolson": [1234 + i for i in range(32)], "marshak": [12345 + i for i in range(16)]}
FIELD = {"suolson": "radenergydens", "marshak": "temp"}
OUT_ORACLE = os.path.join(HERE, "benchmark_oracle_fp64.npz")


def _entries(text):
    """(key, value text) of every ``KEY = value`` entry, arrays joined onto one line."""
    out, key, buf = [], None, None
    for raw in text.splitlines():
        line = raw.strip()
        if not line or line.startswith("#"):
            continue
        if buf is not None:
            buf.append(line)
            if line.endswith("]"):
                out.append((key, " ".join(buf)))
                buf = None
            continue
        m = re.match(r"^(\w+) = (.*)$", line)
        if not m:
            continue
        key, val = m.group(1), m.group(2).strip()
        if val.startswith("[") and not val.endswith("]"):
            buf = [val]
        else:
            out.append((key, val))
    return out


def _floats(val):
    return np.array([float(v) for v in val.strip("[]").split(",") if v.strip()], dtype=np.float64)


def write_decks(ref):
    curves = {}
    for name, rel in DECKS.items():
        ent = _entries(open(os.path.join(ref, rel)).read())
        vals = dict(ent)
        curves[name + "_x"] = _floats(vals["XBENCH"])
        curves[name + "_y"] = _floats(vals["YBENCH"])
        lines = ["# %s: the keywords of the reference deck %s" % (name, rel),
                 "# (comments and the benchmark-curve lines dropped; the curve is in",
                 "# tests/golden/benchmark_curves.npz).  Written by make_benchmark_curves.py."]
        lines += ["%s = %s" % (k, v) for k, v in ent if k not in DROP]
        with open(os.path.join(HERE, "decks", name + ".txt"), "w") as f:
            f.write("\n".join(lines) + "\n")
    np.savez_compressed(os.path.join(HERE, "benchmark_curves.npz"), **curves)
    print("wrote decks/suolson.txt, decks/marshak.txt, benchmark_curves.npz")


def load_inputs(name, seed=None, endtime=None):
    """The deck as the tests run it (ENDTIME of the curve unless given)."""
    if os.path.join(REPO, "mixedprecisionimc.jl_gb300") not in sys.path:
        sys.path.insert(0, os.path.join(REPO, "mixedprecisionimc.jl_gb300"))
    import mpimc
    inputs = mpimc.Input.readInputs(os.path.join(HERE, "decks", name + ".txt"))
    t = endtime or ENDTIME[name]
    if t:
        inputs["ENDTIME"] = t
    if seed is not None:
        inputs["SEED"] = str(seed)
    return inputs


def one(args):
    name, seed = args
    sys.path[:0] = [os.path.join(REPO, "mixedprecisionimc.jl_gb300"), os.path.join(REPO, "oracle")]
    import mpimc
    import oracle
    inputs = load_inputs(name, seed)
    inputs["PRECISION"] = np.float64
    inputs["ENERGYSCALES"] = ["1.0"]
    mesh = mpimc.Mesh.mesh_generation(inputs)
    o = oracle.Oracle(inputs, mesh)
    t0 = time.time()
    steps = o.run()
    return o.field(FIELD[name]), time.time() - t0, len(steps)


def write_oracle(names):
    out = dict(np.load(OUT_ORACLE)) if os.path.exists(OUT_ORACLE) else {}
    with mp.get_context("spawn").Pool(min(8, os.cpu_count() or 1)) as pool:
        for name in names:
            res = pool.map(one, [(name, s) for s in SEEDS[name]])
            v = np.array([r[0] for r in res])
            out[name + "_mean"] = v.mean(0)
            out[name + "_std"] = v.std(0, ddof=1)
            out[name + "_seeds"] = np.array(SEEDS[name])
            out[name + "_steps"] = res[0][2]
            print(name, "runs", len(res), "s/run %.1f" % np.mean([r[1] for r in res]), flush=True)
            np.savez_compressed(OUT_ORACLE, **out)
    print("wrote", OUT_ORACLE)


if __name__ == "__main__":
    if "--decks" in sys.argv:
        ref = os.environ.get("IMC_REFERENCE")
        if not ref:
            sys.exit("set IMC_REFERENCE to the reference checkout")
        write_decks(ref)
    if "--oracle" in sys.argv:
        write_oracle([n for n in ("suolson", "marshak") if n in sys.argv] or ["suolson", "marshak"])
