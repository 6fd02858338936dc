#!/usr/bin/env python
"""Benchmark of the GB300 IMC engine on the 1D linearized slab workload:
2000 cells (dx = 0.005), dt = 0.005 to t = 3 (601 timesteps), NINPUT 2e6,
NMAX 2e7, FP32 particle state with FP64 material update (deck
tests/golden/decks/c2_slab_fine.txt).

One bench step is one full simulation (t = 0 -> 3).  Printed on one JSON line:
  value        particle segments per second over the timed steps (device
               time, inputs resident in HBM; the particle state, ~0.6 GB, is
               larger than L2, so no flush is needed between steps)
  fom          1/(relerr^2 * s), relerr = RMS over cells of the relative error
               of the final cell temperature against the FP64 ensemble mean
               (tests/golden/c2_fp64_mean.npz), s = seconds per simulation
  fp64         the same deck with FP64 particle state (the plain FP64 GPU
               path), max(steps, 6) runs: segments/s, relerr, FOM (relerr of
               the FP32 line: RMS over max(steps, 12) runs, the untimed ones
               outside the timed region).
               Comparisons are paired: every arm runs the same seeds, so its
               histories consume the same variates and the FOM ratios compare
               the methods at the same statistical error
  fp16_state   one run with binary16 particle state
  learned      the learned thick-cell surrogate (trained first, on the GPU)
               with FP32 state on the heated thick slab against plain FP32
               and plain FP64, relerr against the 32-seed FP64 oracle mean
               (tests/golden/oracle_fp64_ensembles.npz), every arm below 1 %
  c3           the nonlinear heat wave, FP32 state against plain FP64,
               relerr against tests/golden/c3_fp64_mean.npz
  c4           the 2D channel through thick walls, FP32 state against plain
               FP64, relerr over the heated cells against
               tests/golden/c4_fp64_mean.npz, and the 2D transport roofline
  c5           the 256-deck batched ensemble (tests/golden/c5_decks.py):
               side by side (learned + FP32, plain FP32) and fused (plain FP32,
               one transport launch per step over all decks, checked
               bit-identical to the side-by-side run) throughput over all
               decks, per-deck error and FOM against plain FP64 on 16 decks
  e2e          segments/s through the public API with host buffers: deck
               upload, run and the read-back of the cell fields per step
  roofline     the transport kernel: algorithmic bytes per launch over its
               CUDA-event duration, against the measured HBM copy bandwidth
  cpu_baseline the oracle (CPU restatement) on this host's cores, sampled
  clocks       SM clock samples taken during the timed region

``--impl reference`` times the CPU restatement of the reference path on all
host cores on the same deck and prints the same JSON line with impl=reference.
Under torchrun (N > 1) every rank runs an independent replica (seed + rank)
on its own GPU; value is the sum of segments over the max time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "mixedprecisionimc.jl_gb300")
GOLDEN = os.path.join(REPO, "tests", "golden")
PEAKS = os.path.join(REPO, "MEASURED_PEAKS.json")
METRIC = "FOM 1/(relerr²·s) & segments/s: learned+FP32 vs plain FP64 GPU at same error"
# bench decks: file, description, FP64 ensemble mean (None = no FOM)
DECKS = {
    "c2": ("c2_slab_fine.txt",
           "1D linearized slab, 2000 cells dx=0.005, dt=0.005 to t=3.0 (601 timesteps), NINPUT=2e6, NMAX=2e7, "
           "sigma_a=1, c=a=1, source 1.0 on [0,0.5], FP32 particle state, FP64 material update",
           "c2_fp64_mean.npz"),
    "c3": ("c3_heatwave.txt",
           "1D nonlinear heat wave, 500 cells on [0,1], sigma_a=10*T^-3 (T>=1e-3), bee 0.1, T_init 0.01, "
           "left surface T=1, RAMP dt0=1e-4 K=1.1 DTMAX=1e-2 to t=1, NINPUT=2e6, NMAX=2e7, FP32 state",
           None),
    "c4": ("c4_channel2d.txt",
           "2D thin channel through thick walls, 140x40 cells over [0,7]x[0,2], channel sigma_a=0.2, walls 2000, "
           "left segment y in [0,0.5] at T=0.5, dt=1e-3 to t=1, NINPUT=1e7, NMAX=5e7, FP32 state",
           None),
}
# DRAM traffic of the transport kernel per algorithmic byte, from one ncu
# capture of the half-size slab launch (bench.py --profile): 389.7 MB read +
# written for ~410 MB of algorithmic bytes
TRAFFIC_PER_ALGO_BYTE = 389.7 / 410.0
# runs behind the RMS temperature error of the headline deck: FP32 (the timed
# runs, plus untimed ones up to this count) and FP64 (paired seeds)
N_ERR_FP32, N_ERR_FP64 = 12, 6
DECK_KEY = "c2"
DECK = os.path.join(GOLDEN, "decks", DECKS[DECK_KEY][0])
REF_MEAN = os.path.join(GOLDEN, DECKS[DECK_KEY][2])
WORKLOAD = DECKS[DECK_KEY][1]
# algorithmic bytes of the FP32 transport kernel: every transported particle
# reads its state (1D t, x, mu, E, E0, cell|scale; 2D adds y, uy; 4 B each)
# and its alive byte; every census particle writes t, x, (y,) direction and E
READ_B, WRITE_B = 25, 16


def select_deck(key):
    global DECK_KEY, DECK, REF_MEAN, WORKLOAD, READ_B, WRITE_B
    DECK_KEY = key
    DECK = os.path.join(GOLDEN, "decks", DECKS[key][0])
    REF_MEAN = os.path.join(GOLDEN, DECKS[key][2]) if DECKS[key][2] else ""
    WORKLOAD = DECKS[key][1]
    READ_B, WRITE_B = (33, 24) if key == "c4" else (25, 16)

for _p in (PKG, os.path.join(REPO, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)


def combine_ranks(dist, dev_ms, segs, hist):
    """Replicas on N GPUs: the job's time is the slowest rank's, its work the
    sum over ranks (no data-path collective; one reduction of three numbers).
    Returns (max device ms, total segments, total histories)."""
    if dist is None:
        return dev_ms, segs, hist
    import torch
    tt = torch.tensor([dev_ms, segs, hist], dtype=torch.float64)
    mx = tt.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(tt, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(tt[1]), float(tt[2])


def _env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi samples during the timed region (SM MHz and throttle reasons)."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([v.strip() for v in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = sorted(float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit())
        mx = max(float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 5 + i and s[5 + i].strip() == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def load_deck(seed_offset=0, **ov):
    import mpimc
    inputs = mpimc.Input.readInputs(DECK)
    inputs["SEED"] = str(int(inputs["SEED"]) + seed_offset)
    inputs.update(ov)
    mesh = mpimc.Mesh.mesh_generation(inputs)
    return inputs, mesh


def relerr(temp, ref):
    import numpy as np
    if ref is None:
        return None
    r = ref["temp"]
    return float(np.sqrt(np.mean(((temp - r) / r) ** 2)))


def load_ref():
    import numpy as np
    if not os.path.exists(REF_MEAN):
        return None
    z = np.load(REF_MEAN)
    return {k: z[k] for k in z.files}


def run_once(inputs, mesh, overrides=None, timing=False):
    """One full simulation on the GPU; returns device ms, segments, histories,
    transport timing and the final temperature."""
    import mpimc
    eng = mpimc.Engine(inputs, mesh, overrides)
    try:
        eng.set_timing(timing)
        steps, ms = eng.run()
        tr_ms, tr_n = eng.transport_timing()
        temp = eng.field("temp")
        kps = eng.kernels_per_step()
    finally:
        eng.close()
    segs = sum(s["segments"] for s in steps)
    hist = sum(s["n_census_in"] + s["n_sourced"] for s in steps)
    flags = 0
    for s in steps:
        flags |= s["error_flags"]
    moved = sum((s["n_census_in"] + s["n_sourced"]) * READ_B + s["n_census_out"] * WRITE_B for s in steps)
    return {"ms": ms, "segments": segs, "histories": hist, "steps": len(steps), "transport_ms": tr_ms,
            "balance": balance_forms(steps),
            "fp16_over_bound_before_last": balance_forms(steps[:-1] or steps)["fp16_error_over_bound_max"],
            "bytes_2d": sum((s["n_census_in"] + s["n_sourced"]) * 33 + s["n_census_out"] * 24 for s in steps),
            "transport_launches": tr_n, "temp": temp, "flags": flags, "bytes": moved, "kernels": kps * len(steps),
            "energy_error": max(abs(s["energy_error"]) for s in steps),
            # the CONSTANT clock's last step is 4.2e-14 long (the reference's
            # N+1-th step); its relative balance divides by ~5e-14 of source
            "energy_error_before_last": max([abs(s["energy_error"]) for s in steps[:-1]] or [0.0])}


def balance_forms(steps):
    """The energy balance of src/imc_energycheck.jl:34 per step in two forms:
    relative to the step's source energy (the reference's; ill-conditioned on
    the CONSTANT clock's last step, 4.2e-14 long on the slab, whose source is
    ~1e-11 of the census energy), and relative to all the energy in play that
    step (source + census carried in), well conditioned on every step.  Also
    the binary16 rounding bound of FP16 state: census energies are stored as
    E/E0 in binary16, so each step's balance may miss up to 2^-11 of the
    census energy (relative to the source energy: 2^-11 E_rad / E_src)."""
    ref = max(abs(s["energy_error"]) for s in steps)
    wc = max(abs(s["energy_error"] * s["total_energy"]) / (s["total_energy"] + s["rad_energy_old"])
             for s in steps)
    bound16 = max(2.0 ** -11 * s["rad_energy"] / s["total_energy"] for s in steps)
    worst16 = max(abs(s["energy_error"]) / (2.0 ** -11 * s["rad_energy"] / s["total_energy"] + 1e-7)
                  for s in steps)
    return {"reference_form_max": ref, "in_play_form_max": wc, "fp16_rounding_bound_max": bound16,
            "fp16_error_over_bound_max": worst16}


def deck_runs(deck_file, offsets, overrides=None, params=None):
    """Full simulations of a test deck (seeds SEED + offset) on the GPU, with
    the learned surrogate when params is given."""
    import mpimc
    out = []
    for off in offsets:
        inputs = mpimc.Input.readInputs(os.path.join(GOLDEN, "decks", deck_file))
        inputs["SEED"] = str(int(inputs["SEED"]) + off)
        mesh = mpimc.Mesh.mesh_generation(inputs)
        eng = mpimc.Engine(inputs, mesh, overrides)
        try:
            if params is not None:
                eng.set_surrogate(params)
            steps, ms = eng.run()
            temp = eng.field("temp")
            kps = eng.kernels_per_step()
        finally:
            eng.close()
        out.append({"ms": ms, "temp": temp, "segments": sum(s["segments"] for s in steps),
                    "calls": sum(s["surrogate_calls"] for s in steps), "kernels": kps * len(steps),
                    "energy_error": max([abs(s["energy_error"]) for s in steps[:-1]] or [0.0])})
    return out


def summarize(runs, ref):
    """ms per run, RMS relative temperature error against the FP64 mean,
    FOM = 1/(relerr^2 s), analog segments and surrogate queries per run."""
    import numpy as np
    secs = sum(r["ms"] for r in runs) / 1000.0 / len(runs)
    rel = float(np.sqrt(np.mean([relerr(r["temp"], ref) ** 2 for r in runs])))
    return {"runs": len(runs), "ms_per_run": 1000.0 * secs, "relerr_T": rel, "fom": 1.0 / (rel ** 2 * secs),
            "segments_per_run": float(np.mean([r["segments"] for r in runs])),
            "surrogate_calls_per_run": float(np.mean([r["calls"] for r in runs])),
            "energy_error_max": max(r["energy_error"] for r in runs)}


def fp64_ref(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name + "_fp64_mean.npz"))


def learned_section(n, n64=8):
    """The learned part on the heated thick slab (tests/golden/decks/
    thick_heated.txt: 30 cells of 40 mean free paths, a source in every cell,
    vacuum on the right): learned surrogate + FP32 state against plain FP32
    and plain FP64, each run's temperature error against the 32-seed FP64
    oracle mean of the same deck (tests/golden/oracle_fp64_ensembles.npz),
    where every arm's error is below 1 %.  Seeds are paired (run i of every
    arm uses seed SEED + i), so per-run FOM ratios show the spread.  The
    network is trained here first, on the GPU."""
    import numpy as np
    from mpimc import surrogate
    t0 = time.perf_counter()
    P = surrogate.train()
    train_s = time.perf_counter() - t0
    ens = np.load(os.path.join(GOLDEN, "oracle_fp64_ensembles.npz"))
    if "thick_temp" not in ens.files:
        return {"deck": "thick_heated.txt", "error": "oracle ensemble of the deck not generated"}
    ref = {"temp": ens["thick_temp"]}
    fp64_ov = {"precision": 0, "scale_select_precision": 0}
    arms = {"learned_fp32": deck_runs("thick_heated.txt", range(1, n + 1), None, P),
            "fp32": deck_runs("thick_heated.txt", range(1, n + 1)),
            "fp64": deck_runs("thick_heated.txt", range(1, n64 + 1), fp64_ov)}
    out = {"deck": "thick_heated.txt",
           "workload": "1D linearized thick slab, 30 cells of 40 mean free paths (sigma_a=800, dx=0.05), "
                       "source 1.0 in every cell, reflect left / vacuum right, dt=0.5 to t=10, NINPUT=2e5, NMAX=2e6",
           "error_reference": "32-seed FP64 oracle mean (CPU restatement), tests/golden/oracle_fp64_ensembles.npz",
           "train_s": train_s, "train": dict(surrogate.DEFAULT_TRAIN)}
    for k, runs in arms.items():
        out[k] = summarize(runs, ref)
        out[k]["relerr_T_each"] = [relerr(r["temp"], ref) for r in runs]
        out[k]["ms_each"] = [r["ms"] for r in runs]
    fom_each = lambda k: [1.0 / (e ** 2 * m / 1000.0) for e, m in zip(out[k]["relerr_T_each"], out[k]["ms_each"])]
    fl, f32, f64 = fom_each("learned_fp32"), fom_each("fp32"), fom_each("fp64")
    pair64 = [a / b for a, b in zip(fl, f64)]
    pair32 = [a / b for a, b in zip(fl, f32)]
    out["fom_ratio_learned_over_fp64"] = out["learned_fp32"]["fom"] / out["fp64"]["fom"]
    out["fom_ratio_learned_over_fp32"] = out["learned_fp32"]["fom"] / out["fp32"]["fom"]
    out["fom_ratio_learned_over_fp64_paired"] = {"median": float(np.median(pair64)), "min": float(np.min(pair64)),
                                                 "max": float(np.max(pair64)), "pairs": len(pair64)}
    out["fom_ratio_learned_over_fp32_paired"] = {"median": float(np.median(pair32)), "min": float(np.min(pair32)),
                                                 "max": float(np.max(pair32)), "pairs": len(pair32)}
    out["segment_ratio_fp32_over_learned"] = out["fp32"]["segments_per_run"] / out["learned_fp32"]["segments_per_run"]
    return out


def c3_section(n):
    """The nonlinear heat wave (the surrogate's gate stays closed there: its
    thick cells never hold walks of 100 collisions) -- FP32 state against
    plain FP64, against the 32-seed FP64 mean."""
    ref = fp64_ref("c3")
    fp32 = summarize(deck_runs("c3_heatwave.txt", range(1, n + 1)), ref)
    fp64 = summarize(deck_runs("c3_heatwave.txt", range(1, n + 1), {"precision": 0, "scale_select_precision": 0}),
                     ref)
    return {"deck": "c3_heatwave.txt", "workload": DECKS["c3"][1], "fp32": fp32, "fp64": fp64,
            "fom_ratio_fp32_over_fp64": fp32["fom"] / fp64["fom"]}


def c4_section(n32=2, n64=2):
    """The 2D channel through thick walls (BASELINE's 2D configuration,
    tests/golden/decks/c4_channel2d.txt): FP32 state against plain FP64, each
    run's temperature error over the heated cells (reference mean above
    1.05 T_init) against the 8-seed GPU FP64 mean tests/golden/c4_fp64_mean.npz
    (the GPU FP64 path is tied to the oracle per history and by the
    reduced-channel ensemble test); the 2D transport kernel's roofline from
    one instrumented FP32 run."""
    import numpy as np
    import mpimc
    deck = os.path.join(GOLDEN, "decks", DECKS["c4"][0])
    refp = os.path.join(GOLDEN, "c4_fp64_mean.npz")
    ref = np.load(refp)["temp"] if os.path.exists(refp) else None

    def runs(ov, n, timing=False):
        out = []
        for i in range(n):
            inputs = mpimc.Input.readInputs(deck)
            inputs["SEED"] = str(int(inputs["SEED"]) + 1 + i)
            mesh = mpimc.Mesh.mesh_generation(inputs)
            out.append(run_once(inputs, mesh, ov, timing=timing))
        return out

    def err(temp):
        if ref is None:
            return None
        live = ref > 1.05 * 0.05
        return float(np.sqrt(np.mean(((temp[live] - ref[live]) / ref[live]) ** 2)))

    def arm(rs):
        secs = sum(r["ms"] for r in rs) / 1000.0 / len(rs)
        e = [err(r["temp"]) for r in rs]
        rel = None if e[0] is None else float(np.sqrt(np.mean(np.square(e))))
        return {"runs": len(rs), "ms_per_run": 1000.0 * secs, "relerr_T": rel, "relerr_T_each": e,
                "fom": None if rel is None else 1.0 / (rel ** 2 * secs),
                "segments_per_s": sum(r["segments"] for r in rs) / (secs * len(rs)),
                "energy_error_max": max(r["energy_error"] for r in rs),
                "kernels_per_run": rs[0]["kernels"]}

    f32 = arm(runs(None, n32))
    f64 = arm(runs({"precision": 0, "scale_select_precision": 0}, n64))
    inst = runs(None, 1, timing=True)[0]
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    hbm = peaks.get("hbm_gbs")
    n_l = max(inst["transport_launches"], 1)
    bpl = inst["bytes_2d"] / n_l
    ach = bpl / (inst["transport_ms"] / 1000.0) / 1e9 if inst["transport_ms"] > 0 else None
    out = {"deck": DECKS["c4"][0], "workload": DECKS["c4"][1], "fp32": f32, "fp64": f64,
           "error_reference": "8-seed GPU FP64 mean (tests/golden/c4_fp64_mean.npz), heated cells",
           "roofline_k_transport2d": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
                                      "frac": (ach / hbm) if (ach and hbm) else None,
                                      "avg_launch_ms": inst["transport_ms"], "launches": inst["transport_launches"],
                                      "algorithmic_bytes_per_launch": bpl,
                                      "transport_share_of_step": inst["transport_ms"] * n_l / inst["ms"]}}
    if f32["fom"] and f64["fom"]:
        out["fom_ratio_fp32_over_fp64"] = f32["fom"] / f64["fom"]
    out["time_ratio_fp64_over_fp32"] = f64["ms_per_run"] / f32["ms_per_run"]
    return out


def c5_section(n_err=16):
    """The batched ensemble (256 1D decks of tests/golden/c5_decks.py): run
    side by side with imc_run_batch (learned surrogate + FP32 state, plain
    FP32 state) and stepped together with imc_run_batch_fused (plain FP32, one
    transport launch per step over all 256 decks, checked bit-identical to the
    side-by-side run) over all 256 decks (throughput), and per-deck
    temperature error on the first n_err decks: learned+FP32 and plain FP64
    runs (seeds + 1000) against plain FP64 runs of other seeds (seeds + 2000)."""
    import numpy as np
    import mpimc
    from mpimc import surrogate
    sys.path.insert(0, GOLDEN)
    from c5_decks import c5_decks

    P = surrogate.train()

    def batch(n, seed_offset, overrides=None, params=None, fused=False):
        engines = [mpimc.Engine(i, m, overrides) for i, m in c5_decks(n, seed_offset=seed_offset)]
        try:
            if params is not None:
                for e in engines:
                    e.set_surrogate(params)
            steps, wall = mpimc.run_batch(engines, threads=32, fused=fused)
            tot = np.array([e.totals() for e in engines], dtype=np.float64)
            temps = [e.field("temp") for e in engines]
        finally:
            for e in engines:
                e.close()
        return {"wall_s": wall, "steps": int(sum(steps)), "segments": float(tot[:, 0].sum()),
                "histories": float(tot[:, 1].sum()), "surrogate_calls": float(tot[:, 2].sum()), "temp": temps}

    fp64 = {"precision": 0, "scale_select_precision": 0}
    learned = batch(256, 0, None, P)
    plain = batch(256, 0)
    fused = batch(256, 0, fused=True)
    same = all(np.array_equal(a, b) for a, b in zip(plain["temp"], fused["temp"]))
    ref = batch(n_err, 2000, fp64)
    l_err = batch(n_err, 1000, None, P)
    f_err = batch(n_err, 1000, fp64)

    def rel(run):
        r = []
        for a, b in zip(run["temp"], ref["temp"]):
            live = b > 0.02
            r.append(float(np.sqrt(np.mean(((a[live] - b[live]) / b[live]) ** 2))) if live.any() else 0.0)
        return r

    rl, rf = rel(l_err), rel(f_err)
    rms_l, rms_f = float(np.sqrt(np.mean(np.square(rl)))), float(np.sqrt(np.mean(np.square(rf))))
    fom_l = 1.0 / (rms_l ** 2 * l_err["wall_s"])
    fom_f = 1.0 / (rms_f ** 2 * f_err["wall_s"])
    return {"decks": 256, "workload": "256 1D decks: cells log-uniform 50-2000, sigma_a log-uniform 0.1-1000 with "
                                      "power 0 or -3, bee 0.05-1, left surface T 0.2-1, NINPUT 1e4-1e6, RAMP to t=1",
            "learned_fp32": {"wall_s": learned["wall_s"], "segments_per_s": learned["segments"] / learned["wall_s"],
                             "histories_per_s": learned["histories"] / learned["wall_s"],
                             "surrogate_calls": learned["surrogate_calls"], "segments": learned["segments"]},
            "fp32": {"wall_s": plain["wall_s"], "segments_per_s": plain["segments"] / plain["wall_s"],
                     "histories_per_s": plain["histories"] / plain["wall_s"], "segments": plain["segments"]},
            "fp32_fused": {"wall_s": fused["wall_s"], "segments_per_s": fused["segments"] / fused["wall_s"],
                           "histories_per_s": fused["histories"] / fused["wall_s"], "segments": fused["segments"],
                           "identical_to_side_by_side": bool(same and fused["segments"] == plain["segments"])},
            "error_decks": n_err,
            "relerr_T_learned_fp32": {"rms": rms_l, "median": float(np.median(rl)), "max": float(np.max(rl)),
                                      "wall_s": l_err["wall_s"]},
            "relerr_T_fp64": {"rms": rms_f, "median": float(np.median(rf)), "max": float(np.max(rf)),
                              "wall_s": f_err["wall_s"]},
            "fom_ratio_learned_over_fp64": fom_l / fom_f,
            "error_reference": "plain FP64 runs of the same decks with other seeds (both arms carry its noise)"}


def e2e_once(seed_offset):
    """Public-API run with host buffers: build the deck on the host, create the
    engine (uploads it), run, read the cell fields back, destroy."""
    import numpy as np
    import mpimc
    inputs, mesh = load_deck(seed_offset)
    d, keep = mpimc.build_deck(inputs, mesh)
    h2d = sum(v.nbytes for v in keep.values())
    t0 = time.perf_counter()
    eng = mpimc.Engine(inputs, mesh)
    steps, _ = eng.run()
    fields = [eng.field(f) for f in ("temp", "radenergydens", "matenergydens")]
    eng.close()
    wall = time.perf_counter() - t0
    d2h = sum(f.nbytes for f in fields) + len(steps) * 96
    return wall, sum(s["segments"] for s in steps), h2d, d2h


def cpu_baseline(threads, steps=120):
    """The oracle on this host: `threads` replicas of the deck at 1/100 of
    the particle counts, first `steps` timesteps; segments per second."""
    import oracle
    import mpimc
    base = mpimc.Input.readInputs(DECK)
    n_in, n_max = int(float(base["NINPUT"])) // 100, int(float(base["NMAX"])) // 100
    inputs, mesh = load_deck(0, NINPUT=str(n_in), NMAX=str(n_max))
    d, keep = mpimc.build_deck(inputs, mesh)
    secs, segs, hist = oracle.bench(d, threads, steps)
    return {"value": segs / secs, "unit": "segments/s", "cores": threads, "kind": "port",
            "sample": "oracle FP32 on the same deck at NINPUT=%d, NMAX=%d (1/100), first %d timesteps, "
                      "%d replicas (seeds SEED+i), %.1f s" % (n_in, n_max, steps, threads, secs),
            "histories_per_s": hist / secs}


def bench_reference(args):
    rank, world, _ = _env_rank()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline(threads, steps=60)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(threads, steps=60))
    wall = time.perf_counter() - t0
    v = sum(x["value"] for x in vals) / len(vals)
    cb = dict(vals[-1])
    cb["value"] = v
    print(json.dumps({
        "metric": METRIC, "value": v, "unit": "segments/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * wall / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (in-repo deck, seeded Philox)",
        "impl": "reference",
        "config": {"workload": WORKLOAD, "step": "one oracle sample (60 timesteps, 1/100 particles, all cores)",
                   "reference": "reference is Julia, not installable here; CPU restatement (oracle port) timed"},
        "cpu_baseline": cb,
        "e2e": {"value": v, "unit": "segments/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))
    return 0


def profile_case():
    """The workload at half the particle counts (C2: NINPUT 1e6, NMAX 1e7, a
    census of ~1e7 particles, ~0.25 GB of state -- larger than L2 but a few GB
    on the device at most), stepped 12 times stage by stage; for ncu captures."""
    import mpimc
    from mpimc import _build
    _build.build()
    base = mpimc.Input.readInputs(DECK)
    inputs, mesh = load_deck(0, NINPUT=str(int(float(base["NINPUT"]) // 2)), NMAX=str(int(float(base["NMAX"]) // 2)))
    eng = mpimc.Engine(inputs, mesh)
    for _ in range(12):
        st, done = eng.step()
        if done:
            break
    print(json.dumps({"profile_case": DECK_KEY, "census": st["n_census_out"], "segments": st["segments"]}))
    eng.close()
    return 0


def profile_learned_case():
    """The thick slab (tests/golden/decks/thick_slab.txt, 2e6 particles) with
    the learned surrogate, 10 timesteps run as graphs; for ncu captures of the
    query pass (k_wave_query) and the list / resume passes."""
    import mpimc
    from mpimc import _build, surrogate
    _build.build()
    P = surrogate.train()
    inputs = mpimc.Input.readInputs(os.path.join(GOLDEN, "decks", "thick_slab.txt"))
    mesh = mpimc.Mesh.mesh_generation(inputs)
    eng = mpimc.Engine(inputs, mesh)
    eng.set_surrogate(P)
    steps, _ = eng.run(10)
    print(json.dumps({"profile_case": "thick_slab+surrogate", "steps": len(steps),
                      "segments": sum(s["segments"] for s in steps),
                      "surrogate_calls": sum(s["surrogate_calls"] for s in steps)}))
    eng.close()
    return 0


def profile_fused_case():
    """The first 64 decks of the 256-deck ensemble at a quarter of their
    particle counts, stepped together 12 times with imc_run_batch_fused (one
    transport launch per step over all 64 decks); for ncu captures of the
    fused transport (k_transport1d_multi) and the step's launch list."""
    import mpimc
    from mpimc import _build
    _build.build()
    sys.path.insert(0, GOLDEN)
    from c5_decks import c5_decks
    engines = [mpimc.Engine(i, m) for i, m in c5_decks(64, particle_scale=0.25)]
    steps, wall = mpimc.run_batch(engines, max_steps=12, fused=True)
    tot = [e.totals() for e in engines]
    print(json.dumps({"profile_case": "c5 first 64 decks x 0.25, fused", "steps": steps[0],
                      "segments": int(sum(t[0] for t in tot)), "histories": int(sum(t[1] for t in tot))}))
    for e in engines:
        e.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparator run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-fp16", action="store_true", help="skip the FP16-state run")
    ap.add_argument("--deck", default="c2", choices=sorted(DECKS), help="workload (c2 is the headline)")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-surrogate comparison (thick slab)")
    ap.add_argument("--no-c3", action="store_true", help="skip the nonlinear heat-wave FP32 / FP64 comparison")
    ap.add_argument("--no-c5", action="store_true", help="skip the 256-deck batched ensemble")
    ap.add_argument("--no-c4", action="store_true", help="skip the 2D channel FP32 / FP64 comparison")
    ap.add_argument("--profile", action="store_true",
                    help="profiling case for ncu: the deck at half the particle counts, 12 timesteps, then exit")
    ap.add_argument("--profile-learned", action="store_true",
                    help="profiling case for ncu: the thick slab with the learned surrogate, 10 timesteps, then exit")
    ap.add_argument("--profile-fused", action="store_true",
                    help="profiling case for ncu: 64 ensemble decks stepped together (fused batch), 12 steps, then exit")
    args = ap.parse_args()
    select_deck(args.deck)
    if args.profile:
        return profile_case()
    if args.profile_learned:
        return profile_learned_case()
    if args.profile_fused:
        return profile_fused_case()
    rank, world, local = _env_rank()
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    if args.impl == "reference":
        return bench_reference(args)
    import numpy as np
    import mpimc
    from mpimc import _build
    _build.build()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    ref = load_ref()
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    hbm = peaks.get("hbm_gbs")
    inputs, mesh = load_deck(rank)
    for _ in range(args.warmup):
        run_once(inputs, mesh)
    if dist:
        dist.barrier()
    runs = []
    # the timed runs replay each step's captured CUDA graph (the product's
    # path, imc_run); device time from CUDA events around the whole run
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            runs.append(run_once(*load_deck(rank + 1000 * (i + 1))))
        wall = time.perf_counter() - t0
    dev_ms = sum(r["ms"] for r in runs)
    segs = sum(r["segments"] for r in runs)
    hist = sum(r["histories"] for r in runs)
    t_max, segs, hist = combine_ranks(dist, dev_ms, segs, hist)
    if rank != 0:
        return 0
    value = segs / (t_max / 1000.0)
    s_per_run = dev_ms / 1000.0 / args.steps
    rel = [relerr(r["temp"], ref) for r in runs]
    if rel[0] is not None and len(runs) < N_ERR_FP32:
        # the per-run error varies several-fold from seed to seed (the wave
        # front's cells): more runs, outside the timed region, for its RMS
        rel += [relerr(run_once(*load_deck(1000 * (i + 1)))["temp"], ref) for i in range(len(runs), N_ERR_FP32)]
    rel_m = None if rel[0] is None else float(np.sqrt(np.mean(np.square(rel))))
    fom = None if rel_m is None else 1.0 / (rel_m ** 2 * s_per_run)
    # roofline of the transport kernel, from a separate instrumented run of
    # the same deck: per-launch CUDA events around each transport launch
    # (direct launches, no graph), on the handle's stream
    inst = run_once(*load_deck(rank + 999), timing=True)
    tr_ms = inst["transport_ms"] * inst["transport_launches"]
    tr_n = inst["transport_launches"]
    bytes_per_launch = inst["bytes"] / max(tr_n, 1)
    avg_ms = tr_ms / max(tr_n, 1)
    achieved = bytes_per_launch / (avg_ms / 1000.0) / 1e9 if avg_ms > 0 else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": (achieved / hbm) if (achieved and hbm) else None,
                "traffic": TRAFFIC_PER_ALGO_BYTE * bytes_per_launch if DECK_KEY == "c2" else None,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the half-size slab "
                                  "launch (389.7 MB for ~410 MB algorithmic), scaled to this launch's "
                                  "algorithmic bytes",
                "kernel": "k_transport2d<StF32>" if DECK_KEY == "c4" else "k_transport1d<StF32>", "avg_launch_ms": avg_ms, "launches": tr_n,
                "algorithmic_bytes_per_launch": bytes_per_launch,
                "transport_share_of_step": tr_ms / inst["ms"] if inst["ms"] else None,
                "timing": "separate instrumented run (per-launch CUDA events, direct launches); the timed "
                          "runs replay CUDA graphs",
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"}
    out = {
        "metric": METRIC, "value": value, "unit": "segments/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (in-repo deck, seeded Philox streams)",
        "config": {"workload": WORKLOAD, "deck": DECKS[DECK_KEY][0], "step": "one full simulation",
                   "l2": "inputs larger than L2 (particle state ~0.6 GB); no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "histories_per_s": hist / (t_max / 1000.0),
        "relerr_T": rel_m, "relerr_runs": len(rel), "fom": fom,
        "energy_error_max": max(r["energy_error"] for r in runs),
        "energy_error_max_before_last_step": max(r["energy_error_before_last"] for r in runs),
        "energy_error_in_play_max": max(r["balance"]["in_play_form_max"] for r in runs),
        "error_flags": int(np.bitwise_or.reduce([r["flags"] for r in runs])),
        "gpu_launches": sum(r["kernels"] for r in runs),
        "clocks": clk.summary(),
        "roofline": roofline,
        "wall_s_timed": wall,
    }
    def comparator(prec_code, seed_base, n):
        """n full runs with another particle-state precision: speed, error, FOM"""
        rs = [run_once(*load_deck(seed_base + 1000 * i), overrides={"precision": prec_code,
                                                                    "scale_select_precision": prec_code})
              for i in range(n)]
        secs = sum(r["ms"] for r in rs) / 1000.0
        rels = [relerr(r["temp"], ref) for r in rs]
        rel_c = None if rels[0] is None else float(np.sqrt(np.mean(np.square(rels))))
        fom_c = None if rel_c is None else 1.0 / (rel_c ** 2 * secs / n)
        return {"value": sum(r["segments"] for r in rs) / secs, "unit": "segments/s", "runs": n,
                "ms_per_step": 1000.0 * secs / n, "relerr_T": rel_c, "fom": fom_c,
                "energy_error_max": max(r["energy_error"] for r in rs),
                "energy_error_max_before_last_step": max(r["energy_error_before_last"] for r in rs),
                "energy_error_in_play_max": max(r["balance"]["in_play_form_max"] for r in rs),
                **({"fp16_error_over_rounding_bound_max_before_last_step":
                    max(r["fp16_over_bound_before_last"] for r in rs)} if prec_code == 2 else {})}

    if not args.no_fp64:
        # the plain FP64 GPU path, as many runs as the timed FP32 runs
        out["fp64"] = comparator(0, 1000, max(args.steps, N_ERR_FP64))
        if fom and out["fp64"]["fom"]:
            out["fom_ratio_fp32_over_fp64"] = fom / out["fp64"]["fom"]
        out["time_ratio_fp64_over_fp32"] = out["fp64"]["ms_per_step"] / (dev_ms / args.steps)
    if not args.no_fp16:
        out["fp16_state"] = comparator(2, 1000, 1)
    if not args.no_learned:
        out["learned"] = learned_section(max(args.steps, 4))
    if not args.no_c3:
        out["c3"] = c3_section(2)
    if not args.no_c4 and DECK_KEY != "c4":
        out["c4"] = c4_section()
    if not args.no_c5:
        out["c5"] = c5_section()
    e2e = [e2e_once(2000 + i) for i in range(3)]
    w = sum(x[0] for x in e2e) / len(e2e)
    s_e = sum(x[1] for x in e2e) / len(e2e)
    out["e2e"] = {"value": s_e / w, "unit": "segments/s", "h2d_bytes_per_step": e2e[0][2],
                  "d2h_bytes_per_step": e2e[0][3], "wall_s_per_step": w, "runs": len(e2e),
                  "wall_s_each": [x[0] for x in e2e]}
    if not args.no_cpu:
        try:
            out["cpu_baseline"] = cpu_baseline(os.cpu_count() or 1)
        except Exception as e:  # the baseline is reported, never required
            out["cpu_baseline"] = {"value": None, "error": str(e)}
    print(json.dumps(out))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
