"""ORACLE -- test infrastructure.  ctypes wrapper of liboracle.so, the CPU
restatement of the reference's per-timestep path (imc_oracle.cpp).  Only the
test suite, the smoke check and bench.py's CPU-baseline leg import this
module, as the checker; the product never does.

``Oracle`` exposes the same methods as the GPU ``mpimc.Engine`` so a test can
drive both through identical calls and compare.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


def build():
    """Compile liboracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_LIB = None


def load():
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        build()
    from mpimc._lib import ImcDeck, ImcParticles, ImcStepStats
    lib = C.CDLL(LIB_PATH)
    V = C.c_void_p
    sig = {
        "orc_create": (V, [C.POINTER(ImcDeck)]),
        "orc_destroy": (None, [V]),
        "orc_update": (C.c_int, [V]), "orc_sourcing": (C.c_int, [V]), "orc_transport": (C.c_int, [V]),
        "orc_clean": (C.c_int, [V]), "orc_tally": (C.c_int, [V]),
        "orc_energycheck": (C.c_int, [V, C.POINTER(C.c_double)]),
        "orc_timestep": (C.c_int, [V, C.POINTER(C.c_int)]),
        "orc_step": (C.c_int, [V, C.POINTER(ImcStepStats), C.POINTER(C.c_int)]),
        "orc_run": (C.c_int, [V, C.c_int64, C.POINTER(ImcStepStats), C.POINTER(C.c_int64)]),
        "orc_get_time": (C.c_int, [V, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
        "orc_set_time": (C.c_int, [V, C.c_double, C.c_double]),
        "orc_set_step": (C.c_int, [V, C.c_int64]),
        "orc_num_particles": (C.c_int64, [V]),
        "orc_get_particles": (C.c_int, [V, C.POINTER(ImcParticles)]),
        "orc_set_particles": (C.c_int, [V, C.POINTER(ImcParticles)]),
        "orc_get_field": (C.c_int, [V, C.c_int, C.POINTER(C.c_double), C.c_int64]),
        "orc_set_field": (C.c_int, [V, C.c_int, C.POINTER(C.c_double), C.c_int64]),
        "orc_get_stats": (C.c_int, [V, C.POINTER(ImcStepStats)]),
        "orc_get_scalars": (C.c_int, [V, C.POINTER(C.c_double)]),
        "orc_segments": (C.c_int64, [V]),
        "orc_flags": (C.c_uint32, [V]),
        "orc_philox": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
        "orc_sorter": (C.c_double, [C.c_int, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double), C.c_int,
                                    C.POINTER(C.c_double), C.POINTER(C.c_int)]),
        "orc_bench": (C.c_int, [C.POINTER(ImcDeck), C.c_int, C.c_int64, C.POINTER(C.c_double),
                                C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
        "orc_surr_walk": (C.c_int, [C.c_uint64, V, C.c_int64, V, V, V]),
        "orc_expm1_seg": (C.c_float, [C.c_float]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def philox(ctr, key):
    lib = load()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib.orc_philox(c, k, o)
    return list(o)


def surr_walk(seed, state):
    """CPU restatement of the surrogate's analog in-cell walk at the given
    (d_n, d_f, mu', lmax) rows: (x, cls, tgt) like imc_surrogate_walk."""
    lib = load()
    st = np.ascontiguousarray(state, dtype=np.float32)
    n = len(st)
    x = np.zeros((n, 4), np.float32)
    cls = np.zeros(n, np.int32)
    tgt = np.zeros((n, 2), np.float32)
    lib.orc_surr_walk(seed, st.ctypes.data_as(C.c_void_p), n, x.ctypes.data_as(C.c_void_p),
                      cls.ctypes.data_as(C.c_void_p), tgt.ctypes.data_as(C.c_void_p))
    return x, cls, tgt


def expm1_seg(x):
    """The FP32 segment arithmetic's e^x - 1 (the kernels' expm1_seg)."""
    return load().orc_expm1_seg(float(x))


def philox_uniforms(seed, step, index, stage, count):
    """The first `count` FP32 uniforms of the kernels' stream (seed, step, index, stage)."""
    words = []
    blk = 0
    while len(words) < count:
        words += philox([blk, step, index, stage], [seed & 0xFFFFFFFF, seed >> 32])
        blk += 1
    return [float(w >> 8) * 2.0 ** -24 for w in words[:count]]


def sorter(vals, scales, prec=0):
    lib = load()
    v = np.ascontiguousarray(vals, dtype=np.float64)
    s = np.ascontiguousarray(scales, dtype=np.float64)
    so, jo = C.c_double(), C.c_int()
    r = lib.orc_sorter(prec, v.ctypes.data_as(C.POINTER(C.c_double)), len(v),
                       s.ctypes.data_as(C.POINTER(C.c_double)), len(s), C.byref(so), C.byref(jo))
    return r, so.value, jo.value


_FIELDS = {"temp": 0, "radenergydens": 1, "matenergydens": 2, "fleck": 3, "beta": 4, "sigma_a": 5,
           "sigma_s": 6, "bee": 7, "energydep": 8, "emittedenergy": 9}


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """CPU restatement with the GPU Engine's method names."""

    def __init__(self, inputs, mesh, overrides=None):
        from mpimc.engine import build_deck
        self.lib = load()
        self.deck, self._keep = build_deck(inputs, mesh, overrides)
        self.geometry = self.deck.geometry
        self.nx, self.ny = self.deck.nx, self.deck.ny
        self.ncells = self.nx * self.ny
        self.nscales = self.deck.n_scales
        self.h = self.lib.orc_create(C.byref(self.deck))
        if not self.h:
            raise ValueError("oracle rejected the deck")

    @classmethod
    def from_deck(cls, deck, keep):
        self = cls.__new__(cls)
        self.lib = load()
        self.deck, self._keep = deck, keep
        self.geometry = deck.geometry
        self.nx, self.ny = deck.nx, deck.ny
        self.ncells = self.nx * self.ny
        self.nscales = deck.n_scales
        self.h = self.lib.orc_create(C.byref(deck))
        return self

    def close(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def update(self):
        self.lib.orc_update(self.h)

    def sourcing(self):
        self.lib.orc_sourcing(self.h)

    def transport(self):
        self.lib.orc_transport(self.h)

    def clean(self):
        self.lib.orc_clean(self.h)

    def tally(self):
        self.lib.orc_tally(self.h)

    def energycheck(self):
        e = C.c_double()
        self.lib.orc_energycheck(self.h, C.byref(e))
        return e.value

    def timestep(self):
        d = C.c_int()
        self.lib.orc_timestep(self.h, C.byref(d))
        return bool(d.value)

    def step(self):
        from mpimc._lib import ImcStepStats
        st, d = ImcStepStats(), C.c_int()
        self.lib.orc_step(self.h, C.byref(st), C.byref(d))
        return st.as_dict(), bool(d.value)

    def run(self, max_steps=1 << 40):
        from mpimc._lib import ImcStepStats
        out = []
        done = False
        while not done and len(out) < max_steps:
            st, done = self.step()
            out.append(st)
        return out

    def time(self):
        t, dt, s = C.c_double(), C.c_double(), C.c_int64()
        self.lib.orc_get_time(self.h, C.byref(t), C.byref(dt), C.byref(s))
        return t.value, dt.value, s.value

    def set_time(self, t, dt):
        self.lib.orc_set_time(self.h, float(t), float(dt))

    def set_step(self, s):
        self.lib.orc_set_step(self.h, int(s))

    def num_particles(self):
        return self.lib.orc_num_particles(self.h)

    def field(self, name):
        n = self.ncells * (self.nscales if name in ("energydep", "emittedenergy") else 1)
        out = np.empty(n)
        rc = self.lib.orc_get_field(self.h, _FIELDS[name], _dp(out), n)
        assert rc == 0
        return out

    def set_field(self, name, values):
        a = np.ascontiguousarray(values, dtype=np.float64).ravel()
        rc = self.lib.orc_set_field(self.h, _FIELDS[name], _dp(a), a.size)
        assert rc == 0

    def particles(self):
        from mpimc._lib import ImcParticles
        n = self.num_particles()
        cols = {k: np.zeros(n) for k in ("t", "x", "y", "mu", "ux", "uy", "E", "E0")}
        cell = np.zeros(n, dtype=np.int32)
        scale = np.zeros(n, dtype=np.int32)
        p = ImcParticles()
        p.n = n
        for k, v in cols.items():
            setattr(p, k, _dp(v))
        p.cell = cell.ctypes.data_as(C.POINTER(C.c_int32))
        p.scale = scale.ctypes.data_as(C.POINTER(C.c_int32))
        rc = self.lib.orc_get_particles(self.h, C.byref(p))
        assert rc == 0
        cols["cell"], cols["scale"] = cell, scale
        return cols

    def set_particles(self, cols):
        from mpimc._lib import ImcParticles
        n = len(cols["E"])
        keep = {}
        p = ImcParticles()
        p.n = n
        for k in ("t", "x", "y", "mu", "ux", "uy", "E", "E0"):
            if k in cols:
                keep[k] = np.ascontiguousarray(cols[k], dtype=np.float64)
                setattr(p, k, _dp(keep[k]))
        keep["cell"] = np.ascontiguousarray(cols["cell"], dtype=np.int32)
        keep["scale"] = np.ascontiguousarray(cols.get("scale", np.zeros(n)), dtype=np.int32)
        p.cell = keep["cell"].ctypes.data_as(C.POINTER(C.c_int32))
        p.scale = keep["scale"].ctypes.data_as(C.POINTER(C.c_int32))
        self.lib.orc_set_particles(self.h, C.byref(p))

    def stats(self):
        from mpimc._lib import ImcStepStats
        st = ImcStepStats()
        self.lib.orc_get_stats(self.h, C.byref(st))
        return st.as_dict()

    def scalars(self):
        a = (C.c_double * 4)()
        self.lib.orc_get_scalars(self.h, a)
        return {"totalenergy": a[0], "totalenergydep": a[1], "lostenergy": a[2], "radenergyold": a[3]}

    def segments(self):
        return self.lib.orc_segments(self.h)

    def flags(self):
        return self.lib.orc_flags(self.h)


def bench(deck, nthreads, max_steps):
    """CPU baseline: nthreads replicas of the deck (seeds SEED+i) for up to
    max_steps steps each.  Returns (seconds, segments, histories)."""
    lib = load()
    s, seg, his = C.c_double(), C.c_int64(), C.c_int64()
    lib.orc_bench(C.byref(deck), int(nthreads), int(max_steps), C.byref(s), C.byref(seg), C.byref(his))
    return s.value, seg.value, his.value
