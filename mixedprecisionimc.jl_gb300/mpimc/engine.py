"""The GPU engine handle: one simulation on one GPU behind the C ABI.

``Engine(inputs, mesh)`` turns a parsed deck and its mesh (the output of
``Input.readInputs`` and ``Mesh.mesh_generation``) into an ``ImcDeck`` and
creates the device state with ``imc_create``.  Every method is one C-ABI call;
nothing here computes physics.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import ImcDeck, ImcParticles, ImcStepStats, check

_PREC = {np.float64: _lib.IMC_FP64, np.float32: _lib.IMC_FP32, np.float16: _lib.IMC_FP16}
_BC = {"VACUUM": _lib.IMC_BC_VACUUM, "REFLECT": _lib.IMC_BC_REFLECT}


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel(order="F"))


def _ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _flag(inputs, key, default="FALSE"):
    return str(inputs.get(key, default)).strip().upper() == "TRUE"


def precision_code(p):
    for k, v in _PREC.items():
        if p is k:
            return v
    raise ValueError("unsupported PRECISION %r" % (p,))


def build_deck(inputs, mesh, overrides=None):
    """Assemble the ImcDeck of include/imc.h.  Returns (deck, keepalive)."""
    ov = dict(overrides or {})
    precision = inputs.get("PRECISION", np.float64)
    geometry = str(inputs["GEOMETRY"]).upper()
    d = ImcDeck()
    d.abi_version = _lib.IMC_ABI_VERSION
    d.geometry = _lib.IMC_GEOM_1D if geometry == "1D" else _lib.IMC_GEOM_2D
    if d.geometry == _lib.IMC_GEOM_1D:
        d.nx, d.ny = int(mesh.Ncells), 1
    else:
        d.nx, d.ny = int(mesh.Ncells[0]), int(mesh.Ncells[1])
    d.precision = ov.get("precision", precision_code(precision))
    d.scale_select_precision = ov.get("scale_select_precision", precision_code(precision))
    keep = {}
    keep["dx"] = _f64(mesh.dx)
    keep["dy"] = _f64(mesh.dy) if d.geometry == _lib.IMC_GEOM_2D else _f64([1.0])
    keep["temp"] = _f64(mesh.temp)
    keep["sav"] = _f64(mesh.sigma_a[..., 1])
    keep["sap"] = _f64(mesh.sigma_a[..., 2])
    keep["ssv"] = _f64(mesh.sigma_s[..., 1])
    keep["ssp"] = _f64(mesh.sigma_s[..., 2])
    keep["bee"] = _f64(mesh.bee)
    keep["rad"] = _f64(mesh.radsource)
    if d.geometry == _lib.IMC_GEOM_1D:
        keep["ts"] = _f64(list(mesh.temp_surf))
    else:
        keep["ts"] = _f64(np.concatenate([np.asarray(f, dtype=np.float64) for f in mesh.temp_surf]))
    keep["scales"] = _f64(mesh.energyscales)
    d.dx, d.dy = _ptr(keep["dx"]), _ptr(keep["dy"])
    d.temp = _ptr(keep["temp"])
    d.sigma_a_val, d.sigma_a_pow = _ptr(keep["sav"]), _ptr(keep["sap"])
    d.sigma_s_val, d.sigma_s_pow = _ptr(keep["ssv"]), _ptr(keep["ssp"])
    d.bee, d.radsource, d.t_surface = _ptr(keep["bee"]), _ptr(keep["rad"]), _ptr(keep["ts"])
    bcs = [str(inputs.get(k, "VACUUM")).strip().upper() for k in ("LEFTBC", "RIGHTBC", "TOPBC", "BOTTOMBC")]
    if d.geometry == _lib.IMC_GEOM_1D:
        bcs[2] = bcs[3] = "VACUUM"
    for i, b in enumerate(bcs):
        if b not in _BC:
            raise ValueError("boundary condition %r must be REFLECT or VACUUM" % b)
        d.bc[i] = _BC[b]
    p = lambda k: float(precision(float(inputs[k])))
    d.phys_c, d.phys_a, d.alpha = p("PHYS_C"), p("PHYS_A"), p("ALPHA")
    d.n_scales = len(keep["scales"])
    d.energyscales = _ptr(keep["scales"])
    d.distancescale = float(mesh.distancescale)
    d.n_input = int(float(inputs["NINPUT"]))
    d.n_max = int(float(inputs["NMAX"]))
    d.cellmin = p("CELLMIN")
    d.linearized = 1 if str(inputs.get("LINEARIZED", "FALSE")) == "TRUE" else 0
    d.marshak_opacity = 1 if str(inputs.get("NAME", "")).upper() == "MARSHAK WAVE" else 0
    d.temp_floor = float(inputs.get("TEMP_FLOOR", 0.0))
    d.seed = int(inputs.get("SEED", "0")) & ((1 << 64) - 1)
    ts = str(inputs.get("TIMESTEPPING", "CONSTANT")).strip().upper()
    d.timestepping = _lib.IMC_TS_RAMP if ts == "RAMP" else _lib.IMC_TS_CONSTANT
    d.sort_census = 0
    # the clock is FP64 for every PRECISION (timestep control stays on the
    # host in FP64), so DT / ENDTIME are not rounded to the deck precision
    f64 = lambda k: float(inputs[k])
    if d.timestepping == _lib.IMC_TS_CONSTANT:
        d.dt = f64("DT")
    else:
        d.dt0, d.k, d.dtmax = f64("DT0"), f64("K"), f64("DTMAX")
        d.dt = d.dt0
    d.t_end = f64("ENDTIME")
    d.capacity = int(float(inputs.get("CAPACITY", 0)))
    d.segment_cap = int(float(inputs.get("SEGMENTCAP", 0)))
    for k, v in ov.items():
        if k not in ("precision", "scale_select_precision"):
            setattr(d, k, v)
    return d, keep


class Engine:
    """One IMC simulation on the current GPU (an ``ImcHandle``)."""

    def __init__(self, inputs, mesh, overrides=None):
        self.lib = _lib.load()
        self.deck, self._keep = build_deck(inputs, mesh, overrides)
        self.geometry = self.deck.geometry
        self.nx, self.ny = self.deck.nx, self.deck.ny
        self.ncells = self.nx * self.ny
        self.nscales = self.deck.n_scales
        h = C.c_void_p()
        rc = self.lib.imc_create(C.byref(self.deck), C.byref(h))
        check(rc, None, self.lib)
        self.h = h

    # ---- lifetime
    def close(self):
        if getattr(self, "h", None):
            self.lib.imc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _c(self, rc):
        check(rc, self.h, self.lib)

    # ---- stages (one C call each)
    def update(self):
        self._c(self.lib.imc_update(self.h))

    def sourcing(self):
        self._c(self.lib.imc_sourcing(self.h))

    def transport(self):
        self._c(self.lib.imc_transport(self.h))

    def clean(self):
        self._c(self.lib.imc_clean(self.h))

    def tally(self):
        self._c(self.lib.imc_tally(self.h))

    def energycheck(self):
        e = C.c_double()
        self._c(self.lib.imc_energycheck(self.h, C.byref(e)))
        return e.value

    def timestep(self):
        done = C.c_int()
        self._c(self.lib.imc_timestep(self.h, C.byref(done)))
        return bool(done.value)

    def step(self):
        st, done = ImcStepStats(), C.c_int()
        self._c(self.lib.imc_step(self.h, C.byref(st), C.byref(done)))
        return st.as_dict(), bool(done.value)

    def run(self, max_steps=1 << 40):
        n = self.steps_remaining(max_steps)
        arr = (ImcStepStats * max(n, 1))()
        ns, ms = C.c_int64(), C.c_double()
        self._c(self.lib.imc_run(self.h, n, arr, C.byref(ns), C.byref(ms)))
        return [arr[i].as_dict() for i in range(ns.value)], ms.value

    def steps_remaining(self, cap=1 << 40):
        """Steps left before t > ENDTIME, from the deterministic clock."""
        t, dt, _ = self.time()
        d = self.deck
        n = 0
        fin = t > d.t_end
        while not fin and n < cap:
            n += 1
            if t == d.t_end:
                t = d.t_end + dt
            elif d.timestepping == _lib.IMC_TS_CONSTANT:
                if t + dt > d.t_end:
                    dt = d.t_end - t
                    t = d.t_end
                else:
                    t = t + dt
            else:
                if dt < d.dtmax:
                    dt = dt * d.k
                    if dt > d.dtmax:
                        dt = d.dtmax
                if t + dt > d.t_end:
                    dt = d.t_end - t
                    t = d.t_end
                else:
                    t = t + dt
            fin = t > d.t_end
        return n

    # ---- state
    def time(self):
        t, dt, s = C.c_double(), C.c_double(), C.c_int64()
        self._c(self.lib.imc_get_time(self.h, C.byref(t), C.byref(dt), C.byref(s)))
        return t.value, dt.value, s.value

    def set_time(self, t, dt):
        self._c(self.lib.imc_set_time(self.h, float(t), float(dt)))

    def num_particles(self):
        n = C.c_int64()
        self._c(self.lib.imc_num_particles(self.h, C.byref(n)))
        return n.value

    def field(self, name):
        code = _lib.FIELDS[name]
        n = self.ncells * (self.nscales if name in ("energydep", "emittedenergy") else 1)
        out = np.empty(n, dtype=np.float64)
        self._c(self.lib.imc_get_field(self.h, code, _ptr(out), n))
        return out

    def set_field(self, name, values):
        code = _lib.FIELDS[name]
        a = _f64(values)
        self._c(self.lib.imc_set_field(self.h, code, _ptr(a), a.size))

    def particles(self):
        n = self.num_particles()
        cols = {k: np.zeros(n) for k in ("t", "x", "y", "mu", "ux", "uy", "E", "E0")}
        cell = np.zeros(n, dtype=np.int32)
        scale = np.zeros(n, dtype=np.int32)
        p = ImcParticles()
        p.n = n
        for k, v in cols.items():
            setattr(p, k, _ptr(v))
        p.cell = cell.ctypes.data_as(C.POINTER(C.c_int32))
        p.scale = scale.ctypes.data_as(C.POINTER(C.c_int32))
        self._c(self.lib.imc_get_particles(self.h, C.byref(p)))
        cols["cell"] = cell
        cols["scale"] = scale
        return cols

    def set_particles(self, cols):
        n = len(cols["E"])
        keep = {}
        p = ImcParticles()
        p.n = n
        for k in ("t", "x", "y", "mu", "ux", "uy", "E", "E0"):
            if k in cols:
                keep[k] = _f64(cols[k])
                setattr(p, k, _ptr(keep[k]))
        keep["cell"] = np.ascontiguousarray(cols["cell"], dtype=np.int32)
        keep["scale"] = np.ascontiguousarray(cols.get("scale", np.zeros(n)), dtype=np.int32)
        p.cell = keep["cell"].ctypes.data_as(C.POINTER(C.c_int32))
        p.scale = keep["scale"].ctypes.data_as(C.POINTER(C.c_int32))
        self._c(self.lib.imc_set_particles(self.h, C.byref(p)))

    def stats(self):
        st = ImcStepStats()
        self._c(self.lib.imc_get_stats(self.h, C.byref(st)))
        return st.as_dict()

    def save_state(self):
        """The whole simulation state as bytes (imc_save_state)."""
        n = C.c_size_t(0)
        self._c(self.lib.imc_save_state(self.h, None, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        self._c(self.lib.imc_save_state(self.h, C.cast(buf, C.c_void_p), C.byref(n)))
        return buf.raw[:n.value]

    def load_state(self, blob):
        """Restores a state saved from an Engine of the same deck."""
        b = C.create_string_buffer(bytes(blob), len(blob))
        self._c(self.lib.imc_load_state(self.h, C.cast(b, C.c_void_p), len(blob)))

    def totals(self):
        """(segments, histories, surrogate calls) over every step run so far."""
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        self._c(self.lib.imc_get_totals(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def set_surrogate(self, params):
        """Turn the learned thick-cell surrogate on (FP32 parameters from
        mpimc.surrogate.train) or off (None); 1D, FP32 / FP16 state."""
        import numpy as np
        if params is None:
            self._c(self.lib.imc_set_surrogate(self.h, None, 0))
            return
        P = np.ascontiguousarray(params, dtype=np.float32)
        self._c(self.lib.imc_set_surrogate(self.h, P.ctypes.data_as(C.c_void_p), P.size))

    def surrogate_active(self):
        a = C.c_int()
        self._c(self.lib.imc_get_surrogate_active(self.h, C.byref(a)))
        return bool(a.value)

    def set_timing(self, on=True):
        self._c(self.lib.imc_set_timing(self.h, 1 if on else 0))

    def transport_timing(self):
        ms, n = C.c_double(), C.c_int64()
        self._c(self.lib.imc_transport_timing(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def kernels_per_step(self):
        n = C.c_int()
        self._c(self.lib.imc_kernels_per_step(self.h, C.byref(n)))
        return n.value


def device_info():
    lib = _lib.load()
    name = C.create_string_buffer(256)
    sm, ma, mi = C.c_int(), C.c_int(), C.c_int()
    rc = lib.imc_device_info(name, 256, C.byref(sm), C.byref(ma), C.byref(mi))
    check(rc, None, lib)
    return {"name": name.value.decode(), "sm_count": sm.value, "cc": (ma.value, mi.value)}


def run_batch(engines, max_steps=1 << 40, threads=32, fused=False):
    """Batched ensemble: runs every Engine to the end of its clock.  With
    fused=False (imc_run_batch) `threads` host threads drive the decks' own
    step graphs side by side on the GPU; with fused=True
    (imc_run_batch_fused) the decks step together, one graph per step with a
    single transport launch over every deck (1D decks of one state precision
    without the surrogate).  Returns (steps per engine, host wall seconds).
    Raises ImcError naming the first failure."""
    lib = _lib.load()
    n = len(engines)
    hs = (C.c_void_p * max(n, 1))(*[e.h for e in engines])
    steps = (C.c_int64 * max(n, 1))()
    wall = C.c_double()
    bad = C.c_int32(-1)
    if fused:
        rc = lib.imc_run_batch_fused(hs, n, max_steps, steps, C.byref(wall), C.byref(bad))
    else:
        rc = lib.imc_run_batch(hs, n, max_steps, threads, steps, C.byref(wall), C.byref(bad))
    if rc != _lib.IMC_OK:
        e = engines[bad.value] if bad.value >= 0 else None
        check(rc, e.h if e else None, lib)
    return [steps[i] for i in range(n)], wall.value / 1000.0
