"""imc_clean_noalloc -- the compaction for callers that cannot allocate device
memory (hosts whose pool allocator owns every byte of device memory, loops
that cannot take an allocation's device-wide sync).  The caller owns the
particle arrays; the scratch is a fixed __device__ array inside the library.

Each call is checked against the input filtered stably in numpy (survivors in
order, every field copied exactly) and, for FP64 and FP32 state, against the
handle-based compaction (imc_clean) on the same particles.  Several calls run
in a row on the shared scratch, and the size-independent checks (missing,
misaligned or overlapping arrays, oversized lists) run before any device work.

This file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_deck

pytestmark = pytest.mark.gpu

# state storage type and E0 type per precision code (IMC_FP64, IMC_FP32, IMC_FP16)
_TYPES = {0: (np.float64, np.float64), 1: (np.float32, np.float32), 2: (np.float16, np.float32)}
_STATE = ("t", "x", "ux", "E")


def _columns(rng, n, prec, geom, ncells, nscales, dead_frac):
    st, e0t = _TYPES[prec]
    cols = {k: rng.uniform(0.0, 1.0, n).astype(st) for k in _STATE}
    cols["ux"] = rng.uniform(-1.0, 1.0, n).astype(st)
    if geom == 2:
        cols["y"] = rng.uniform(0.0, 1.0, n).astype(st)
        cols["uy"] = rng.uniform(-1.0, 1.0, n).astype(st)
    dead = rng.uniform(size=n) < dead_frac
    cols["E0"] = np.where(dead, -1.0, rng.uniform(1e-3, 2e-3, n)).astype(e0t)
    cols["cs"] = (rng.integers(0, ncells, n) | (rng.integers(0, nscales, n) << 24)).astype(np.int32)
    cols["alive"] = (~dead).astype(np.uint8)
    return cols


def _noalloc(lib, prec, geom, cols):
    import torch
    from mpimc._lib import ImcDeviceParticles
    dev = torch.device("cuda:0")
    n = len(cols["E"])
    src = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in cols.items()}
    dst = {k: torch.full_like(v, 7) for k, v in src.items()}

    def view(d):
        g = lambda k: d[k].data_ptr() if k in d else None
        return ImcDeviceParticles(g("t"), g("x"), g("y"), g("ux"), g("uy"), g("E"), g("E0"), g("cs"), g("alive"))

    s, o = view(src), view(dst)
    n_out = C.c_int64(-1)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.imc_clean_noalloc(prec, geom, C.byref(s), C.byref(o), n, C.byref(n_out), C.c_void_p(stream))
    assert rc == 0, rc
    torch.cuda.synchronize()
    k = n_out.value
    return {key: v[:k].cpu().numpy() for key, v in dst.items()}, k


def _via_imc_clean(eng, cols, geom):
    cs = cols["cs"]
    p = {"t": cols["t"], "x": cols["x"], "E": cols["E"], "E0": cols["E0"],
         "cell": (cs & 0xFFFFFF).astype(np.int32), "scale": (cs >> 24).astype(np.int32)}
    if geom == 1:
        p["mu"] = cols["ux"]
    else:
        p.update(ux=cols["ux"], y=cols["y"], uy=cols["uy"])
    eng.set_particles(p)
    eng.clean()
    return eng.particles()


@pytest.mark.parametrize("geom", [1, 2])
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_noalloc_matches_stable_filter_and_imc_clean(gpu_lib, prec, geom):
    pytest.importorskip("torch")
    import mpimc
    inputs, mesh = load_deck("tiny_1d" if geom == 1 else "tiny_2d", PRECISION=_TYPES[prec][0])
    eng = mpimc.Engine(inputs, mesh)
    rng = np.random.default_rng(11 + 3 * prec + geom)
    # several calls in a row on the shared scratch: empty, whole tiles, ragged
    for n, dead in ((0, 0.0), (4096, 0.3), (8192, 0.0), (123_457, 0.05)):
        cols = _columns(rng, n, prec, geom, eng.ncells, eng.nscales, dead)
        got, k = _noalloc(gpu_lib, prec, geom, cols)
        keep = cols["alive"] != 0
        assert k == int(keep.sum())
        for key in cols:
            want = cols[key][keep] if key != "alive" else np.ones(k, np.uint8)
            np.testing.assert_array_equal(got[key], want, err_msg="%s n=%d" % (key, n))
        if prec == 2 or n == 0:
            continue  # FP16 state: the handle stores normalised fields; the filter above is exact
        exp = _via_imc_clean(eng, cols, geom)
        assert len(exp["E"]) == k
        for key in _STATE + (("y", "uy") if geom == 2 else ()):
            name = "mu" if (key == "ux" and geom == 1) else key
            np.testing.assert_array_equal(got[key].astype(np.float64), exp[name], err_msg=key)
        np.testing.assert_array_equal(got["E0"].astype(np.float64), exp["E0"])
        np.testing.assert_array_equal(got["cs"] & 0xFFFFFF, exp["cell"])
        np.testing.assert_array_equal(got["cs"] >> 24, exp["scale"])
    eng.close()


def _fake(base=1 << 20, stride=1 << 16, **over):
    """Distinct 256-byte aligned non-NULL addresses, never dereferenced: every
    case below is rejected by the host-side checks before any device work."""
    from mpimc._lib import ImcDeviceParticles
    names = ("t", "x", "y", "ux", "uy", "E", "E0", "cs", "alive")
    v = {k: base + i * stride for i, k in enumerate(names)}
    v.update(over)
    return ImcDeviceParticles(*[v[k] for k in names])


def test_noalloc_rejects_bad_arguments(gpu_lib):
    n_out = C.c_int64()
    call = lambda s, d, n=1000, prec=1, geom=1: gpu_lib.imc_clean_noalloc(
        prec, geom, C.byref(s), C.byref(d), n, C.byref(n_out), None)
    good_s, good_d = _fake(), _fake(base=1 << 30)
    INVALID = 1  # IMC_ERR_INVALID_ARG
    assert call(good_s, good_d, n=4096 * 4096 + 1) == INVALID  # beyond the scratch's 4096 tiles
    for f in ("t", "x", "ux", "E", "E0", "cs", "alive"):
        assert call(_fake(**{f: None}), good_d) == INVALID, f
        assert call(good_s, _fake(base=1 << 30, **{f: None})) == INVALID, f
    # 2D needs y and uy; 1D does not read them
    assert call(_fake(y=None), good_d, geom=2) == INVALID
    assert call(good_s, _fake(base=1 << 30, uy=None), geom=2) == INVALID
    # alive bytes are read 16 at a time from tile starts; state fields by element
    assert call(_fake(alive=(1 << 20) + 8), good_d) == INVALID
    assert call(_fake(x=(1 << 20) + 2), good_d) == INVALID
    assert call(_fake(x=(1 << 20) + 4), good_d, prec=0) == INVALID
    # in-place or overlapping src / dst arrays
    assert call(good_s, _fake(base=1 << 30, E=good_s.E)) == INVALID
    assert call(good_s, _fake(base=1 << 30, cs=good_s.cs + 64), n=1000) == INVALID
