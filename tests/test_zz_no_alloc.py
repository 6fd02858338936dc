"""imc_clean_noalloc -- the compaction for callers that cannot allocate device
memory (work issued during a stream capture, hosts that own all device memory
through their own pool, loops that cannot take an allocation's device-wide
sync).  The caller owns the particle arrays; the scratch is a fixed __device__
array inside the library.  Two calls in a row, each checked against the
existing handle-based compaction (imc_clean) on the same particles: the
results must be identical, since compaction copies values exactly.

This file is named to be collected last."""
import ctypes as C

import numpy as np
import pytest

from conftest import load_deck

pytestmark = pytest.mark.gpu


def _particles(rng, n, ncells, dead_frac):
    return {
        "t": rng.uniform(0, 1e-3, n), "x": rng.uniform(0, 0.05, n), "mu": rng.uniform(-1, 1, n),
        "E": rng.uniform(1e-6, 1e-3, n),
        "E0": np.where(rng.uniform(size=n) < dead_frac, -1.0, rng.uniform(1e-3, 2e-3, n)),
        "cell": rng.integers(0, ncells, n).astype(np.int32), "scale": rng.integers(0, 2, n).astype(np.int32),
    }


def _expected(eng, cols):
    eng.set_particles(cols)
    eng.clean()
    return eng.particles()


def _noalloc(lib, cols):
    import torch
    from mpimc._lib import ImcDeviceParticles
    dev = torch.device("cuda:0")
    n = len(cols["E"])
    f32 = lambda a: torch.tensor(np.asarray(a, dtype=np.float32), device=dev)
    src = {k: f32(cols[k]) for k in ("t", "x", "mu", "E", "E0")}
    src["cs"] = torch.tensor(cols["cell"] | (cols["scale"] << 24), dtype=torch.int32, device=dev)
    src["alive"] = torch.tensor((cols["E0"] >= 0).astype(np.uint8), device=dev)
    dst = {k: torch.full_like(v, 7) for k, v in src.items()}

    def view(d):
        return ImcDeviceParticles(d["t"].data_ptr(), d["x"].data_ptr(), None, d["mu"].data_ptr(), None,
                                  d["E"].data_ptr(), d["E0"].data_ptr(), d["cs"].data_ptr(), d["alive"].data_ptr())

    s, o = view(src), view(dst)
    n_out = C.c_int64(-1)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.imc_clean_noalloc(1, 1, C.byref(s), C.byref(o), n, C.byref(n_out), C.c_void_p(stream))
    assert rc == 0, rc
    torch.cuda.synchronize()
    k = n_out.value
    return {key: v[:k].cpu().numpy() for key, v in dst.items()}, k


def test_noalloc_matches_imc_clean_twice(gpu_lib):
    pytest.importorskip("torch")
    import mpimc
    inputs, mesh = load_deck("tiny_1d", PRECISION=np.float32)
    eng = mpimc.Engine(inputs, mesh)
    rng = np.random.default_rng(11)
    for n, dead in ((50_000, 0.3), (123_457, 0.05)):
        cols = _particles(rng, n, eng.ncells, dead)
        exp = _expected(eng, cols)
        got, k = _noalloc(gpu_lib, cols)
        assert k == len(exp["E"]) == int((cols["E0"] >= 0).sum())
        for key in ("t", "x", "mu", "E", "E0"):
            np.testing.assert_array_equal(got[key].astype(np.float64), exp[key], err_msg=key)
        np.testing.assert_array_equal(got["cs"] & 0xFFFFFF, exp["cell"])
        np.testing.assert_array_equal(got["cs"] >> 24, exp["scale"])
        assert np.all(got["alive"] == 1)
    eng.close()


def test_noalloc_rejects_oversized_lists(gpu_lib):
    from mpimc._lib import ImcDeviceParticles
    p = ImcDeviceParticles(1, 1, None, 1, None, 1, 1, 1, 1)
    n_out = C.c_int64()
    rc = gpu_lib.imc_clean_noalloc(1, 1, C.byref(p), C.byref(p), 4096 * 4096 + 1, C.byref(n_out), None)
    assert rc == 1  # IMC_ERR_INVALID_ARG, before any device work
