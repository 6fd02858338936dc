"""GPU parity: each CUDA stage against the CPU oracle on the same deck, the
same Philox streams and the same input state.

Tolerances: FP64 state -- the kernels and the oracle share every formula,
and differ only where CUDA's exp/expm1/log/pow round differently from
glibc's (1-2 ulp), so per-particle states agree to 1e-12 relative and
tallies to 1e-10.  FP32 state -- same, at single-precision ulps: 1e-4 relative
per particle, with a small fraction of histories allowed to take a different
branch after an ulp-level tie.
"""
import numpy as np
import pytest

from conftest import load_deck

pytestmark = pytest.mark.gpu


def _pair(name, gpu_lib, **ov):
    import mpimc
    import oracle
    inputs, mesh = load_deck(name, **ov)
    return mpimc.Engine(inputs, mesh), oracle.Oracle(inputs, mesh)


def _cmp_particles(g, o, rtol, frac_ok=1.0, keys=("t", "x", "mu", "E", "E0")):
    pg, po = g.particles(), o.particles()
    assert len(pg["E"]) == len(po["E"])
    n = len(pg["E"])
    if n == 0:
        return
    same_cell = pg["cell"] == po["cell"]
    alive_g, alive_o = pg["E0"] >= 0, po["E0"] >= 0
    ok = same_cell & (alive_g == alive_o) & (pg["scale"] == po["scale"])
    for k in keys:
        a, b = pg[k], po[k]
        close = np.abs(a - b) <= rtol * np.maximum(np.abs(b), 1e-300) + 1e-300
        ok &= close | ~alive_o
    frac = ok.mean()
    assert frac >= frac_ok, "only %.6f of %d particles agree" % (frac, n)


@pytest.mark.parametrize("deck", ["tiny_1d", "tiny_2d", "c1_slab"])
def test_update_parity(deck, gpu_lib):
    g, o = _pair(deck, gpu_lib)
    g.update()
    o.update()
    for f in ("fleck", "beta", "sigma_a", "sigma_s", "bee"):
        np.testing.assert_allclose(g.field(f), o.field(f), rtol=1e-14, atol=0, err_msg=f)


@pytest.mark.parametrize("deck", ["tiny_1d", "tiny_2d", "c1_slab"])
def test_sourcing_parity(deck, gpu_lib):
    g, o = _pair(deck, gpu_lib)
    for e in (g, o):
        e.update()
        e.sourcing()
    assert g.num_particles() == o.num_particles() > 0
    np.testing.assert_allclose(g.field("emittedenergy"), o.field("emittedenergy"), rtol=1e-14)
    keys = ("t", "x", "mu", "E", "E0") if g.geometry == 1 else ("t", "x", "y", "ux", "uy", "E", "E0")
    _cmp_particles(g, o, rtol=1e-14, keys=keys)


@pytest.mark.parametrize("deck", ["tiny_1d", "tiny_2d", "c1_slab"])
def test_transport_parity_fp64(deck, gpu_lib):
    g, o = _pair(deck, gpu_lib)
    for e in (g, o):
        e.update()
        e.sourcing()
        e.transport()
    keys = ("t", "x", "mu", "E") if g.geometry == 1 else ("t", "x", "y", "E")
    _cmp_particles(g, o, rtol=1e-10, frac_ok=0.999, keys=keys)
    dg, do = g.field("energydep"), o.field("energydep")
    np.testing.assert_allclose(dg, do, rtol=1e-8, atol=1e-12 * np.abs(do).max())


@pytest.mark.parametrize("deck", ["tiny_1d", "tiny_2d", "c1_slab", "infinite_medium"])
def test_step_parity_fp64(deck, gpu_lib):
    """Three full steps: temperatures, radiation and material energy track the
    oracle because both consume the same variates."""
    g, o = _pair(deck, gpu_lib)
    for _ in range(3):
        sg, _ = g.step()
        so, _ = o.step()
        assert sg["n_sourced"] == so["n_sourced"]
        assert abs(sg["n_census_out"] - so["n_census_out"]) <= max(2, 1e-4 * so["n_census_out"])
        np.testing.assert_allclose(sg["total_energy"], so["total_energy"], rtol=1e-13)
        np.testing.assert_allclose(sg["energy_error"], so["energy_error"], atol=1e-9)
    for f in ("temp", "radenergydens", "matenergydens"):
        a, b = g.field(f), o.field(f)
        np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-9 * np.abs(b).max(), err_msg=f)


def test_transport_parity_fp32(gpu_lib):
    g, o = _pair("tiny_1d", gpu_lib, PRECISION=np.float32)
    for e in (g, o):
        e.update()
        e.sourcing()
    _cmp_particles(g, o, rtol=0, keys=("t", "x", "mu", "E", "E0"))
    for e in (g, o):
        e.transport()
    _cmp_particles(g, o, rtol=1e-4, frac_ok=0.99, keys=("x", "mu", "E"))
    dg, do = g.field("energydep"), o.field("energydep")
    np.testing.assert_allclose(dg, do, rtol=1e-3, atol=1e-6 * np.abs(do).max())


def test_transport_parity_fp32_2d(gpu_lib):
    """Transport.MC2D (src/imc_transport.jl:483-732) with FP32 state, in the
    FP32 formulation the kernel and the oracle share: direction cosines,
    -log(v)/seff collision distances with the hardware logarithm, one expm1
    for attenuation and deposit, reciprocal cell areas.  The kernel re-emits
    with the hardware sine and cosine (the oracle with libm's, ~1 ulp apart),
    so histories that collide carry 1e-7-level direction differences:
    positions, times and weights agree to 1e-4 for >= 99% of histories."""
    g, o = _pair("tiny_2d", gpu_lib, PRECISION=np.float32)
    for e in (g, o):
        e.update()
        e.sourcing()
    _cmp_particles(g, o, rtol=1e-6, keys=("t", "x", "y", "E", "E0"))
    for e in (g, o):
        e.transport()
    _cmp_particles(g, o, rtol=1e-4, frac_ok=0.99, keys=("t", "x", "y", "E"))
    dg, do = g.field("energydep"), o.field("energydep")
    np.testing.assert_allclose(dg, do, rtol=1e-3, atol=1e-6 * np.abs(do).max())


def test_step_parity_fp32_2d(gpu_lib):
    """Three FP32 2D steps track the oracle's FP32 steps (fields to 1e-3)."""
    g, o = _pair("tiny_2d", gpu_lib, PRECISION=np.float32)
    for _ in range(3):
        sg, _ = g.step()
        so, _ = o.step()
        assert sg["n_sourced"] == so["n_sourced"]
        assert abs(sg["n_census_out"] - so["n_census_out"]) <= max(3, 1e-3 * so["n_census_out"])
    for f in ("temp", "radenergydens", "matenergydens"):
        a, b = g.field(f), o.field(f)
        np.testing.assert_allclose(a, b, rtol=1e-3, atol=1e-6 * np.abs(b).max(), err_msg=f)


def test_energy_conservation_fp64(gpu_lib):
    """src/imc_energycheck.jl:34 balance in FP64 over the whole C1 run.  In the
    reference's form (relative to the step's source energy) <= 1e-10 on every
    step but the CONSTANT clock's last one, whose dt is a rounding residue
    of t_end and whose source is a vanishing fraction of the energy in play;
    relative to all the energy in play (source + census carried in) <= 1e-12
    on every step, the last included."""
    import mpimc
    inputs, mesh = load_deck("c1_slab")
    g = mpimc.Engine(inputs, mesh)
    steps, _ = g.run()
    assert len(steps) == 101
    for s in steps:
        in_play = abs(s["energy_error"] * s["total_energy"]) / (s["total_energy"] + s["rad_energy_old"])
        assert in_play <= 1e-12, s
        if s["dt"] > 1e-9 * 0.01:
            assert abs(s["energy_error"]) <= 1e-10, s


def test_fp16_state_balance_within_storage_rounding(gpu_lib):
    """FP16 particle state stores each census energy as E/E0 in binary16, so a
    step's balance misses at most the rounding of the census energy:
    |error| <= 2^-11 E_rad / E_src (plus the FP32 arithmetic's 1e-6)."""
    import mpimc
    inputs, mesh = load_deck("c1_slab", PRECISION=np.float16)
    g = mpimc.Engine(inputs, mesh)
    steps, _ = g.run(max_steps=60)
    worst = 0.0
    for s in steps:
        bound = 2.0 ** -11 * s["rad_energy"] / s["total_energy"] + 1e-6
        assert abs(s["energy_error"]) <= bound, s
        worst = max(worst, abs(s["energy_error"]) / bound)
    assert worst > 0.0


def test_run_matches_step(gpu_lib):
    """The graph-replayed run and stage-by-stage steps give identical fields."""
    import mpimc
    inputs, mesh = load_deck("tiny_1d")
    a = mpimc.Engine(inputs, mesh)
    b = mpimc.Engine(inputs, mesh)
    sa, _ = a.run()
    sb = []
    done = False
    while not done:
        st, done = b.step()
        sb.append(st)
    assert len(sa) == len(sb)
    for f in ("temp", "radenergydens", "matenergydens", "energydep"):
        np.testing.assert_array_equal(a.field(f), b.field(f), err_msg=f)


def test_bit_reproducible(gpu_lib):
    """Fixed-point tallies: two runs give bit-identical fields."""
    import mpimc
    inputs, mesh = load_deck("c1_slab", PRECISION=np.float32)
    out = []
    for _ in range(2):
        e = mpimc.Engine(inputs, mesh)
        e.run(max_steps=20)
        out.append([e.field(f) for f in ("temp", "radenergydens", "energydep")])
        e.close()
    for x, y in zip(*out):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("dx", ["0.0025", "0.002"])
def test_step_parity_fp64_large_slab(gpu_lib, dx):
    """Slabs past the shared-memory tallies: 4000 cells (FP64 table and
    deposition tallies in shared memory, census tallies in global memory) and
    5000 cells (every tally in global memory, warp-combined; the FP64 table
    alone still fits, up to ~7000 cells); three steps still track the
    oracle."""
    g, o = _pair("c1_slab", gpu_lib, DX=dx, NINPUT="20000", NMAX="200000")
    assert len(g.field("temp")) == (4000 if dx == "0.0025" else 5000)
    for _ in range(3):
        sg, _ = g.step()
        so, _ = o.step()
        assert sg["n_sourced"] == so["n_sourced"]
        np.testing.assert_allclose(sg["energy_error"], so["energy_error"], atol=1e-9)
    for f in ("temp", "radenergydens", "matenergydens"):
        a, b = g.field(f), o.field(f)
        np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-9 * np.abs(b).max(), err_msg=f)


@pytest.mark.parametrize("ysize", ["0.625", "1.0"])
def test_step_parity_fp64_2d_large_mesh(gpu_lib, ysize):
    """2D meshes past the shared-memory tallies: 80x50 cells (FP64 table and
    deposition tallies in shared memory, census tallies in global memory) and
    80x80 cells (every tally in global memory) track the oracle for three
    steps."""
    g, o = _pair("tiny_2d", gpu_lib, MESHTYPE="UNIFORM", XSIZE="1.0", YSIZE=ysize, DX="0.0125", DY="0.0125",
                 NINPUT="20000", NMAX="60000")
    assert len(g.field("temp")) == (4000 if ysize == "0.625" else 6400)
    for _ in range(3):
        sg, _ = g.step()
        so, _ = o.step()
        assert sg["n_sourced"] == so["n_sourced"]
        assert abs(sg["n_census_out"] - so["n_census_out"]) <= max(2, 1e-4 * so["n_census_out"])
        np.testing.assert_allclose(sg["total_energy"], so["total_energy"], rtol=1e-13)
    for f in ("temp", "radenergydens", "matenergydens"):
        a, b = g.field(f), o.field(f)
        np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-9 * np.abs(b).max(), err_msg=f)


# FP32 selection needs products beyond binary32's range to fall back
_MULTISCALE = {
    "fp16": {"PRECISION": np.float16},
    "fp32": {"PRECISION": np.float32, "ENERGYSCALES": ["1e38", "1000.0", "1.0"],
             "RADSOURCE_VALS": ["1e6", "1e4", "100.0", "0.01", "0.0"]},
}


@pytest.mark.parametrize("prec", ["fp16", "fp32"])
def test_multiscale_sorter_fallback_parity(gpu_lib, prec):
    """Utilities.sorter's retry with the next energy scale
    (src/imc_utilities.jl:23-54) on the device, in the deck precision: the
    multi-scale slab's slots overflow binary16 (binary32) at the first scales,
    so its births carry several scale indices.  Sourcing equals the oracle
    particle for particle (scale index included); three steps track the
    oracle's fields and balance."""
    g, o = _pair("multiscale_1d", gpu_lib, **_MULTISCALE[prec])
    for e in (g, o):
        e.update()
        e.sourcing()
    assert g.num_particles() == o.num_particles() > 0
    pg, po = g.particles(), o.particles()
    assert len(np.unique(po["scale"])) >= 2, "the deck no longer exercises the fallback"
    np.testing.assert_array_equal(pg["scale"], po["scale"])
    np.testing.assert_allclose(g.field("emittedenergy"), o.field("emittedenergy"), rtol=1e-14)
    _cmp_particles(g, o, rtol=1e-6, keys=("t", "x", "mu", "E", "E0"))
    g, o = _pair("multiscale_1d", gpu_lib, **_MULTISCALE[prec])
    for s in range(3):
        sg, _ = g.step()
        so, _ = o.step()
        assert sg["n_sourced"] == so["n_sourced"]
        assert sg["error_flags"] == 0
        # the first step's energies come from the deck alone; later ones from
        # temperatures that carry the transports' last-ulp differences
        np.testing.assert_allclose(sg["total_energy"], so["total_energy"], rtol=1e-13 if s == 0 else 1e-6)
        assert abs(sg["energy_error"] - so["energy_error"]) < 1e-4
    for f in ("temp", "radenergydens", "matenergydens"):
        a, b = g.field(f), o.field(f)
        np.testing.assert_allclose(a, b, rtol=2e-3, atol=1e-6 * np.abs(b).max(), err_msg=f)
