"""Host logic on the CPU: the deck grammar of src/imc_input.jl, mesh generation
of src/imc_mesh.jl, the SimVars / timestep control of
src/MixedPrecisionIMC.jl, and the reference test suite's input checks
(test/runtests.jl:37-52)."""
import os

import numpy as np
import pytest

from conftest import DECKS, REFERENCE, deck_path, load_deck, reference_file

import mpimc
from mpimc import Input, Mesh


def test_reference_style_input_checks():
    inputs = Input.readInputs(deck_path("tiny_2d"))
    assert inputs and isinstance(inputs, dict) and "PRECISION" in inputs
    mpimc.Constants.set_constants(inputs)
    assert isinstance(mpimc.Constants.phys_c, np.float64)
    mesh = Mesh.mesh_generation(inputs)
    assert isinstance(mesh.nodes, tuple) and all(isinstance(n, np.ndarray) for n in mesh.nodes)


def test_grammar(tmp_path):
    p = tmp_path / "d.txt"
    p.write_text("""NAME = x y
# comment
PRECISION = FLOAT32

A = [1.0, 2.5,
     3.0,
     4.0]
B = [7.5]
C = []
XMESHNODES = [0.0, 0.1,
  0.30000000000000004]
T_SURFACE_REGS = [(7.0),(7.0),(0.5,2.0),(2.0)]
REGS = [((0.0, 7.0),(0.0,2.0)) , ((0.0, 3.0),(0.0,0.5))]
D = 3 = 4
lower = 1
""")
    d = Input.readInputs(str(p))
    assert d["PRECISION"] is np.float32
    assert d["NAME"] == "x y"
    assert [float(v) for v in d["A"]] == [1.0, 2.5, 3.0, 4.0] and isinstance(d["A"][0], np.float32)
    assert d["B"] == ["7.5"] and d["C"] == [""]
    assert d["XMESHNODES"][2] == 0.30000000000000004 and isinstance(d["XMESHNODES"][2], np.float64)
    assert d["T_SURFACE_REGS"] == [(7.0, 7.0, (0.5, 2.0), 2.0)]
    assert d["REGS"] == [(((0.0, 7.0), (0.0, 2.0)), ((0.0, 3.0), (0.0, 0.5)))]
    assert d["D"] == "3"
    assert d["lower"] == "1"


def test_tuple_arrays_are_not_executed(tmp_path):
    p = tmp_path / "d.txt"
    p.write_text("PRECISION = FLOAT64\nX = [(__import__('os').system('false'), 1)]\n")
    with pytest.raises((ValueError, SyntaxError)):
        Input.readInputs(str(p))


def test_mesh_1d_uniform_regions():
    inputs, mesh = load_deck("c1_slab")
    assert mesh.Ncells == 100 and np.all(mesh.dx == 0.1)
    src = mesh.radsource
    assert np.all(src[:5] == 1.0) and np.all(src[5:] == 0.0)
    assert mesh.sigma_a.shape == (100, 3) and np.all(mesh.sigma_a[:, 0] == 1.0)
    assert list(mesh.energyscales) == [1.0]


def test_mesh_1d_nonuniform_and_scales():
    inputs, mesh = load_deck("tiny_1d")
    assert mesh.Ncells == 10
    np.testing.assert_allclose(mesh.dx, np.diff([0.0, 0.05, 0.1, 0.2, 0.3, 0.35, 0.4, 0.5, 0.6, 0.8, 1.0]))
    assert list(mesh.energyscales) == [4.0, 1.0]
    assert np.all(mesh.sigma_a[:4, 1] == 5.0) and np.all(mesh.sigma_a[4:, 1] == 1.0)
    assert np.all(mesh.sigma_a[4:, 2] == -1.0)


def test_mesh_2d_regions_and_surfaces():
    inputs, mesh = load_deck("c4_channel2d")
    assert mesh.Ncells == (140, 40)
    sa = mesh.sigma_a[..., 1]
    # channel on x in [0, 3], y in [0, 0.5]; walls elsewhere
    assert sa[0, 0] == np.float32(0.2) and sa[10, 9] == np.float32(0.2)
    assert sa[10, 20] == 2000.0 and sa[139, 39] == 2000.0
    left = mesh.temp_surf[2]
    assert np.all(left[:10] == 0.5) and np.all(left[10:] == 0.0)
    assert all(np.all(f == 0) for f in (mesh.temp_surf[0], mesh.temp_surf[1], mesh.temp_surf[3]))


def test_linrange_matches_julia_rule():
    n = Mesh.linrange(0.0, 10.0, 2001, np.float64)
    assert n[0] == 0.0 and n[-1] == 10.0 and n[100] == 100 / 2000 * 10.0


def test_timestep_constant_and_ramp():
    sv = mpimc.SimVars(0.0, 0.3, 0.0, 0.0, 0.0, 1.0, [], 0, 1, 1, 1.0, "FALSE", ("VACUUM", "VACUUM"),
                       np.float64, "1D")
    ts = []
    while sv.t <= sv.t_end:
        ts.append(sv.t)
        mpimc.timestep("CONSTANT", sv)
    assert ts == [0.0, 0.3, 0.6, 0.8999999999999999, 1.0]
    sv = mpimc.SimVars(0.0, 0.1, 0.1, 2.0, 0.35, 1.0, [], 0, 1, 1, 1.0, "FALSE", ("VACUUM", "VACUUM"),
                       np.float64, "1D")
    dts = []
    while sv.t <= sv.t_end:
        dts.append(sv.dt)
        mpimc.timestep("RAMP", sv)
    assert dts[:4] == [0.1, 0.2, 0.35, 0.35]


def test_build_deck_layout():
    import ctypes as C
    from mpimc._lib import ImcDeck
    inputs, mesh = load_deck("tiny_2d")
    d, keep = mpimc.build_deck(inputs, mesh)
    assert (d.nx, d.ny, d.geometry) == (9, 3, 2)
    temp = np.ctypeslib.as_array(d.temp, shape=(27,))
    assert np.all(temp == 0.2)
    sa = np.ctypeslib.as_array(d.sigma_a_val, shape=(27,)).reshape((9, 3), order="F")
    assert sa[2, 1] == 30.0 and sa[2, 0] == 2.0 and sa[0, 2] == 2.0
    ts = np.ctypeslib.as_array(d.t_surface, shape=(2 * 9 + 2 * 3,))
    assert list(ts[18:21]) == [0.5, 0.5, 0.1]  # left face: segment ends at y = 0.5
    assert list(d.bc) == [0, 1, 0, 1]
    # the C struct size the library expects: 6 ints, 10 pointers, ...
    assert C.sizeof(ImcDeck) == 6 * 4 + 10 * 8 + 16 + 24 + 8 + 8 + 8 + 16 + 8 + 8 + 8 + 8 + 8 + 40 + 16


@pytest.mark.skipif(reference_file("src/inputs") is None, reason="IMC_REFERENCE unset or without src/inputs")
@pytest.mark.parametrize("name", ["SuOlson", "MarshakWave", "InfiniteMedium", "1DNonUniform", "2DNonUniform",
                                  "CrookedPipe"])
def test_reference_decks_parse_and_mesh(name):
    inputs = Input.readInputs(os.path.join(REFERENCE, "src/inputs", name + ".txt"))
    mesh = Mesh.mesh_generation(inputs)
    d, _ = mpimc.build_deck(inputs, mesh)
    assert d.nx > 0 and d.n_scales >= 1


@pytest.mark.skipif(reference_file("test/test_input.txt") is None,
                    reason="reference checkout not present")
def test_reference_test_deck():
    """The reference suite's own deck: readInputs gives a non-empty Dict with
    PRECISION, phys_c is Float64 and mesh.nodes is a pair of Float64 vectors
    (test/runtests.jl:37-52)."""
    inputs = Input.readInputs(os.path.join(REFERENCE, "test/test_input.txt"))
    assert inputs and "PRECISION" in inputs
    mpimc.Constants.set_constants(inputs)
    assert isinstance(mpimc.Constants.phys_c, np.float64)
    mesh = Mesh.mesh_generation(inputs)
    assert isinstance(mesh.nodes, tuple) and all(n.dtype == np.float64 for n in mesh.nodes)
