"""The device building blocks, checked on the CPU through their host paths
(imc_device.cuh is __host__ __device__): Philox known answers, the stream
layout shared with the oracle, exact order-independent fixed-point tallies,
and the sorter against the oracle's restatement."""
import os
import random
import subprocess
from fractions import Fraction

import numpy as np
import pytest

from conftest import REPO

import oracle

SRC = os.path.join(REPO, "tests", "native", "device_host_check.cu")
BIN = os.path.join(REPO, "tests", "native", "_build", "device_host_check")


@pytest.fixture(scope="module")
def tool():
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    hdr = os.path.join(REPO, "mixedprecisionimc.jl_gb300", "csrc", "imc_device.cuh")
    if not os.path.exists(BIN) or os.path.getmtime(BIN) < max(os.path.getmtime(SRC), os.path.getmtime(hdr)):
        nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
        subprocess.run([nvcc if os.path.exists(nvcc) else "nvcc", "-std=c++17", "-O2", "-Xcompiler",
                        "-ffp-contract=off", SRC, "-o", BIN], check=True)

    def ask(lines):
        r = subprocess.run([BIN], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
        return r.stdout.strip().split("\n")
    return ask


def test_philox_kat_host_path(tool):
    out = tool(["P 0 0 0 0 0 0", "P 4294967295 4294967295 4294967295 4294967295 4294967295 4294967295",
                "P 608135816 2242054355 320440878 57701188 2752067618 698298832"])
    assert [list(map(int, o.split())) for o in out] == [
        [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8],
        [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd],
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]]


def test_stream_layout_matches_oracle(tool):
    seed, step, pid, stage = 0x123456789ABCDEF, 7, 4242, 1
    out = list(map(int, tool(["S %d %d %d %d 9" % (seed, step, pid, stage)])[0].split()))
    exp = []
    for blk in range(3):
        exp += oracle.philox([blk, step, pid, stage], [seed & 0xFFFFFFFF, seed >> 32])
    assert out == exp[:9]


def _exact(vals, b):
    return sum(Fraction(v).limit_denominator(1 << 2000) if False else Fraction(v) for v in vals)


def test_fixed_point_exact_and_order_independent(tool):
    rng = random.Random(5)
    vals = [rng.uniform(0, 1) * 10 ** rng.uniform(-12, 0) for _ in range(300)]
    vals += [-rng.uniform(0, 1e-9) for _ in range(20)]  # compensation terms may be negative
    b = -95 + 1  # exponent for vmax = 1
    lines = []
    for _ in range(4):
        rng.shuffle(vals)
        lines.append("F %d %s ." % (b, " ".join(repr(v) for v in vals)))
    out = [o.split() for o in tool(lines)]
    assert all(o[0] == "1" for o in out)
    assert len({tuple(o[1:4]) for o in out}) == 1  # identical limb sums in every order
    total = float(out[0][4])
    exact = float(sum(Fraction(v) for v in vals))
    # each value is rounded to 2^b once: error <= n * 2^(b-1)
    assert abs(total - exact) <= len(vals) * 2.0 ** (b - 1) + abs(exact) * 2 ** -52


def test_fixed_point_range_flag(tool):
    out = tool(["F 0 1e40 ."])[0].split()
    assert out[0] == "0"


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_sorter_matches_oracle(tool, prec):
    rng = np.random.default_rng(prec)
    lines, cases = [], []
    for _ in range(40):
        n = int(rng.integers(2, 12))
        v = (10.0 ** rng.uniform(-6, 6, n)).tolist()
        s = sorted((2.0 ** rng.integers(-20, 20, int(rng.integers(1, 5)))).tolist(), reverse=True)
        lines.append("R %d %d %s %d %s" % (prec, n, " ".join(repr(x) for x in v), len(s), " ".join(repr(x) for x in s)))
        cases.append((v, s))
    out = tool(lines)
    for (v, s), o in zip(cases, out):
        p_hex, j = o.split()
        p, _, jo = oracle.sorter(v, s, prec)
        assert int(j) == jo
        assert float.fromhex(p_hex) == p


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_sorter_special_values_match_oracle(tool, prec):
    """isless order with signed zeros, infinities, NaN, negatives and ties:
    the register sort of the device header (integer isless keys) picks the
    same product and scale as the oracle's restated insertion sort."""
    rng = np.random.default_rng(10 + prec)
    special = [0.0, -0.0, np.inf, -np.inf, np.nan, -1.5, 2.0, 2.0, 1e-300, -1e300, 3.0e38, 7e4]
    lines, cases = [], []
    for _ in range(200):
        n = int(rng.integers(1, 13))
        v = [float(special[k]) if rng.uniform() < 0.5 else float(10.0 ** rng.uniform(-8, 8))
             for k in rng.integers(0, len(special), n)]
        s = [float(x) for x in rng.choice([1.0, 2.0 ** -30, 2.0 ** 30, -4.0, 0.0], int(rng.integers(1, 4)))]
        lines.append("R %d %d %s %d %s" % (prec, n, " ".join(repr(x) for x in v), len(s),
                                           " ".join(repr(x) for x in s)))
        cases.append((v, s))
    out = tool(lines)
    for (v, s), o in zip(cases, out):
        p_hex, j = o.split()
        p, _, jo = oracle.sorter(v, s, prec)
        assert int(j) == jo, (v, s)
        pg = float.fromhex(p_hex)
        assert pg == p and np.signbit(pg) == np.signbit(p), (v, s, pg, p)


def test_f32_two_word_placement_equals_fix_split(tool):
    """The shared-memory flush's FP32 path (f32_words: a positive normal value
    as at most two adjacent 32-bit words) places exactly the bits fix_split
    does wherever it applies, and declines zero, subnormal, negative,
    non-finite, below-resolution and out-of-range values (left to fix_split)."""
    rng = np.random.default_rng(3)
    took = 0
    for b in (-93, -60, -30, 0, 17):
        vals = list(np.float32(rng.uniform(0.5, 1.0, 200) * 2.0 ** rng.integers(-80, 40, 200)))
        vals += [np.float32(2.0 ** e) for e in range(-149, 128, 7)]
        vals += [0.0, -1.5, np.float32(1e-45), float("inf"), float("nan"), np.float32(3.4e38)]
        toks = ["%r" % float(v) for v in vals]
        out = tool(["W %d %s ." % (b, " ".join(toks))])
        assert len(out) == len(vals)
        for v, line in zip(vals, out):
            f, w2, w1, w0, ok, l0, l1, l2 = map(int, line.split())
            if f:
                took += 1
                assert ok == 1 and (w2, w1, w0) == (l0, l1, l2), (b, v, line)
                assert v > 0 and np.isfinite(v)
            elif ok == 1 and v > 0 and np.float32(v) >= np.float32(2.0 ** -126):
                # declined although fix_split places it: only below the
                # resolution (fix_split rounds there)
                e = int(np.floor(np.log2(v)))
                assert e - 23 - b < 0, (b, v, line)
    assert took > 300



def test_binary32_birth_angle_equals_float64_rounding(tool):
    """two_pi_u24 (2D births, FP32 / FP16 state) equals the reference's
    Float64 2 pi rand rounded to binary32 for all 2^24 uniforms."""
    out = tool(["A"])
    assert out == ["done 0"], out


def test_binary32_cutoff_energy_equals_float64_rounding(tool):
    """cutoff_energy (the 1 % cut-off of FP32 / FP16 state) equals the
    reference's Float64 0.01 E0 rounded to binary32 for every non-negative
    binary32 and infinity (about 30 s on one core)."""
    out = tool(["C"])
    assert out == ["done 0"], out


def test_binary32_surface_birth_angles_equal_float64_rounding(tool):
    """pi_n24 (2D surface births, FP32 / FP16 state) gives the reference's
    Float64 angles -pi u and pi (1/2 - u) rounded to binary32 for all 2^24
    uniforms u."""
    out = tool(["B"])
    assert out == ["done 0"], out
