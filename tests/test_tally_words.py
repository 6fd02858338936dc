"""The shared-memory tally arithmetic of the transport kernels, restated on
the CPU and checked for exactness.

A block-private tally slot holds, per limb position, a 32-bit word that wraps
and a signed carry count (imc_transport.cuh: add_word_smem, folded into the
three int64 accumulators by flush_block_tallies).  The 3-limb fixed-point
value of a flush (imc_device.cuh: fix_split / fix_place) has limbs of weight
2^64, 2^32 and 1 with |limb| < 2^32, all of one sign.  Whatever the order of
the adds, the folded slot must equal the exact sum of the flushed values;
the GPU parity tests check the kernels against the oracle, this checks the
scheme itself over adversarial orders and wrap-heavy inputs."""
import random

import pytest

MASK = (1 << 32) - 1


def add_word(w, cy, limb):
    """add_word_smem: the 32-bit add returns the old word; a wrap bumps the
    carry count, a negative limb enters as 2^32 + limb with a carry of -1."""
    u = limb & MASK
    old = w
    w = (old + u) & MASK
    c = (1 if old + u > MASK else 0) - (1 if limb < 0 else 0)
    return w, cy + c


def fold(w, cy):
    """flush_block_tallies: limb q gets its word plus the carries out of the
    limb below it; the top limb also takes its own carries times 2^32."""
    v0 = w[0] + cy[1] + cy[0] * (1 << 32)
    v1 = w[1] + cy[2]
    v2 = w[2]
    return v0, v1, v2


def value(v0, v1, v2):
    return (v0 << 64) + (v1 << 32) + v2


def limbs_of(V):
    """A fixed-point value |V| < 2^94 as fix_place splits it: limbs of one
    sign, |limb| < 2^32 (top limb < 2^30)."""
    neg = V < 0
    m = -V if neg else V
    l2, l1, l0 = m & MASK, (m >> 32) & MASK, m >> 64
    s = -1 if neg else 1
    return s * l0, s * l1, s * l2


def accumulate(values):
    w, cy = [0, 0, 0], [0, 0, 0]
    for V in values:
        for q, limb in enumerate(limbs_of(V)):
            if limb:
                w[q], cy[q] = add_word(w[q], cy[q], limb)
    return value(*fold(w, cy))


@pytest.mark.parametrize("seed", range(6))
def test_word_carry_tally_is_exact_in_any_order(seed):
    rng = random.Random(seed)
    # magnitudes over the whole fixed-point range, low words near 2^32 so the
    # words wrap on most adds, and a few negative values (compensation terms)
    vals = []
    for _ in range(3000):
        e = rng.randrange(0, 93)
        V = rng.randrange(1 << e, 1 << (e + 1))
        V |= MASK if rng.random() < 0.3 else 0
        vals.append(-V if rng.random() < 0.05 else V)
    exact = sum(vals)
    for _ in range(4):
        rng.shuffle(vals)
        assert accumulate(vals) == exact


def test_word_carry_tally_many_maximal_low_words():
    # every add wraps the low word: the carry count carries the whole sum
    vals = [MASK] * 100000
    assert accumulate(vals) == MASK * 100000
    vals = [(1 << 93) - 1] * 64 + [-((1 << 93) - 1)] * 63
    assert accumulate(vals) == (1 << 93) - 1


def test_limbs_match_the_device_split():
    # fix_place's limbs for a few values (signed, one sign for all limbs)
    assert limbs_of(0) == (0, 0, 0)
    assert limbs_of(1) == (0, 0, 1)
    assert limbs_of(-(1 << 40) - 5) == (0, -(1 << 8), -5)
    assert limbs_of((1 << 70) + (3 << 32) + 7) == (1 << 6, 3, 7)
