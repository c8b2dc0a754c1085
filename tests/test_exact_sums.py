"""Exact per-bin sums (include/mcgpu.h, MC_EXACT_LIMBS): the representation,
the merge of disjoint parts and the rounding to the nearest double, on the
host (no GPU).  mc_exact_round is host arithmetic in the library; the Python
restatement in mcgpu/parallel.py is checked against Python's integer true
division, which rounds correctly, and against math.fsum, which returns the
correctly rounded sum of a list of doubles."""
import math
import random

import numpy as np
import pytest

from mcgpu import parallel as P

K = P.EXACT_LIMBS


def _random_double(rng):
    kind = rng.random()
    if kind < 0.1:
        return rng.choice([5e-324, 2.2250738585072014e-308, 1e150, 1.0, -1.0])
    if kind < 0.2:
        return math.ldexp(rng.randrange(1, 1 << 52), -1074)        # subnormal
    e = rng.randrange(-1000, 500)      # squares stay finite
    return math.copysign(math.ldexp(1.0 + rng.random(), e), rng.random() - 0.3)


def test_limbs_round_trip_and_normal_form():
    rng = random.Random(1)
    for _ in range(300):
        M = rng.getrandbits(rng.randrange(1, 2100)) * rng.choice([1, -1])
        limbs = P.limbs_of_int(M)
        assert P.int_of_limbs(limbs) == M
        assert np.all((limbs[:-1] >= 0) & (limbs[:-1] < 2 ** 32))


def test_library_rounding_matches_correct_rounding():
    """mc_exact_round on normalised and on carry-save (unnormalised) limbs,
    random magnitudes from subnormal to ~1e300, both signs, and exact ties."""
    import mcgpu
    rng = random.Random(2)
    vals, want = [], []
    for i in range(2000):
        bits = rng.randrange(1, 2100)
        M = rng.getrandbits(bits) * rng.choice([1, -1])
        if i % 7 == 0 and bits > 60:          # an exact tie between two doubles
            top = M.bit_length()
            M = (abs(M) >> (top - 54)) << (top - 54) | (1 << (top - 55))
        limbs = P.limbs_of_int(M)
        if i % 3 == 0:                         # carry-save form: move value between limbs
            j = rng.randrange(0, K - 1)
            c = rng.randrange(-1000, 1000)
            limbs[j] += c << 32
            limbs[j + 1] -= c
        vals.append(limbs)
        want.append(M / (1 << 1074))
    got = mcgpu.exact_round(np.array(vals))
    assert np.array_equal(got.view(np.uint64), np.array(want).view(np.uint64))
    assert np.array_equal(P.round_exact(np.array(vals)).view(np.uint64), np.array(want).view(np.uint64))


def test_exact_sums_equal_fsum_and_merge_in_any_order():
    """Per-history rows split into parts in any way: the merged exact sums
    are the exact sums of the whole, and they round to math.fsum."""
    rng = random.Random(3)
    rows = np.array([[_random_double(rng) if rng.random() < 0.7 else 0.0 for _ in range(4)] for _ in range(200)])
    whole = P.exact_limbs_from_values(rows)
    for cut in ((0, 200), (0, 1, 200), (0, 37, 38, 150, 200)):
        parts = [P.exact_limbs_from_values(rows[a:b]) for a, b in zip(cut[:-1], cut[1:])]
        for order in (parts, parts[::-1]):
            assert np.array_equal(P.merge_exact(order), whole)
    r = P.round_exact(whole)
    for b in range(rows.shape[1]):
        assert r[b, 0] == math.fsum(rows[:, b])
        assert r[b, 1] == math.fsum(rows[:, b] * rows[:, b])
