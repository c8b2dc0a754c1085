"""Particle comb (population_control.cpp:55-84, setup.cpp:57-67) on the GPU.

The comb runs in the history-ordered FP64 modes.  Replay reproduces the
oracle's event digests and tally sums bit for bit for several (bank_max,
teeth) pairs.  The oracle's comb is pinned to the compiled reference's own
particle_comb by the comb_slab golden fixture.  Plain FP64 agrees with replay
statistically.  The event engine and batches refuse a combed problem with a
status, because they keep no per-history bank."""
import tempfile

import numpy as np
import pytest

import cases
from helpers import same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mc():
    import build as B
    B.build()
    import mcgpu
    return mcgpu


@pytest.mark.parametrize("bank_max,teeth", [(1, 1), (2, 2), (4, 1), (5, 3), (12, 7)])
def test_comb_replay_bit_exact_vs_oracle(mc, bank_max, teeth):
    from oracle import problem as OP
    with tempfile.TemporaryDirectory() as d:
        cases.comb_slab(d, samples=1500, bank_max=bank_max, teeth=teeth)
        p = mc.Problem(d, d + "/xs_library")
        c = p.run(mode="replay", record_digests=1)
        _, _, s, q = p.all_tallies()
        dg = p.digests(p.nsample)
        pb = OP.load(d, xs_dir=d + "/xs_library")
        r = OP.run(pb, seed=mc.DEFAULT_SEED, digests=True)
        p.close()
    assert r.status == 0
    assert np.array_equal(dg, r.digest)
    assert same_bits(s, r.sum) and same_bits(q, r.sq)
    assert c["flights"] == int(r.counters[0]) and c["splits"] == int(r.counters[5])


def test_comb_plain_agrees_with_replay(mc):
    with tempfile.TemporaryDirectory() as d:
        cases.comb_slab(d, samples=20000, bank_max=3, teeth=2)
        p = mc.Problem(d, d + "/xs_library")
        p.run(mode="replay")
        m1, s1, _, _ = p.all_tallies()
        p.reset()
        p.run(mode="plain", seed=mc.DEFAULT_SEED + 1)
        m2, s2, _, _ = p.all_tallies()
        p.close()
    both = (s1 > 0) & (s2 > 0)
    z = np.abs(m1 - m2)[both] / np.sqrt(s1[both] ** 2 + s2[both] ** 2)
    assert both.sum() > 50 and np.mean(z <= 3.0) >= 0.97, np.sort(z)[-5:]


def test_comb_refused_where_no_history_bank_exists(mc):
    with tempfile.TemporaryDirectory() as d:
        cases.comb_slab(d, samples=100)
        p = mc.Problem(d, d + "/xs_library")
        with pytest.raises(mc.McError) as e:
            p.run(mode="event")
        assert e.value.status == 1 and "comb" in str(e.value)
        with pytest.raises(mc.McError) as e:
            mc.Batch([p], [100])
        assert e.value.status == 1
        p.run(n=50, mode="replay")     # the handle stays usable
        p.close()
