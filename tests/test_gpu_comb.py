"""Particle comb (population_control.cpp:55-84, setup.cpp:57-67) on the GPU.

The comb runs in the history-ordered FP64 modes and in the per-thread FP32
kernel, each of which keeps one history's bank.  Replay reproduces the
oracle's event digests and tally sums bit for bit for several (bank_max,
teeth) pairs.  The oracle's comb is pinned to the compiled reference's own
particle_comb by the comb_slab golden fixture.  Plain FP64 and the mixed
per-thread kernel agree with replay statistically, and a batch runs every
combed problem as its lone run does.  The tile kernel refuses a combed
problem with a status, because it keeps no per-history bank."""
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


@pytest.mark.parametrize("bank_max,teeth", [(3, 2), (1, 1), (6, 4)])
def test_comb_mixed_agrees_with_replay(mc, bank_max, teeth):
    """The per-thread kernel's comb (FP32 tracking, FP64 weight sums) against
    FP64 replay of the same problem: every resolved bin within 3 sigma in at
    least 97 % of the bins, and the population per history equal in
    expectation (particles / histories within 5 sigma of replay's)."""
    with tempfile.TemporaryDirectory() as d:
        cases.comb_slab(d, samples=40000, bank_max=bank_max, teeth=teeth)
        p = mc.Problem(d, d + "/xs_library")
        cr = p.run(mode="replay")
        m1, s1, _, _ = p.all_tallies()
        p.reset()
        ce = p.run(mode="event", seed=mc.DEFAULT_SEED + 7, kernel=2)
        m2, s2, _, _ = p.all_tallies()
        p.close()
    both = (s1 > 0) & (s2 > 0)
    z = np.abs(m1 - m2)[both] / np.sqrt(s1[both] ** 2 + s2[both] ** 2)
    assert both.sum() > 50 and np.mean(z <= 3.0) >= 0.97, np.sort(z)[-5:]
    assert ce["histories"] == cr["histories"]
    # particles per history: a rough check that the comb fires as often
    a, b = cr["particles"] / cr["histories"], ce["particles"] / ce["histories"]
    assert abs(a - b) <= 0.05 * a, (a, b)


def test_comb_mixed_default_shape_and_tuned_tile_shape(mc):
    """Without a tune the mixed mode runs the per-thread kernel; a problem
    autotuned with the comb picks a per-thread shape."""
    with tempfile.TemporaryDirectory() as d:
        cases.comb_slab(d, samples=2000, bank_max=3, teeth=2)
        p = mc.Problem(d, d + "/xs_library")
        c = p.run(mode="event")
        assert c["histories"] == 2000
        t = p.autotune(sample=4000)
        assert t["kernel"] == 2
        p.reset()
        p.run(mode="event")
        p.close()


def test_comb_refused_where_no_history_bank_exists(mc):
    with tempfile.TemporaryDirectory() as d:
        cases.comb_slab(d, samples=100)
        p = mc.Problem(d, d + "/xs_library")
        with pytest.raises(mc.McError) as e:
            p.run(mode="event", kernel=1)
        assert e.value.status == 8
        with pytest.raises(mc.McError) as e:
            p.run(mode="event", kernel=3)   # the event-split engine keeps no per-history bank either
        assert e.value.status == 8 and "comb" in str(e.value)    # MC_ERR_ARG
        b = mc.Batch([p], [100])
        with pytest.raises(mc.McError) as e:
            b.run(seed=3, kernel=1)
        assert e.value.status == 8 and "comb" in str(e.value)
        b.close()
        p.run(n=50, mode="replay")     # the handle stays usable
        p.close()


def test_comb_in_a_batch_equals_lone_runs(mc):
    """A batch mixing combed problems (different bank_max / teeth) with an
    uncombed one: problem i follows the histories of its lone run with seed
    batch_problem_seed(seed, i), so the event counts of the whole batch
    equal the sum of the lone runs' and every tally agrees."""
    import os
    seed = 4242
    settings = [(3, 2), (1, 1), (6, 4), None]
    hist = [3000, 2000, 2500, 1500]
    with tempfile.TemporaryDirectory() as root:
        probs = []
        for k, st in enumerate(settings):
            d = os.path.join(root, "p%d" % k)
            os.makedirs(d)
            if st is None:
                cases.write_case("slab_features", d)
            else:
                cases.comb_slab(d, samples=hist[k], bank_max=st[0], teeth=st[1])
            probs.append(mc.Problem(d, d + "/xs_library"))
        b = mc.Batch(probs, hist)
        cb = b.run(seed=seed)
        assert cb["histories"] == sum(hist)
        res = [p.all_tallies() for p in probs]
        b.close()
        tot = {}
        for i, p in enumerate(probs):
            p.reset()
            c = p.run(n=hist[i], seed=mc.batch_problem_seed(seed, i), mode="event")
            for k in ("flights", "collisions", "crossings", "tally_updates", "particles", "splits"):
                tot[k] = tot.get(k, 0) + c[k]
            m2, s2, su2, _ = p.all_tallies()
            assert np.allclose(res[i][2], su2, rtol=1e-6, atol=1e-12), f"problem {i}"
            p.close()
    for k, v in tot.items():
        assert cb[k] == v, k
