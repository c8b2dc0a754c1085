"""FP64 replay on the GPU against the oracle and the golden fixtures.

Replay mode must reproduce, bit for bit, every history's event sequence
(per-history digests) and every tally bin of the CPU oracle, which is itself
pinned to the compiled reference (tests/golden)."""
import tempfile

import numpy as np
import pytest

import cases
from helpers import digest_sha, golden_arrays, load_golden, same_bits

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mc():
    import build as B
    B.build()
    import mcgpu
    return mcgpu


def _oracle(d, seed, n=None):
    from oracle import problem as OP
    pb = OP.load(d, xs_dir=d + "/xs_library")
    return OP.run(pb, n=n, seed=seed, digests=True)


@pytest.mark.parametrize("name", list(cases.REFERENCE_CASES))
def test_replay_bit_exact_vs_golden_and_oracle(mc, name):
    g = load_golden(name)
    with tempfile.TemporaryDirectory() as d:
        cases.write_case(name, d)
        p = mc.Problem(d, d + "/xs_library")
        c = p.run(seed=g["seed"], mode="replay", record_digests=1)
        mean, unc, s, q = p.all_tallies()
        dg = p.digests(p.nsample)
        r = _oracle(d, g["seed"])
        p.close()
    gm, gu = golden_arrays(g)
    assert same_bits(mean, gm) and same_bits(unc, gu)
    bad = np.nonzero(dg != r.digest)[0]
    assert bad.size == 0, (f"{bad.size} of {dg.size} history digests differ, first {bad[:5]}: "
                           f"gpu {[hex(int(x)) for x in dg[bad[:3]]]} oracle {[hex(int(x)) for x in r.digest[bad[:3]]]}")
    assert digest_sha(dg) == g["digest_sha256"]
    assert c["flights"] == g["ntrack"]
    assert same_bits(s, r.sum) and same_bits(q, r.sq)
    assert np.array_equal(dg, r.digest)
    for k, name_ in enumerate(["flights", "collisions", "crossings", "tally_updates", "particles",
                               "splits", "xs_evals", "freegas_iters", "nuc_lookups"]):
        assert c[name_] == int(r.counters[k]), name_


def _extension_cases():
    import mcgpu.workloads as W
    return {
        "slab_1g": lambda d: W.slab_1g(d, samples=400, n_flux_bins=20),
        "mg_deep_slab": lambda d: W.mg_deep_slab(d, samples=400, G=6),
        "mg_layered_slab": lambda d: W.mg_layered_slab(d, samples=600),
        "user_nuclides": lambda d: cases.absorber_slab_user_nuclides(d, samples=500),
        # the benchmark configurations as written, on a few hundred histories
        "slab_1g_100_bins": lambda d: W.slab_1g(d, samples=400),
        "mg_deep_slab_30_groups": lambda d: W.mg_deep_slab(d, samples=400),
        "mg_layered_slab_detectors": lambda d: W.mg_layered_slab(d, samples=600, detectors=True),
    }


@pytest.mark.parametrize("name", ["slab_1g", "mg_deep_slab", "mg_layered_slab", "user_nuclides",
                                  "slab_1g_100_bins", "mg_deep_slab_30_groups", "mg_layered_slab_detectors"])
def test_replay_bit_exact_vs_oracle_on_extensions(mc, name):
    """Inputs the reference cannot express (hemisphere source, multigroup
    data, wr/ws override, capture-only user nuclides): GPU replay = oracle.
    Among them the 1-group slab with its 100-bin flux, the 30-group
    deep-penetration slab (importance doubling, wr 0.25 / ws 1) and the
    16-layer slab, each exactly as benchmarked."""
    with tempfile.TemporaryDirectory() as d:
        _extension_cases()[name](d)
        p = mc.Problem(d, d + "/xs_library")
        c = p.run(mode="replay", record_digests=1)
        _, _, s, q = p.all_tallies()
        dg = p.digests(p.nsample)
        r = _oracle(d, mc.DEFAULT_SEED)
        p.close()
    assert same_bits(s, r.sum) and same_bits(q, r.sq)
    assert np.array_equal(dg, r.digest)
    assert c["flights"] == int(r.counters[0])


def test_replay_history_ranges_merge_exactly(mc):
    """Running [0, a) then [a, n) equals one run of [0, n) bit for bit: the
    Philox keying makes history ranges independent (resume = run the rest)."""
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("slab_features", d)
        p = mc.Problem(d, d + "/xs_library")
        p.run(mode="replay")
        one = p.all_tallies()
        p.reset()
        p.run(n=157, first=0, mode="replay")
        p.run(n=p.nsample - 157, first=157, mode="replay")
        two = p.all_tallies()
        p.reset()
        p.run(mode="replay", chunk=64)     # several fold chunks in one call
        three = p.all_tallies()
        p.close()
    for a, b, c in zip(one, two, three):
        assert same_bits(a, b) and same_bits(a, c)


def test_plain_fp64_agrees_statistically(mc):
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("ce_sphere_small", d)
        p = mc.Problem(d, d + "/xs_library")
        p.run(n=4000, mode="replay")
        m1, s1, _, _ = p.all_tallies()
        p.reset()
        p.run(n=4000, mode="plain")
        m2, s2, _, _ = p.all_tallies()
        p.close()
    ok = np.abs(m1 - m2) <= 4 * np.sqrt(s1 ** 2 + s2 ** 2) + 1e-300
    assert ok.mean() > 0.95


def test_absorber_slab_integral_on_gpu(mc):
    with tempfile.TemporaryDirectory() as d:
        cases.absorber_slab_user_nuclides(d, samples=200_000)
        p = mc.Problem(d)
        p.run(mode="replay")
        m, s, _, _ = p.tally(0)
        p.close()
    assert abs(m[0] - 0.0149956) <= 3 * s[0]


def test_split_stack_overflow_is_a_status(mc):
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("slab_features", d)
        p = mc.Problem(d, d + "/xs_library")
        with pytest.raises(mc.McError) as e:
            p.run(mode="replay", stack_depth=1)
        assert e.value.status == 3
        p.reset()
        p.run(n=50, mode="replay")        # the handle stays usable
        p.close()


def test_exact_sums_match_the_oracle_and_merge_bit_exactly(mc):
    """The FP64 modes' exact per-bin sums (mc_exact_sums_read): in replay
    they are the exact sums of the oracle's per-history totals (limb for
    limb); two handles running disjoint halves merged limb by limb equal the
    single run; rounded once they equal math.fsum of the history totals, and
    the running FP64 sums differ from them by rounding only.  After a
    mixed-mode run the exact sums are refused until the next reset."""
    import math
    from mcgpu import parallel
    from oracle import problem as OP
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("slab_features", d)
        n, a = 600, 233
        p = mc.Problem(d, d + "/xs_library")
        p.run(n=n, mode="replay")
        whole = p.exact_sums()
        s_run = p.all_tallies()[2]
        q = mc.Problem(d, d + "/xs_library")
        q.run(n=a, first=0, mode="replay")
        h0 = q.exact_sums()
        q.reset()
        q.run(n=n - a, first=a, mode="replay")
        h1 = q.exact_sums()
        q.reset()
        q.run(n=n, mode="plain")               # plain FP64 keeps exact sums too
        plain = q.exact_sums()
        plain_run = q.all_tallies()[2]
        q.run(n=100, first=n, mode="event")
        with pytest.raises(mc.McError) as e:
            q.exact_sums()
        assert e.value.status == 8
        q.reset()
        assert q.exact_sums().shape == whole.shape
        q.close()
        p.close()
        r = OP.run(OP.load(d, xs_dir=d + "/xs_library"), n=n, hist=True)
    assert np.array_equal(whole, parallel.exact_limbs_from_values(r.hist))
    assert np.array_equal(parallel.merge_exact([h1, h0]), whole)
    rounded = mc.exact_round(whole)
    assert same_bits(rounded, parallel.round_exact(whole))
    for b in range(r.hist.shape[1]):
        assert rounded[b, 0] == math.fsum(r.hist[:, b])
    assert np.allclose(rounded[:, 0], s_run, rtol=1e-13, atol=1e-300)
    # plain FP64's tree fold rounds differently from its exact sums, by rounding only
    assert np.allclose(mc.exact_round(plain)[:, 0], plain_run, rtol=1e-13, atol=1e-300)
