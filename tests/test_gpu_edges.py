"""Edge cases of the history loop on the GPU: no histories, one history,
history indices above 2^32 (the upper key word), and problems with more
tally bins than the per-CTA shared sums and the register mask hold."""
import tempfile

import numpy as np
import pytest

import cases
from helpers import same_bits
from stats import assert_agree

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mc():
    import build as B
    B.build()
    import mcgpu
    return mcgpu


@pytest.mark.parametrize("mode", ["replay", "plain", "event"])
def test_zero_histories_leave_the_tallies_alone(mc, mode):
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("slab_features", d)
        p = mc.Problem(d, d + "/xs_library")
        p.run(n=300, mode=mode)
        before = [a.copy() for a in p.all_tallies()[2:]]
        c = p.run(n=0, first=300, mode=mode)
        after = p.all_tallies()[2:]
        assert c["histories"] == 0 and c["flights"] == 0
        assert p.histories_run() == 300
        for a, b in zip(before, after):
            assert same_bits(a, b)
        p.close()


@pytest.mark.parametrize("mode", ["replay", "event"])
def test_single_history(mc, mode):
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("ce_sphere_small", d)
        p = mc.Problem(d, d + "/xs_library")
        c = p.run(n=1, first=12345, mode=mode)
        _, _, s, q = p.all_tallies()
        p.close()
    assert c["histories"] == 1 and c["particles"] >= 1 and c["flights"] >= 1
    assert np.all(np.isfinite(s)) and np.all(q >= 0)
    assert same_bits(q, s * s)   # one history: the sum of squares is the square


def test_history_indices_above_2_32_replay_bit_exact(mc):
    """The history index enters the Philox key's upper word above 2^32; the
    GPU replay and the oracle agree there too."""
    from oracle import problem as OP
    first = (1 << 40) + 7
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("slab_features", d)
        p = mc.Problem(d, d + "/xs_library")
        p.run(n=200, first=first, mode="replay", record_digests=1)
        _, _, s, q = p.all_tallies()
        dg = p.digests(200)
        r = OP.run(OP.load(d, xs_dir=d + "/xs_library"), n=200, first=first, digests=True)
        p.close()
    assert np.array_equal(dg, r.digest)
    assert same_bits(s, r.sum) and same_bits(q, r.sq)


@pytest.mark.parametrize("kernel", [1, 2])
def test_many_bins_use_global_sums_and_memory_masks(mc, kernel):
    """4200 flux bins: more than the per-CTA shared sums (4096) and the
    register mask (64) hold, so histories fold into the global sums through
    the row masks in memory; results agree with FP64 replay."""
    import mcgpu.workloads as W
    with tempfile.TemporaryDirectory() as d:
        W.slab_1g(d, samples=100, n_flux_bins=4200)
        p = mc.Problem(d, d + "/xs_library")
        assert sum(p.sizes) > 4096
        p.run(n=200_000, mode="event", kernel=kernel)
        m1, s1, _, _ = p.all_tallies()
        p.reset()
        p.run(n=50_000, mode="replay")
        m2, s2, _, _ = p.all_tallies()
        p.close()
    # compare well-resolved bins; one flight crosses hundreds of these thin
    # bins, so neighbouring bins are strongly correlated and a chi-square over
    # all of them would not follow its distribution: take every 40th
    ok = (s1 > 0) & (s2 > 0) & (s1 < 0.1 * np.abs(m1)) & (s2 < 0.1 * np.abs(m2))
    idx = np.nonzero(ok)[0][::40]
    assert idx.size > 20
    assert_agree(m1[idx], s1[idx], m2[idx], s2[idx], f"4200-bin slab, kernel {kernel}")
