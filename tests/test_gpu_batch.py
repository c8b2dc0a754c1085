"""Batches of independent problems in one persistent launch (CUDA graph) and
the launch-shape autotuners."""
import tempfile

import numpy as np
import pytest

from stats import assert_agree

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mc():
    import build as B
    B.build()
    import mcgpu
    return mcgpu


def _problems(mc, root, n, lo=2000, hi=20000):
    import mcgpu.workloads as W
    specs = W.batch_shields(root, n_problems=n, min_hist=lo, max_hist=hi)
    return [mc.Problem(d) for d, _ in specs], [h for _, h in specs]


@pytest.mark.parametrize("kernel", [1, 2])
def test_batch_equals_problems_run_alone(mc, kernel):
    """Problem i of a batch follows the histories of a lone run with seed
    batch_problem_seed(seed, i): same answers (summation order aside), with
    either event kernel in the batch."""
    seed = 777
    with tempfile.TemporaryDirectory() as root:
        probs, hist = _problems(mc, root, 24)
        b = mc.Batch(probs, hist)
        c = b.run(seed=seed, kernel=kernel)
        assert c["histories"] == sum(hist)
        assert c["launches"] == 2   # the transport kernel and the fold of the replicated sums
        batch_res = [p.all_tallies() for p in probs]
        for i, p in enumerate(probs):
            assert p.histories_run() == hist[i]
        b.close()
        for i, (d_p, n) in enumerate(zip(probs, hist)):
            d_p.reset()
            d_p.run(n=n, seed=mc.batch_problem_seed(seed, i), mode="event")
            m1, s1, su1, _ = batch_res[i]
            m2, s2, su2, _ = d_p.all_tallies()
            assert np.allclose(su1, su2, rtol=1e-6, atol=1e-12), f"problem {i}"
            assert_agree(m1, s1, m2, s2, f"problem {i}")
        for p in probs:
            p.close()


def test_batch_agrees_with_fp64(mc):
    with tempfile.TemporaryDirectory() as root:
        probs, hist = _problems(mc, root, 16)
        b = mc.Batch(probs, hist)
        b.run(seed=5)
        ev = [p.all_tallies() for p in probs]
        b.close()
        for i, p in enumerate(probs):
            p.reset()
            p.run(n=hist[i], seed=99, mode="replay")
            m2, s2, _, _ = p.all_tallies()
            assert_agree(ev[i][0], ev[i][1], m2, s2, f"problem {i}")
            p.close()


def test_batch_graph_replays_with_new_seeds(mc):
    with tempfile.TemporaryDirectory() as root:
        probs, hist = _problems(mc, root, 12)
        b = mc.Batch(probs, hist)
        b.run(seed=1)
        first = [p.all_tallies()[2].copy() for p in probs]
        for p in probs:
            p.reset()
        b.run(seed=2)                 # replays the captured graph
        second = [p.all_tallies()[2].copy() for p in probs]
        for p in probs:
            p.reset()
        b.run(seed=1)
        again = [p.all_tallies()[2].copy() for p in probs]
        b.close()
        assert any(not np.allclose(a, c) for a, c in zip(first, second))
        for a, c in zip(first, again):
            assert np.allclose(a, c, rtol=1e-9, atol=1e-12)
        for p in probs:
            p.close()


def test_autotune_single_and_batch(mc):
    import cases
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("ce_sphere_small", d)
        p = mc.Problem(d, d + "/xs_library")
        p.run(n=1000, mode="event")
        before = p.all_tallies()[2].copy()
        t = p.autotune(sample=20000)
        assert t["kernel"] in (1, 2) and t["blocks_per_sm"] in ((2, 3, 4) if t["kernel"] == 1 else (4, 6, 7, 8))
        assert t["kernel"] == 2 or t["bank_capacity"] in (256, 512, 1024, 2048)
        assert t["kernel"] == 1 or t["refill"] in (0, 2, 4, 8, 16)
        assert np.array_equal(p.all_tallies()[2], before)       # tallies untouched
        assert p.histories_run() == 1000
        p.run(n=1000, first=1000, mode="event")                 # uses the tuned shape
        assert p.histories_run() == 2000
        p.close()
    with tempfile.TemporaryDirectory() as root:
        probs, hist = _problems(mc, root, 8)
        b = mc.Batch(probs, hist)
        t = b.autotune(fraction=0.05)
        assert t["kernel"] in (1, 2)
        assert t["refill"] == 0
        assert all(p.histories_run() == 0 for p in probs)
        b.run(seed=3)
        assert all(p.histories_run() == h for p, h in zip(probs, hist))
        b.close()
        for p in probs:
            p.close()


def test_batch_wide_upload_reset_and_read(mc):
    """mc_batch_upload / mc_batch_reset / mc_batch_tally_read do for every
    problem what the per-problem calls do, with one wait each: the batch's
    read-back equals every problem's own mc_tally_read bit for bit, a reset
    zeroes every problem, and after a batch upload the same seed gives the
    same tallies again."""
    with tempfile.TemporaryDirectory() as root:
        probs, hist = _problems(mc, root, 16)
        b = mc.Batch(probs, hist)
        b.run(seed=5)
        got = b.tallies()
        want = [np.concatenate([p.all_tallies()[k] for p in probs]) for k in range(4)]
        for g, w in zip(got, want):
            assert g.shape == w.shape and np.array_equal(g.view(np.uint64), w.view(np.uint64))
        b.reset()
        assert all(p.histories_run() == 0 for p in probs)
        assert not np.any(b.tallies()[2]) and not np.any(b.tallies()[3])
        b.upload()
        b.run(seed=5)
        again = b.tallies()
        assert all(p.histories_run() == h for p, h in zip(probs, hist))
        assert np.allclose(again[2], got[2], rtol=1e-12, atol=1e-300)   # same histories; atomics' order aside
        b.close()
        for p in probs:
            p.close()


def test_batch_replicated_sums_equal_lone_runs(mc):
    """A batch folds histories into replicas of its sums (a copy per group
    of CTAs) and adds them into each problem's sums after the launch: a
    batch of a few problems of 2*10^5 histories each gives what lone runs
    give, and a second run adds to the first (the replicas were cleared)."""
    import mcgpu.workloads as W
    seed = 4242
    with tempfile.TemporaryDirectory() as root:
        specs = W.batch_shields(root, n_problems=3, min_hist=200000, max_hist=200001)
        probs = [mc.Problem(d) for d, _ in specs]
        hist = [h for _, h in specs]
        b = mc.Batch(probs, hist)
        b.run(seed=seed)
        first = [p.all_tallies() for p in probs]
        b.run(seed=seed + 1)
        second = [p.all_tallies() for p in probs]
        b.close()
        for i, p in enumerate(probs):
            assert p.histories_run() == 2 * hist[i]
            # the sums of the second run add to the first's
            assert np.all(second[i][2] >= first[i][2] - 1e-12)
            p.reset()
            p.run(n=hist[i], seed=mc.batch_problem_seed(seed, i), mode="event")
            m2, s2, su2, _ = p.all_tallies()
            assert np.allclose(first[i][2], su2, rtol=1e-6, atol=1e-12), f"problem {i}"
            assert_agree(first[i][0], first[i][1], m2, s2, f"problem {i}")
        for p in probs:
            p.close()
