"""Mixed-precision event engine against FP64 replay and the CPU oracle.

Production mode tracks in FP32 and crosses surfaces without the reference's
FLT_EPSILON nudge, so it is compared statistically: every tally bin within
combined 3 sigma of the FP64 result (allowing the 2 % of bins a fair test
misses) and the chi-square over bins consistent with zero difference.  The
FP64 replay it is compared with is itself bit-identical to the CPU oracle."""
import tempfile

import numpy as np
import pytest

import cases
from stats import assert_agree

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mc():
    import build as B
    B.build()
    import mcgpu
    return mcgpu


def _run(mc, d, n, mode, xs=True, **kw):
    p = mc.Problem(d, d + "/xs_library" if xs else None)
    c = p.run(n=n, mode=mode, **kw)
    m, s, _, _ = p.all_tallies()
    p.close()
    return m, s, c


CASES = {
    "ce_sphere_small": (lambda d: cases.write_case("ce_sphere_small", d), 20000),
    "slab_features": (lambda d: cases.write_case("slab_features", d), 20000),
    "quadrics": (lambda d: cases.write_case("quadrics", d), 20000),
    "absorber_slab": (lambda d: cases.write_case("absorber_slab", d), 200000),
}


@pytest.mark.parametrize("kernel", [1, 2, 3])
@pytest.mark.parametrize("name", list(CASES))
def test_event_agrees_with_fp64(mc, name, kernel):
    writer, n = CASES[name]
    with tempfile.TemporaryDirectory() as d:
        writer(d)
        m1, s1, c1 = _run(mc, d, n, "event", kernel=kernel)
        m2, s2, c2 = _run(mc, d, n, "replay")
    assert c1["histories"] == n
    assert_agree(m1, s1, m2, s2, name)
    # event counts agree to a few percent (same physics, different streams)
    assert abs(c1["flights"] / c2["flights"] - 1) < 0.05


def test_event_agrees_with_cpu_oracle(mc):
    from oracle import problem as OP
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("ce_sphere_small", d)
        m1, s1, _ = _run(mc, d, 3000, "event")
        r = OP.run(OP.load(d, xs_dir=d + "/xs_library"), n=3000)
        m2, s2 = r.finalize()
    assert_agree(m1, s1, m2, s2, "event vs CPU oracle")


def _ext():
    import mcgpu.workloads as W
    return {
        "slab_1g": (lambda d: W.slab_1g(d, samples=100, n_flux_bins=20), 100000),
        "mg_deep_slab": (lambda d: W.mg_deep_slab(d, samples=100, G=8), 100000),
        "mg_layered_slab": (lambda d: W.mg_layered_slab(d, samples=100), 100000),
    }


@pytest.mark.parametrize("kernel", [1, 2, 3])
@pytest.mark.parametrize("name", ["slab_1g", "mg_deep_slab", "mg_layered_slab"])
def test_event_agrees_with_fp64_extensions(mc, name, kernel):
    writer, n = _ext()[name]
    with tempfile.TemporaryDirectory() as d:
        writer(d)
        m1, s1, c1 = _run(mc, d, n, "event", kernel=kernel)
        m2, s2, c2 = _run(mc, d, n, "replay")
    assert_agree(m1, s1, m2, s2, name)


@pytest.mark.parametrize("name", ["slab_features", "ce_sphere_small", "quadrics", "mg_layered_slab",
                                  "mg_deep_slab"])
def test_per_thread_kernel_follows_the_same_histories(mc, name):
    """The per-thread kernel (k_track) and the event-split engine (k_bank_*
    over the HBM bank) run the tile kernel's event functions with the same
    Philox keying, so every particle follows the same track: event counts
    are equal, and the tally sums differ only by the order of FP64
    additions and the last-bit rounding of FP32 scores (the kernels are
    compiled separately and may fuse multiply-adds differently).  The deep
    slab adds importance splitting (split copies through each engine's own
    store: overflow bank, thread stack, HBM split stack)."""
    with tempfile.TemporaryDirectory() as d:
        if name == "mg_layered_slab":
            import mcgpu.workloads as W
            W.mg_layered_slab(d, samples=100)
            xs = None
        elif name == "mg_deep_slab":
            import mcgpu.workloads as W
            W.mg_deep_slab(d, samples=100, G=8)
            xs = None
        else:
            cases.write_case(name, d)
            xs = d + "/xs_library"
        out = []
        for kernel in (1, 2, 3):
            p = mc.Problem(d, xs)
            c = p.run(n=20000, mode="event", kernel=kernel)
            out.append((p.all_tallies()[2].copy(), c))
            p.close()
    (s1, c1) = out[0]
    for s2, c2 in out[1:]:
        for k in ("flights", "collisions", "crossings", "tally_updates", "particles", "splits", "freegas_iters",
                  "xs_evals", "nuc_lookups", "histories"):
            assert c1[k] == c2[k], (k, c1[k], c2[k])
        assert np.allclose(s1, s2, rtol=1e-6, atol=1e-14)


def test_event_tiles_and_grids(mc):
    """Other tile sizes and grid shapes give statistically equal answers and
    every history is run exactly once."""
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("slab_features", d)
        ref = _run(mc, d, 20000, "event")
        for tile, grid in ((256, 7), (1024, 0), (512, 1)):
            m, s, c = _run(mc, d, 20000, "event", kernel=1, bank_capacity=tile, grid_blocks=grid)
            assert c["histories"] == 20000
            assert_agree(m, s, ref[0], ref[1], f"tile {tile} grid {grid}")
        for minb, grid in ((4, 0), (6, 5), (8, 1)):
            m, s, c = _run(mc, d, 20000, "event", kernel=2, blocks_per_sm=minb, grid_blocks=grid)
            assert c["histories"] == 20000
            assert_agree(m, s, ref[0], ref[1], f"per-thread kernel, {minb} CTAs/SM, grid {grid}")
        # the event-split engine with a bank far smaller than the run (many
        # refills per slot, rows reused) and with a grid of one block
        for bank, grid in ((1024, 0), (4096, 1), (1 << 16, 0)):
            m, s, c = _run(mc, d, 20000, "event", kernel=3, bank_capacity=bank, grid_blocks=grid)
            assert c["histories"] == 20000 and c["particles"] == ref[2]["particles"]
            assert_agree(m, s, ref[0], ref[1], f"event-split engine, bank {bank}, grid {grid}")


def test_per_thread_stack_overflow_is_a_status(mc):
    """Split copies beyond the per-thread stack report MC_ERR_OVERFLOW and the
    handle stays usable."""
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("slab_features", d)
        p = mc.Problem(d, d + "/xs_library")
        with pytest.raises(mc.McError) as e:
            p.run(n=5000, mode="event", kernel=2, stack_depth=1)
        assert e.value.status == 3
        p.reset()
        c = p.run(n=500, mode="event", kernel=2)
        assert c["histories"] == 500
        p.close()


@pytest.mark.parametrize("kernel", [1, 3])
def test_event_overflow_is_a_status(mc, kernel):
    """The tile kernel's per-CTA overflow bank (kernel 1) or the event-split
    engine's split stack (kernel 3) shrunk to one slot, on a
    two-region slab whose importance rises 4x at the interface: every
    crossing into the second region makes three split copies at once, more
    than the slot holds, so the run stops with MC_ERR_OVERFLOW.  The handle
    then runs again with the default bank, every history once, in agreement
    with FP64 replay."""
    import mcgpu.workloads as W
    from stats import assert_agree
    with tempfile.TemporaryDirectory() as d:
        tot = np.array([[0.5], [0.5]])
        sca = np.array([[[0.25]], [[0.25]]])
        est = ("    <estimator name=\"transmitted\" scores=\"cross\">\n        <surface name=\"p@R\"/>\n"
               "    </estimator>\n    <estimator name=\"reflected\" scores=\"cross\">\n"
               "        <surface name=\"p0\"/>\n    </estimator>\n")
        W._mg_slab_xml(d, "split4", 100, [2.0, 2.0], tot, sca, [1.0, 4.0], est)
        p = mc.Problem(d)
        with pytest.raises(mc.McError) as e:
            p.run(n=20000, mode="event", kernel=kernel, stack_depth=1)
        assert e.value.status == 3
        assert "overflow" in str(e.value)
        p.reset()
        c = p.run(n=20000, mode="event", kernel=kernel)
        assert c["histories"] == 20000 and c["splits"] > 0
        m1, s1, _, _ = p.all_tallies()
        p.reset()
        p.run(n=20000, first=20000, mode="replay")
        m2, s2, _, _ = p.all_tallies()
        p.close()
    assert_agree(m1, s1, m2, s2, f"kernel {kernel} after an overflow vs FP64 replay")


def test_upload_recopies_the_mixed_engine_tables(mc):
    """mc_problem_upload copies the FP32 event tables again once the mixed
    engine has built them (the end-to-end timing moves them every step); the
    re-copied tables give the same tracks."""
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("ce_sphere_small", d)
        p = mc.Problem(d, d + "/xs_library")
        b0 = p.table_bytes()
        c1 = p.run(n=20000, mode="event", kernel=2)
        b1 = p.table_bytes()
        assert b1 > b0
        p.upload()
        p.reset()
        c2 = p.run(n=20000, mode="event", kernel=2)
        p.close()
    for k in ("flights", "collisions", "crossings", "tally_updates", "freegas_iters"):
        assert c1[k] == c2[k], k


@pytest.mark.parametrize("case", ["ce_sphere_small", "slab_features"])
def test_refill_threshold_keeps_every_track(mc, case):
    """mc_tune.refill only changes when a warp's idle lanes take new
    histories: every history keeps its own random stream, so the event
    counts are identical for any threshold, and every history runs once."""
    with tempfile.TemporaryDirectory() as d:
        cases.write_case(case, d)
        p = mc.Problem(d, d + "/xs_library")
        out = []
        for r in (1, 4, 32):
            p.reset()
            c = p.run(n=30000, mode="event", kernel=2, refill=r)
            out.append((c, p.all_tallies()[2]))
        with pytest.raises(mc.McError):
            p.run(n=10, mode="event", kernel=2, refill=33)
        p.close()
    (c0, s0) = out[0]
    for c, s in out[1:]:
        assert c["histories"] == 30000
        for k in ("flights", "collisions", "crossings", "tally_updates", "particles", "splits", "freegas_iters"):
            assert c[k] == c0[k], k
        assert np.allclose(s, s0, rtol=1e-9, atol=1e-14)


@pytest.mark.parametrize("name", ["ce_sphere_small", "slab_features", "quadrics", "absorber_slab", "comb_slab"])
def test_event_agrees_with_the_reference_run(mc, name):
    """The mixed mode against the compiled reference's own output for the
    same input (the golden fixtures: means and uncertainties the reference
    wrote), with the reference's history count and an independent random
    stream: every bin within combined 3 sigma, chi-square consistent."""
    from helpers import golden_arrays, load_golden
    g = load_golden(name)
    with tempfile.TemporaryDirectory() as d:
        cases.write_case(name, d)
        p = mc.Problem(d, d + "/xs_library")
        p.run(n=g["nsample"], seed=g["seed"] + 1000, mode="event")
        m, s, _, _ = p.all_tallies()
        p.close()
    gm, gu = golden_arrays(g)
    assert_agree(m, s, gm, gu, f"{name}: mixed mode vs the reference")


def test_many_bins_fold_through_replicated_sums(mc):
    """Beyond 4096 bins a problem's sums do not fit in shared memory: its
    histories fold into replicas of the sums, which a second kernel adds
    into the problem's sums and clears.  On a 5002-bin slab the tile and
    the per-thread kernels, which follow the same tracks, give the same
    sums up to summation order, a second run adds to the first, and the
    mixed mode agrees with FP64 replay: the reflected and transmitted
    currents within combined 3 sigma, and the flux and absorption in 2500
    cells of 0.008 mean free paths bin by bin (neighbouring bins are nearly
    the same quantity, so a chi-square over them, which assumes independent
    bins, does not apply; the fraction within 3 sigma does)."""
    from stats import compare
    import mcgpu.workloads as W
    n = 100000
    sums = {}
    with tempfile.TemporaryDirectory() as d:
        W.slab_1g(d, samples=10, n_flux_bins=2500)    # 2 x 2500 + 2 bins
        p = mc.Problem(d, d + "/xs_library")
        assert int(sum(p.sizes)) > 4096
        for kernel in (1, 2):
            p.reset()
            c = p.run(n=n, mode="event", kernel=kernel)
            assert c["launches"] == 2
            half = p.all_tallies()[2].copy()
            p.run(n=n, first=n, mode="event", kernel=kernel)
            assert p.histories_run() == 2 * n
            su1 = p.all_tallies()[2]
            assert np.all(su1 >= half - 1e-12) and su1.sum() > half.sum()
            sums[kernel] = su1
        ev = {k: p.tally(p.names.index(k))[:2] for k in ("transmission", "reflection", "slab")}
        p.reset()
        p.run(n=2 * n, first=10 * n, mode="replay")
        rp = {k: p.tally(p.names.index(k))[:2] for k in ("transmission", "reflection", "slab")}
        p.close()
    assert np.allclose(sums[1], sums[2], rtol=1e-9, atol=1e-300)
    for k in ("transmission", "reflection"):
        assert_agree(*ev[k], *rp[k], k)
    frac, _, _, _ = compare(*ev["slab"], *rp["slab"])
    assert frac >= 0.95, f"slab flux / absorption: {frac:.3f} of bins within 3 sigma"
