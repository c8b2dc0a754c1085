"""Failure detection and checkpoint / resume on the GPU, as status codes and
files, without faulting the GPU.

* An event cap of one (mc_tune.max_events) makes every particle exceed its
  event budget: each engine stops with MC_ERR_TIMEOUT, reports it as a
  status, and the handle keeps working.
* mc_state_save / mc_state_load carry the tallies of [0, a) into another
  handle that runs [a, n): the result equals one run of [0, n) bit for bit in
  FP64 replay.  A state of another problem is refused."""
import os
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


@pytest.mark.parametrize("mode,kw", [("replay", {}), ("plain", {}), ("event", {"kernel": 1}),
                                     ("event", {"kernel": 2}), ("event", {"kernel": 3})])
def test_event_cap_reports_a_timeout(mc, mode, kw):
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("ce_sphere_small", d)
        p = mc.Problem(d, d + "/xs_library")
        with pytest.raises(mc.McError) as e:
            p.run(n=2000, mode=mode, max_events=1, **kw)
        assert e.value.status == 5          # MC_ERR_TIMEOUT
        p.reset()
        c = p.run(n=500, mode=mode, **kw)    # the handle stays usable
        assert c["histories"] == 500
        p.close()


def test_checkpoint_resume_is_bit_exact_in_replay(mc):
    with tempfile.TemporaryDirectory() as d:
        cases.write_case("slab_features", d)
        xs = d + "/xs_library"
        one = mc.Problem(d, xs)
        one.run(mode="replay")
        ref = one.all_tallies()
        n = one.nsample
        one.close()
        a = mc.Problem(d, xs)
        a.run(n=157, mode="replay")
        state = os.path.join(d, "state.bin")
        a.save_state(state)
        a.close()
        b = mc.Problem(d, xs)
        b.load_state(state)
        assert b.histories_run() == 157
        b.run(n=n - 157, first=157, mode="replay")
        got = b.all_tallies()
        assert b.histories_run() == n
        b.close()
        other = os.path.join(d, "other")
        cases.write_case("quadrics", other)
        c = mc.Problem(other, other + "/xs_library")
        with pytest.raises(mc.McError) as e:
            c.load_state(state)
        assert e.value.status == 1          # MC_ERR_INPUT: not this problem's state
        c.close()
    for x, y in zip(ref, got):
        assert same_bits(x, y)


def test_event_cap_in_a_batch_is_a_status_and_the_batch_recovers(mc):
    """The batch launch reports an exceeded event budget as MC_ERR_TIMEOUT;
    the next run (a new graph with the default budget) completes."""
    import mcgpu.workloads as W
    with tempfile.TemporaryDirectory() as root:
        specs = W.batch_shields(root, n_problems=8, min_hist=1000, max_hist=3000)
        probs = [mc.Problem(d) for d, _ in specs]
        hist = [h for _, h in specs]
        b = mc.Batch(probs, hist)
        with pytest.raises(mc.McError) as e:
            b.run(seed=9, max_events=1)
        assert e.value.status == 5          # MC_ERR_TIMEOUT
        for p in probs:
            p.reset()
        c = b.run(seed=9)
        assert c["histories"] == sum(hist)
        b.close()
        for p in probs:
            p.close()
