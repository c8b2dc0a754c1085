"""mc_run_replay_noalloc: the FP64 replay transport without device allocation.

Callers whose device memory is owned by another allocator, or that forbid
allocation once they are serving requests, load the problem at start-up and
then call this entry point, which keeps its scratch in a fixed 64 MiB
file-scope device array and writes the tally sums to buffers the caller
passes.  Its results must equal mc_run's FP64 replay bit for bit (replay is
exact), on two calls in a row -- the second call reuses the array the first
one left behind.

The file name makes pytest collect it last."""
import ctypes
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
    L = mcgpu.lib()
    L.mc_run_replay_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                        ctypes.c_void_p, ctypes.c_void_p]
    L.mc_run_replay_noalloc.restype = ctypes.c_int
    return mcgpu


@pytest.mark.parametrize("name", ["slab_features", "ce_sphere_small", "comb_slab"])
def test_noalloc_matches_mc_run_twice(mc, name):
    import torch
    L = mc.lib()
    with tempfile.TemporaryDirectory() as d:
        cases.write_case(name, d)
        p = mc.Problem(d, d + "/xs_library")
        n, first, seed = 700, 123, 0x4D43
        p.run(n=n, first=first, seed=seed, mode="replay")
        _, _, s_ref, q_ref = p.all_tallies()
        nb = int(sum(p.sizes))
        out_s = torch.full((nb,), 7.0, dtype=torch.float64, device="cuda")
        out_q = torch.full((nb,), 7.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for call in range(2):
            st = L.mc_run_replay_noalloc(p._h, first, n, seed, out_s.data_ptr(), out_q.data_ptr())
            assert st == 0, L.mc_last_error(p._h).decode()
            s = out_s.cpu().numpy()
            q = out_q.cpu().numpy()
            assert same_bits(s, s_ref), f"call {call + 1}: sums differ from mc_run"
            assert same_bits(q, q_ref), f"call {call + 1}: sums of squares differ from mc_run"
        p.close()


def test_noalloc_spans_several_chunks(mc):
    """A problem with ~5000 tally bins leaves room for ~1090 history rows in
    the fixed array, so 3000 histories run in three chunks: the chunk loop's
    reset of the history counter, the reuse of the rows and the ordered fold
    carrying the sums from one chunk to the next must still give mc_run's
    replay bit for bit, on two calls in a row."""
    import torch
    import mcgpu.workloads as W
    L = mc.lib()
    with tempfile.TemporaryDirectory() as d:
        W.slab_1g(d, samples=10, n_flux_bins=2500)    # 2 x 2500 + 2 bins
        p = mc.Problem(d, d + "/xs_library")
        nb = int(sum(p.sizes))
        assert nb > 5000
        n, first, seed = 3000, 77, 0x4D43 + 9
        p.run(n=n, first=first, seed=seed, mode="replay")
        _, _, s_ref, q_ref = p.all_tallies()
        out_s = torch.full((nb,), 3.0, dtype=torch.float64, device="cuda")
        out_q = torch.full((nb,), 3.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for call in range(2):
            st = L.mc_run_replay_noalloc(p._h, first, n, seed, out_s.data_ptr(), out_q.data_ptr())
            assert st == 0, L.mc_last_error(p._h).decode()
            assert same_bits(out_s.cpu().numpy(), s_ref), f"call {call + 1}: sums differ from mc_run"
            assert same_bits(out_q.cpu().numpy(), q_ref), f"call {call + 1}: squares differ from mc_run"
        assert p.counters()["histories"] == n
        p.close()


def test_noalloc_rejects_too_many_bins(mc):
    """A problem whose tally rows cannot fit the fixed scratch is refused
    with a message, not run."""
    import torch
    L = mc.lib()
    import mcgpu.workloads as W
    with tempfile.TemporaryDirectory() as d:
        W.slab_1g(d, samples=10, n_flux_bins=8000)
        p = mc.Problem(d, d + "/xs_library")
        nb = int(sum(p.sizes))
        out = torch.zeros(2 * nb, dtype=torch.float64, device="cuda")
        st = L.mc_run_replay_noalloc(p._h, 0, 10, 1, out.data_ptr(), out.data_ptr() + 8 * nb)
        assert st == 8
        assert "static scratch" in L.mc_last_error(p._h).decode()
        p.close()
