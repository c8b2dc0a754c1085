"""Sharding of histories over two ranks (gloo, CPU): each rank runs its
disjoint range, the merged (sum, sum of squares) equals the rank-order sum
of the two halves bit for bit and the single-process run to rounding.  The
transport here is the CPU oracle; the GPU ranks of bench.py use the same
sharding and merge."""
import os
import socket
import tempfile

import numpy as np
import pytest
import torch.multiprocessing as tmp_mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, d, n_total, out_dir):
    import sys
    root = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
    sys.path[:0] = [root, os.path.join(root, "mc-old_gb300")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    from mcgpu import parallel
    from oracle import problem as OP
    dist.init_process_group("gloo", rank=rank, world_size=world)
    first, n = parallel.shard_range(n_total, world, rank)
    r = OP.run(OP.load(d, xs_dir=d + "/xs_library"), n=n, first=first)
    s, q = parallel.gather_sums(r.sum, r.sq, dist)
    np.save(os.path.join(out_dir, f"part{rank}.npy"), np.stack([r.sum, r.sq]))
    if rank == 0:
        np.save(os.path.join(out_dir, "merged.npy"), np.stack([s, q]))
    dist.barrier()
    dist.destroy_process_group()


def _worker_exact(rank, world, port, d, n_total, out_dir):
    import sys
    root = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
    sys.path[:0] = [root, os.path.join(root, "mc-old_gb300")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    from mcgpu import parallel
    from oracle import problem as OP
    dist.init_process_group("gloo", rank=rank, world_size=world)
    first, n = parallel.shard_range(n_total, world, rank)
    r = OP.run(OP.load(d, xs_dir=d + "/xs_library"), n=n, first=first, hist=True)
    mine = parallel.exact_limbs_from_values(r.hist)
    merged = parallel.gather_exact(mine, dist)
    np.save(os.path.join(out_dir, f"exact{rank}.npy"), merged)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_exact_merge_is_bit_exact(oracle_lib):
    """The replay-exact merge: each rank sums its histories exactly
    (integers in units of 2^-1074), the ranks' sums are added limb by limb;
    every rank ends with the exact sums of the single run over all the
    histories, and their rounding equals math.fsum of all the histories'
    totals -- bit for bit, whatever the split."""
    import math
    import cases
    OP = oracle_lib
    from mcgpu import parallel
    with tempfile.TemporaryDirectory() as d, tempfile.TemporaryDirectory() as out:
        cases.write_case("slab_features", d)
        n = 300
        tmp_mp.spawn(_worker_exact, args=(2, _free_port(), d, n, out), nprocs=2, join=True)
        e0 = np.load(os.path.join(out, "exact0.npy"))
        e1 = np.load(os.path.join(out, "exact1.npy"))
        whole = OP.run(OP.load(d, xs_dir=d + "/xs_library"), n=n, hist=True)
    single = parallel.exact_limbs_from_values(whole.hist)
    assert np.array_equal(e0, single) and np.array_equal(e1, single)
    r = parallel.round_exact(e0)
    for b in range(whole.hist.shape[1]):
        assert r[b, 0] == math.fsum(whole.hist[:, b])
    # the running FP64 sums of the single run differ from the exact ones by rounding only
    assert np.allclose(r[:, 0], whole.sum, rtol=1e-13, atol=1e-300)


def test_shard_ranges_cover_exactly():
    from mcgpu import parallel
    for n in (0, 1, 7, 1000, 10_000_001):
        for w in (1, 2, 3, 8):
            spans = [parallel.shard_range(n, w, r, first=5) for r in range(w)]
            assert sum(k for _, k in spans) == n
            pos = 5
            for f, k in spans:
                assert f == pos
                pos += k


def test_two_rank_merge_matches_single_run(oracle_lib):
    import cases
    OP = oracle_lib
    with tempfile.TemporaryDirectory() as d, tempfile.TemporaryDirectory() as out:
        cases.write_case("slab_features", d)
        n = 300
        tmp_mp.spawn(_worker, args=(2, _free_port(), d, n, out), nprocs=2, join=True)
        merged = np.load(os.path.join(out, "merged.npy"))
        p0 = np.load(os.path.join(out, "part0.npy"))
        p1 = np.load(os.path.join(out, "part1.npy"))
        whole = OP.run(OP.load(d, xs_dir=d + "/xs_library"), n=n)
    assert np.array_equal(merged[0], p0[0] + p1[0]) and np.array_equal(merged[1], p0[1] + p1[1])
    assert np.allclose(merged[0], whole.sum, rtol=1e-12, atol=1e-300)
    assert np.allclose(merged[1], whole.sq, rtol=1e-12, atol=1e-300)
