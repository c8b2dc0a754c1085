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
