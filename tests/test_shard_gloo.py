"""The N>1 path on the CPU: two gloo ranks each compute their contiguous
share of a pair batch (with the oracle), gather to rank 0, and the result
equals the single-process answer; the timing reduction is a max."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from distance3d_gb300.shard import concat_results, shard_range


def test_shard_range_partitions():
    for n in (0, 1, 7, 1000, 1001):
        for world in (1, 2, 3, 8):
            ranges = [shard_range(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(ranges[k][1] == ranges[k + 1][0] for k in range(world - 1))
            sizes = [hi - lo for lo, hi in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, queue):
    import torch.distributed as dist
    from distance3d_gb300 import workloads
    from distance3d_gb300.shard import gather_results, max_over_ranks
    from oracle import oracle
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cs, i1, i2 = workloads.pairs_mixed_six(301, seed=9, center_half_width=workloads.INTERSECT30_HALF_WIDTH)
        lo, hi = shard_range(len(i1), rank, world)
        r = oracle.gjk_distance(cs, np.asarray(i1[lo:hi]), np.asarray(i2[lo:hi]))
        part = {k: r[k] for k in ("dist", "cp1", "cp2", "n_simplex", "status")}
        full = gather_results(part)
        slowest = max_over_ranks(10.0 + rank)
        if rank == 0:
            queue.put((full, slowest))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_match_single_process():
    from distance3d_gb300 import workloads
    from oracle import oracle
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    full, slowest = q.get()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    cs, i1, i2 = workloads.pairs_mixed_six(301, seed=9, center_half_width=workloads.INTERSECT30_HALF_WIDTH)
    want = oracle.gjk_distance(cs, np.asarray(i1), np.asarray(i2))
    for k in full:
        assert np.array_equal(full[k], want[k], equal_nan=True), k
    assert slowest == 11.0
    assert concat_results([None]) == {}
