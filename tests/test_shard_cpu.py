"""Family sharding over ranks, without a GPU: the shard ranges, the
deterministic cross-rank combination of -lnL, and a world_size-2 gloo run
in which each rank scores its shard (with the CPU oracle standing in for a
GPU) and both ranks end up with the single-process total."""
import math
import os
import socket

import numpy as np
import pytest

from cafe5_gb300.shard import combine_totals, neumaier_sum, shard_range


def test_shard_ranges_cover_every_family_once():
    for n in (0, 1, 7, 1000, 10001):
        for world in (1, 2, 3, 8):
            ranges = [shard_range(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            for (a, b), (c, d) in zip(ranges, ranges[1:]):
                assert b == c
            sizes = [b - a for a, b in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def test_combine_totals_rules():
    assert combine_totals([[1.0, 2.0], [3.0, 4.0]]) == [4.0, 6.0]
    assert combine_totals([[1.0], [math.inf]]) == [math.inf]
    assert math.isnan(combine_totals([[math.inf], [math.nan]])[0])
    # compensated: the large-cancellation case a plain sum loses
    assert neumaier_sum([1e16, 1.0, -1e16]) == 1.0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        from cafe5_gb300.families import global_bounds
        from cafe5_gb300.inputs import RootPrior
        from cafe5_gb300.shard import allgather_totals, shard_range
        from cafe5_gb300.synth import workload
        w = workload(0, n_families=240, seed=41)
        S, R = global_bounds(w.families)
        prior = RootPrior.uniform(R).vector()
        ta = oracle.TreeArrays.from_tree(w.tree)
        lo, hi = shard_range(w.families.n_families, rank, world)
        totals = []
        for lam in (0.002, 0.003, -0.001):
            tot, _, _ = oracle.score(ta, w.families.counts[lo:hi], [lam], prior=prior, S=S, R=R, dedupe=False)
            totals.append(tot)
        q.put((rank, allgather_totals(totals)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_the_single_process_total():
    import multiprocessing as mp
    import oracle
    from cafe5_gb300.families import global_bounds
    from cafe5_gb300.inputs import RootPrior
    from cafe5_gb300.synth import workload
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got[0] == got[1]                       # every rank holds the same totals
    w = workload(0, n_families=240, seed=41)
    S, R = global_bounds(w.families)
    prior = RootPrior.uniform(R).vector()
    ta = oracle.TreeArrays.from_tree(w.tree)
    for lam, t in zip((0.002, 0.003), got[0][:2]):
        ref, _, _ = oracle.score(ta, w.families.counts, [lam], prior=prior, S=S, R=R, dedupe=False)
        assert abs(t - ref) <= 1e-12 * abs(ref)
    assert got[0][2] == math.inf                  # lambda <= 0: rejected on every rank
