"""Family sharding across GPUs (one process per GPU).

Gene families are independent in every likelihood the reference computes
(base_model::infer_family_likelihoods, src/base_model.cpp:53-100, and the
gamma model, src/gamma_core.cpp:168-237, both sum independent per-family
terms), so N ranks each score a contiguous family range with their own
device-resident copy of the tree, prior and matrix cache (matrices are
rebuilt per GPU rather than exchanged). The only exchange is the per-rank
partial -lnL of each candidate, combined here in rank order with the same
compensated (Neumaier) sum the device uses within a GPU, so every rank holds
the identical total. Rejections keep the reference's meaning: a rank that
reports +inf (a family failed, a lambda was rejected) makes the total +inf.
"""
from __future__ import annotations

import math
from typing import List, Sequence, Tuple

import numpy as np


def shard_range(n_families: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous [start, stop) of `rank`: the first n % world ranks take one
    family more, so shard sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world {world}")
    base, extra = divmod(int(n_families), world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def neumaier_sum(values: Sequence[float]) -> float:
    s, c = 0.0, 0.0
    for x in values:
        t = s + x
        if abs(s) >= abs(x):
            c += (s - t) + x
        else:
            c += (x - t) + s
        s = t
    return s + c


def combine_totals(per_rank: Sequence[Sequence[float]]) -> List[float]:
    """-lnL of each candidate from the ranks' partial totals (rank order).
    +inf wins over finite values; NaN (a rank's bounded wait gave up)
    wins over everything."""
    n_cand = len(per_rank[0]) if per_rank else 0
    out = []
    for b in range(n_cand):
        col = [float(r[b]) for r in per_rank]
        if any(math.isnan(x) for x in col):
            out.append(math.nan)
        elif any(math.isinf(x) for x in col):
            out.append(math.inf)
        else:
            out.append(neumaier_sum(col))
    return out


def allgather_totals(totals: Sequence[float], group=None) -> List[float]:
    """Combine this rank's partial totals with every other rank's through
    torch.distributed (gloo on CPU, NCCL on GPUs: 8 bytes per candidate)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    mine = torch.tensor(list(totals), dtype=torch.float64, device=dev)
    parts = [torch.empty_like(mine) for _ in range(world)]
    dist.all_gather(parts, mine, group=group)
    return combine_totals([p.cpu().numpy().tolist() for p in parts])


class ShardedModel:
    """A family set split over the ranks of the default process group: each
    rank uploads only its shard to its own GPU context and scores it; the
    candidates' totals are combined across ranks. Per-family lnL stay on
    their rank (`family_range` says which)."""

    def __init__(self, ctx, tree, counts: np.ndarray, rank: int, world: int, lambda_of_node=None):
        self.ctx = ctx
        self.rank, self.world = rank, world
        self.family_range = shard_range(counts.shape[0], rank, world)
        lo, hi = self.family_range
        self.tree_id = ctx.upload_tree(tree, lambda_of_node)
        self.set_id = ctx.upload_families(self.tree_id, np.ascontiguousarray(counts[lo:hi]))

    def score_batch(self, candidates, group=None, **kw):
        """Per-candidate (total -lnL over all ranks, this rank's ScoreResult)."""
        local = self.ctx.score_batch(self.tree_id, self.set_id, candidates, **kw)
        totals = allgather_totals([r.total for r in local], group)
        return totals, local
