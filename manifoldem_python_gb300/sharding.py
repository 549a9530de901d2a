"""Multi-GPU distribution of projection directions: one process per GPU, no collective on the
data path (PDs are independent, as in the reference's MPI scatter, GetDistancesS2_mpi.py:58-65).

Each rank takes a static share of the PDs chosen by longest-processing-time-first on an estimated
cost, runs them through its own plan, and writes its own pickles; ranks only agree on timing /
metrics through small host-side reductions."""
from __future__ import annotations

import heapq
import math
from typing import List, Sequence


def pd_cost(n: int, N: int) -> float:
    """Estimated device time of one PD: the contraction n^2 K plus the prologue n N^2 log N^2."""
    K = 4 * N * (N // 2 + 1)
    return float(n) * n * K + float(n) * N * N * 2 * math.log2(max(N, 2)) * 40.0


def lpt_partition(costs: Sequence[float], world: int) -> List[List[int]]:
    """Assign items to `world` bins, largest first onto the least-loaded bin (ties: lower rank).
    Each bin keeps its items in ascending index order."""
    if world < 1:
        raise ValueError('world must be >= 1')
    heap = [(0.0, r) for r in range(world)]
    bins: List[List[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        load, r = heapq.heappop(heap)
        bins[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(b) for b in bins]


def shard(counts: Sequence[int], N: int, rank: int, world: int) -> List[int]:
    """PD indices of `rank`."""
    return lpt_partition([pd_cost(int(n), N) for n in counts], world)[rank]


def max_over_ranks(value: float) -> float:
    """Max of a host scalar over the initialised torch.distributed group (identity if none)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    dev = 'cuda' if dist.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
