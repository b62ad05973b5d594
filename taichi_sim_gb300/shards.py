"""Shots across GPUs: the only multi-GPU pattern this path has.

Shots (emission laws, full-matrix-capture firings, phantoms) are independent
simulations, so N GPUs run disjoint sets of them with no exchange during
stepping ("replicas"); a single grid fits one GB300.  The one collective is
the sum of per-cell gradients over shots after an adjoint pass (one
all-reduce of three grids).  One process per GPU, ranks from the usual
``torch.distributed`` environment (RANK, WORLD_SIZE, LOCAL_RANK, MASTER_*).
"""
import torch
import torch.distributed as dist


def world():
    """(rank, world size) of the initialised process group, or (0, 1)."""
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(), dist.get_world_size()
    return 0, 1


def shot_shard(n_shots, rank=None, size=None):
    """The contiguous, balanced share of ``range(n_shots)`` of a rank (the
    first ``n_shots % size`` ranks take one more)."""
    if rank is None or size is None:
        rank, size = world()
    if not 0 <= rank < size:
        raise ValueError("rank outside the world")
    base, extra = divmod(int(n_shots), size)
    start = rank * base + min(rank, extra)
    return list(range(start, start + base + (1 if rank < extra else 0)))


def weighted_shard(costs, rank=None, size=None):
    """Indices of ``costs`` (e.g. cells x shots of each phantom) for a rank:
    greedy longest-first assignment to the least loaded rank, deterministic
    on every rank."""
    if rank is None or size is None:
        rank, size = world()
    load = [0.0] * size
    owner = {}
    for i in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        r = min(range(size), key=lambda r: (load[r], r))
        owner[i] = r
        load[r] += costs[i]
    return sorted(i for i, r in owner.items() if r == rank)


def reduce_gradients(tensors):
    """Sum each tensor over all ranks in place (gradients of the shots each
    rank ran); a no-op on one rank."""
    _, size = world()
    if size > 1:
        for t in tensors:
            dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return tensors


def max_over_ranks(value, device=None):
    """The maximum of a float over all ranks (the job's time is its slowest
    rank's)."""
    _, size = world()
    if size == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
