"""Multi-GPU ensembles: runs shard across ranks, accumulators merge once.

Newman-Ziff runs are independent, so N ranks (one GPU each) take disjoint,
contiguous ranges of run ids and no data moves between them while they run
(weak scaling).  At the end each rank's running (number_of_runs, mean, M2)
state -- the reference's canonical_averages rows (percolate/hpc.py:518-558)
-- is gathered and merged with the associative, commutative pairwise
reduction of percolate/hpc.py:638-702 (``bond_reduce``), as the reference's
jug workflow merges its task results (percolate/share/jugfile.py:240-244).
"""
import functools

import numpy as np


def shard_runs(total_runs, world_size, rank):
    """(first run id, number of runs) of `rank`: contiguous, disjoint, covering
    range(total_runs), sizes differing by at most one."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError('invalid rank / world size')
    base, extra = divmod(int(total_runs), int(world_size))
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def gather_rows(rows, group=None):
    """All-gather one structured array per rank (any backend: gloo, nccl)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    out = [None] * world
    dist.all_gather_object(out, np.ascontiguousarray(rows), group=group)
    return out


def merge_rows(rows_per_rank, reducer=None):
    """Pairwise merge of per-rank canonical-averages arrays.  `reducer`
    defaults to the GPU bond_reduce of this package."""
    if reducer is None:
        from .hpc import bond_reduce as reducer
    parts = [r for r in rows_per_rank if r is not None and np.all(r['number_of_runs'] > 0)]
    if not parts:
        raise ValueError('no rank contributed runs')
    return functools.reduce(reducer, parts)


def merged_canonical_averages(ensemble, group=None, reducer=None):
    """Canonical averages of all ranks' runs, available on every rank."""
    return merge_rows(gather_rows(ensemble.canonical_averages(), group), reducer)
