"""Multi-GPU ensembles: runs shard across ranks, accumulators merge once.

Newman-Ziff runs are independent, so N ranks (one GPU each) take disjoint,
contiguous ranges of run ids and no data moves between them while they run
(weak scaling).  At the end each rank's ensemble state -- the running
(number_of_runs, mean, M2) per (p, statistic), i.e. the reference's
canonical_averages rows (percolate/hpc.py:518-558), plus the exact
microcanonical accumulators -- is gathered and merged with the associative,
commutative pairwise reduction of percolate/hpc.py:638-702 (``bond_reduce``),
as the reference's jug workflow merges its task results
(percolate/share/jugfile.py:240-244).  The exchange is one gather of a few
hundred KB to a few tens of MB per rank, after all runs are done.

Two merges of gathered states, the same arithmetic:
  merged_ensemble  on the device, with the library's nz_canonical_merge /
                   nz_micro_merge kernels (Ensemble.merge), on every rank;
  merge_states     on the host (numpy), for a coordinating process that holds
                   the ranks' states without a GPU of its own (e.g. states
                   read back from checkpoint files).
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


def gather_objects(obj, group=None):
    """All-gather one picklable object per rank (any backend: gloo, nccl)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    out = [None] * world
    dist.all_gather_object(out, obj, group=group)
    return out


def gather_rows(rows, group=None):
    """All-gather one structured array per rank."""
    return gather_objects(np.ascontiguousarray(rows), group)


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


def merged_ensemble(ensemble, group=None):
    """An Ensemble holding every rank's runs, on every rank: the ranks'
    states are gathered and merged on this rank's GPU by Ensemble.merge
    (canonical (n, mean, M2) pairwise, exact microcanonical sums added).
    Raises ValueError if two ranks share a run."""
    from .ensemble import Ensemble
    states = gather_objects(ensemble.state(), group)
    out = Ensemble.from_state(states[0], window=ensemble.window)
    for st in states[1:]:
        out.merge(st)
    return out


# ------------------------------------------------------------ host merge
def _pairwise(na, ma, sa, nb, mb, sb):
    """(mean, M2) of two disjoint sets of runs, the update of
    percolate/hpc.py:674-692 in the operation order of the device kernels
    (chan_merge in nz_canonical.cu); an empty side leaves the other as is."""
    n = na + nb
    with np.errstate(invalid='ignore', divide='ignore'):
        d = mb - ma
        mean = ma + d * nb / n
        m2 = sa + (sb + d * d * na * nb / n)
    mean = np.where(nb == 0, ma, np.where(na == 0, mb, mean))
    m2 = np.where(nb == 0, sa, np.where(na == 0, sb, m2))
    return mean, m2


def _u128(lo, hi):
    """Exact 128-bit values (Python ints) from their two 64-bit halves."""
    return (np.asarray(lo).view(np.uint64).astype(object)
            + (np.asarray(hi).view(np.uint64).astype(object) << 64))


def _halves(x):
    """(low, high) 64-bit halves, as int64 views, of exact 128-bit values."""
    lo = np.array([int(v) & 0xFFFFFFFFFFFFFFFF for v in x], dtype=np.uint64)
    hi = np.array([int(v) >> 64 for v in x], dtype=np.uint64)
    return lo.view(np.int64), hi.view(np.int64)


def _u128_to_f64(x):
    """FP64 of exact 128-bit sums as the device converts them (u128_to_f64 in
    nz_canonical.cu): each 64-bit half to FP64, then one rounded addition."""
    lo, hi = _halves(x)
    return np.ldexp(hi.view(np.uint64).astype(np.float64), 64) + lo.view(np.uint64).astype(np.float64)


def merge_states(states):
    """Host-side merge of ensemble states (the dicts Ensemble.state()
    returns, one per rank or checkpoint) of disjoint runs of one lattice and
    p grid: counts add, (mean, M2) merge pairwise, exact microcanonical sums
    add as 128-bit integers and their M2 merge pairwise with means from the
    sums.  Raises ValueError for incompatible states or shared runs."""
    from . import store
    states = [s for s in states if s is not None]
    if not states:
        raise ValueError('no states to merge')
    first = states[0]
    for st in states:
        store.check_state(st)
        if not store.compatible(first['meta'], st['meta'], first['ps'], st['ps']):
            raise ValueError('states differ in lattice, p grid or arithmetic')
    ledger = store.ledger_array(np.concatenate([store.ledger_array(s['ledger']) for s in states]))
    if store.ledger_overlaps(ledger):
        raise ValueError('states share runs; merging would count them twice')
    out = {'meta': dict(first['meta']), 'ps': np.asarray(first['ps']).copy(), 'ledger': ledger,
           'count': np.asarray(first['count'], np.int64).reshape(1).copy(),
           'mean': np.asarray(first['mean'], np.float64).copy(),
           'm2': np.asarray(first['m2'], np.float64).copy(), 'micro': None}
    micro = first['micro'] is not None
    if micro:
        mc = first['micro']
        out['micro'] = {'count': np.asarray(mc['count'], np.int64).reshape(1).copy(),
                        'span_count': np.asarray(mc['span_count'], np.int64).copy(),
                        'sum_lo': np.asarray(mc['sum_lo'], np.int64).copy(),
                        'sum_hi': np.asarray(mc['sum_hi'], np.int64).copy(),
                        'm2': np.asarray(mc['m2'], np.float64).copy()}
    for st in states[1:]:
        na, nb = float(out['count'][0]), float(np.asarray(st['count']).reshape(1)[0])
        out['mean'], out['m2'] = _pairwise(na, out['mean'], out['m2'], nb,
                                           np.asarray(st['mean'], np.float64),
                                           np.asarray(st['m2'], np.float64))
        out['count'] = out['count'] + np.asarray(st['count'], np.int64).reshape(1)
        if micro:
            a, b = out['micro'], st['micro']
            ca, cb = float(a['count'][0]), float(np.asarray(b['count']).reshape(1)[0])
            sa, sb = _u128(a['sum_lo'], a['sum_hi']), _u128(b['sum_lo'], b['sum_hi'])
            ma = _u128_to_f64(sa) / ca if ca > 0 else np.zeros(len(sa))
            mb = _u128_to_f64(sb) / cb if cb > 0 else np.zeros(len(sb))
            _, a['m2'] = _pairwise(ca, ma, np.asarray(a['m2'], np.float64), cb, mb,
                                   np.asarray(b['m2'], np.float64))
            a['sum_lo'], a['sum_hi'] = _halves(sa + sb)
            a['span_count'] = a['span_count'] + np.asarray(b['span_count'], np.int64)
            a['count'] = a['count'] + np.asarray(b['count'], np.int64).reshape(1)
    return out
