"""Multi-rank path on CPU (gloo, world size 2): run sharding, gathering and
the associative merge give the single-process result over all runs."""
import os
import socket

import numpy as np
import pytest

from conftest import REPO


def test_shard_runs_partition():
    from pypercolate_gb300.distributed import shard_runs
    for total in (0, 1, 7, 100, 100003):
        for world in (1, 2, 3, 8):
            ranges = [shard_runs(total, world, r) for r in range(world)]
            ids = [i for s, n in ranges for i in range(s, s + n)]
            assert ids == list(range(total))
            assert max(n for _, n in ranges) - min(n for _, n in ranges) <= 1
    with pytest.raises(ValueError):
        shard_runs(10, 2, 2)


def _rank_state(oracle, L, key, run0, count, ps):
    """One rank's ensemble state (the dict Ensemble.state() returns:
    canonical (count, mean, M2) per (p, statistic), exact microcanonical
    accumulators, ledger) for `count` oracle runs -- a CPU stand-in for the
    state of that rank's GPU ensemble."""
    N, M = L * L, 2 * L * (L - 1)
    W = np.stack([oracle.binomial_pmf(M, p) for p in ps])
    acc = None
    vals = np.zeros((6, count, M + 1), dtype=object)
    span = np.zeros(M + 1, dtype=np.int64)
    for i, r in enumerate(range(run0, run0 + count)):
        run = oracle.lattice_run(oracle.GRID_2D, L, oracle.philox_permutation(key, r, M))
        row = (1.0, W @ oracle.q_matrix(run), np.zeros((len(ps), 7)))
        acc = row if acc is None else oracle.reduce_rows(acc, row)
        exact = run['moments_u64'].astype(object) + run['moments_hi'].astype(object) * (1 << 64)
        mx = run['max'].astype(object)
        for k, v in enumerate((mx, exact[:, 0], N - mx, exact[:, 2], exact[:, 3], exact[:, 4])):
            vals[k, i] = v
        span += run['span']
    n, mean, m2 = acc
    sums = vals.sum(axis=1).reshape(-1)
    fl = vals.astype(np.float64)
    micro_m2 = ((fl - fl.mean(axis=1, keepdims=True)) ** 2).sum(axis=1).reshape(-1)
    meta = {'kind': 'grid', 'model': 'bond', 'wrap': 'either', 'length': L, 'N': N, 'M': M,
            'spanning': True, 'precision': 'fp64', 'window': 0, 'cutoff': 80.0, 'micro': True}
    return {'meta': meta, 'ps': np.asarray(ps, np.float64),
            'count': np.array([count], np.int64), 'mean': mean.reshape(-1),
            'm2': m2.reshape(-1), 'ledger': np.array([[key, run0, count]], np.uint64),
            'micro': {'count': np.array([count], np.int64), 'span_count': span,
                      'sum_lo': np.array([int(v) & (2 ** 64 - 1) for v in sums],
                                         np.uint64).view(np.int64),
                      'sum_hi': np.array([int(v) >> 64 for v in sums], np.uint64).view(np.int64),
                      'm2': micro_m2}}


def _worker(rank, world, port, total, result_path):
    import sys
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    from oracle import oracle as O
    from pypercolate_gb300 import store
    from pypercolate_gb300.distributed import gather_objects, merge_states, shard_runs
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    ps = np.linspace(0.3, 0.7, 5)
    run0, count = shard_runs(total, world, rank)
    state = _rank_state(O, 6, 77, run0, count, ps)
    merged = merge_states(gather_objects(state))
    if rank == 0:
        store.save_state(result_path, merged)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_rank_merge_equals_single_process(tmp_path):
    """Two gloo ranks each hold the state of their shard of runs; the
    package's gather and host merge give the state of all runs in one
    process: canonical means to 1e-12, M2 to 1e-9, exact micro sums and
    spanning counts equal, the ledger covering every run once."""
    import torch.multiprocessing as mp
    from oracle import oracle as O
    from pypercolate_gb300 import store
    total = 23
    out = str(tmp_path / 'merged.npz')
    mp.start_processes(_worker, args=(2, _free_port(), total, out), nprocs=2, join=True,
                       start_method='spawn')
    merged = store.load_state(out)
    single = _rank_state(O, 6, 77, 0, total, np.linspace(0.3, 0.7, 5))
    assert int(merged['count'][0]) == total
    assert store.ledger_runs(merged['ledger']) == total
    np.testing.assert_allclose(merged['mean'], single['mean'], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(merged['m2'], single['m2'], rtol=1e-9, atol=1e-9)
    for k in ('sum_lo', 'sum_hi', 'span_count', 'count'):
        assert np.array_equal(merged['micro'][k], single['micro'][k]), k
    np.testing.assert_allclose(merged['micro']['m2'], single['micro']['m2'], rtol=1e-9, atol=1e-6)


def test_host_merge_refuses_shared_runs():
    from oracle import oracle as O
    from pypercolate_gb300.distributed import merge_states
    ps = np.linspace(0.4, 0.6, 3)
    a = _rank_state(O, 4, 5, 0, 3, ps)
    b = _rank_state(O, 4, 5, 2, 3, ps)  # run 2 in both
    with pytest.raises(ValueError):
        merge_states([a, b])
