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


def _rank_rows(oracle, hpc, L, key, run0, count, ps):
    """Canonical-averages rows of `count` oracle runs (CPU stand-in for one
    rank's GPU ensemble)."""
    M = 2 * L * (L - 1)
    W = np.stack([oracle.binomial_pmf(M, p) for p in ps])
    acc = None
    for r in range(run0, run0 + count):
        q = oracle.q_matrix(oracle.lattice_run(oracle.GRID_2D, L,
                                               oracle.philox_permutation(key, r, M)))
        row = (1.0, W @ q, np.zeros((len(ps), 7)))
        acc = row if acc is None else oracle.reduce_rows(acc, row)
    n, mean, m2 = acc
    out = np.empty(len(ps), dtype=hpc.canonical_averages_dtype(True))
    out['number_of_runs'] = int(n)
    out['percolation_probability_mean'] = mean[:, 0]
    out['percolation_probability_m2'] = m2[:, 0]
    out['max_cluster_size_mean'] = mean[:, 1]
    out['max_cluster_size_m2'] = m2[:, 1]
    out['moments_mean'] = mean[:, 2:]
    out['moments_m2'] = m2[:, 2:]
    return out


def _oracle_reducer(a, b):
    """bond_reduce restated on the CPU (test stand-in for the GPU kernel)."""
    from oracle import oracle as O
    out = a.copy()
    na = a['number_of_runs'].astype(float)
    nb = b['number_of_runs'].astype(float)
    for key in ('percolation_probability', 'max_cluster_size', 'moments'):
        ma, sa = a[key + '_mean'], a[key + '_m2']
        mb, sb = b[key + '_mean'], b[key + '_m2']
        shape = (-1,) + (1,) * (ma.ndim - 1)
        _, m, s = O.reduce_rows((na.reshape(shape), ma, sa), (nb.reshape(shape), mb, sb))
        out[key + '_mean'], out[key + '_m2'] = m, s
    out['number_of_runs'] = a['number_of_runs'] + b['number_of_runs']
    return out


def _worker(rank, world, port, total, result_path):
    import sys
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    from oracle import oracle as O
    from pypercolate_gb300 import hpc
    from pypercolate_gb300.distributed import gather_rows, merge_rows, shard_runs
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    ps = np.linspace(0.3, 0.7, 5)
    run0, count = shard_runs(total, world, rank)
    rows = _rank_rows(O, hpc, 6, 77, run0, count, ps)
    merged = merge_rows(gather_rows(rows), reducer=_oracle_reducer)
    if rank == 0:
        np.save(result_path, merged)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_rank_merge_equals_single_process(tmp_path):
    import torch.multiprocessing as mp
    from oracle import oracle as O
    from pypercolate_gb300 import hpc
    total = 23
    out = str(tmp_path / 'merged.npy')
    mp.start_processes(_worker, args=(2, _free_port(), total, out), nprocs=2, join=True,
                       start_method='spawn')
    merged = np.load(out)
    single = _rank_rows(O, hpc, 6, 77, 0, total, np.linspace(0.3, 0.7, 5))
    assert np.all(merged['number_of_runs'] == total)
    for k in ('percolation_probability_mean', 'max_cluster_size_mean', 'moments_mean'):
        np.testing.assert_allclose(merged[k], single[k], rtol=1e-12)
    for k in ('percolation_probability_m2', 'max_cluster_size_m2', 'moments_m2'):
        np.testing.assert_allclose(merged[k], single[k], rtol=1e-9, atol=1e-9)
