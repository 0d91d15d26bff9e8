"""Batched uneven ensembles (one persistent launch over runs of different
lattices) against the CPU oracle: per-lattice run counts, exact per-checkpoint
sums of every statistic, spanning counts and M2; CUDA-graph replay."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZE_TAG = 0x53495A45


@pytest.fixture(scope='module')
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from pypercolate_gb300 import _native as nat
    nat.lib_handle()
    return nat


def _oracle_mix(oracle, ens, key):
    """Exact per-class checkpoint sums recomputed run by run on the CPU."""
    from pypercolate_gb300.mix import log_uniform_thresholds
    sp = ens.spec
    thr_g = log_uniform_thresholds(sp.grid_min, sp.grid_max)
    thr_c = log_uniform_thresholds(sp.chain_min, sp.chain_max)
    C, F = ens.n_classes, ens.F
    count = np.zeros(C, dtype=np.int64)
    span = np.zeros((C, F), dtype=np.int64)
    sums = np.zeros((6, C, F), dtype=object)
    sq = np.zeros((6, C, F), dtype=object)
    for r in range(ens.n_runs):
        w = oracle.philox4x32_10([r, 0, 0, SIZE_TAG], [key & 0xffffffff, key >> 32])
        if int(w[0]) < sp.chain_share:
            L = sp.chain_min + int(np.searchsorted(thr_c, w[1], side='right')) - 1
            c, kind = ens.n_grid + L - sp.chain_min, oracle.CHAIN_1D
        else:
            L = sp.grid_min + int(np.searchsorted(thr_g, w[1], side='right')) - 1
            c, kind = L - sp.grid_min, oracle.GRID_2D
        N, M = oracle.lattice_size(kind, L)
        run = oracle.lattice_run(kind, L, oracle.philox_permutation(key, r, M))
        rows = [(j * M) // (F - 1) for j in range(F)]
        count[c] += 1
        exact = (run['moments_hi'].astype(object) << 64) + run['moments_u64'].astype(object)
        for j, n in enumerate(rows):
            x = [int(run['max'][n]), int(exact[n, 0]), N - int(run['max'][n]),
                 int(exact[n, 2]), int(exact[n, 3]), int(exact[n, 4])]
            span[c, j] += int(run['span'][n])
            for k in range(6):
                sums[k, c, j] += x[k]
                sq[k, c, j] += x[k] * x[k]
    return count, span, sums, sq


@pytest.mark.parametrize('smem_words,fused', [(0, False), (128, False), (0, True), (128, True)])
def test_mix_exact_against_oracle(gpu, oracle, smem_words, fused):
    from pypercolate_gb300.mix import MixEnsemble
    key = 0x1234567890
    ens = MixEnsemble(1500, grid=(3, 20), chain=(10, 300), chain_share=0.5, checkpoints=16,
                      threads=256, block=64, smem_words=smem_words, fused=fused)
    ens.run(key)
    got = ens.results()
    count, span, sums, sq = _oracle_mix(oracle, ens, key)
    assert np.array_equal(got['count'].astype(np.int64), count)
    assert np.array_equal(got['span'].astype(np.int64), span)
    exact = (got['sum_hi'].astype(object) << 64) + got['sum_lo'].astype(object)
    assert (exact == sums).all()
    with np.errstate(invalid='ignore', divide='ignore'):
        cnt = count[None, :, None].astype(object)
        m2 = np.where(cnt > 0, (cnt * sq - sums * sums), 0).astype(np.float64) / np.maximum(
            count[None, :, None], 1)
    np.testing.assert_allclose(got['m2'], m2, rtol=1e-12, atol=1e-9)
    assert ens.additions == int((count * ens.class_edges()).sum())


def test_mix_graph_replay(gpu):
    from pypercolate_gb300.mix import MixEnsemble
    a = MixEnsemble(3000, grid=(4, 40), chain=(50, 2000), chain_share=0.3, checkpoints=8,
                    threads=512, block=128)
    a.capture()
    a.replay(77)
    ga = a.results()
    b = MixEnsemble(3000, grid=(4, 40), chain=(50, 2000), chain_share=0.3, checkpoints=8,
                    threads=512, block=128)
    b.run(77)
    gb = b.results()
    for k in ga:
        assert np.array_equal(ga[k], gb[k]), k
    a.replay(78)
    assert not np.array_equal(a.results()['sum_lo'], gb['sum_lo'])


def test_mix_fused_equals_records(gpu):
    """The reduction fused into the union-find (integer atomics into per-lattice
    sums) gives the same integers and M2 as per-run records reduced by a
    second kernel, including lattices with more checkpoints than rows
    (F - 1 > M: several checkpoints per row) and runs sharing warps."""
    from pypercolate_gb300.mix import MixEnsemble
    out = []
    for fused in (False, True):
        e = MixEnsemble(20000, grid=(2, 64), chain=(3, 5000), chain_share=0.4, checkpoints=300,
                        threads=4096, block=128, fused=fused)
        e.run(99)
        out.append(e.results())
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k


def test_mix_fused_graph_replay(gpu):
    from pypercolate_gb300.mix import MixEnsemble
    a = MixEnsemble(3000, grid=(4, 40), chain=(50, 2000), chain_share=0.3, checkpoints=8,
                    threads=512, block=128, fused=True)
    a.capture()
    a.replay(77)
    ga = a.results()
    b = MixEnsemble(3000, grid=(4, 40), chain=(50, 2000), chain_share=0.3, checkpoints=8,
                    threads=512, block=128, fused=False)
    b.run(77)
    gb = b.results()
    for k in ga:
        assert np.array_equal(ga[k], gb[k]), k


def test_tune_mix_times_both_reductions(gpu):
    from pypercolate_gb300.autotune import tune_mix
    t = tune_mix(4000, grid=(4, 24), chain=(64, 1024), checkpoints=32, cache_path=None,
                 candidates=[(1024, 128, 0), (2048, 64, 0)])
    assert len(t['best']) == 4
    assert [row[3] for row in t['table']] == [False, False, True]
    assert all(row[4] > 0 for row in t['table'])
