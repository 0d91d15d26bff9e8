"""Checkpoint files of ensemble state: format, validation, atomic writes and
the run ledger (host logic; the GPU round trip is in test_gpu_store.py)."""
import json
import os

import numpy as np
import pytest

from pypercolate_gb300 import store


def fake_state(P=5, M=12, micro=True, runs=((7, 0, 30), (7, 30, 20)), seed=0):
    rng = np.random.default_rng(seed)
    n = sum(r[2] for r in runs)
    st = {'meta': {'kind': 'grid', 'model': 'bond', 'wrap': 'either', 'length': 3, 'N': 9,
                   'M': M, 'spanning': True,
                   'precision': 'fp32', 'window': 0, 'cutoff': 80.0, 'micro': micro},
          'ps': np.linspace(0, 1, P), 'count': np.array([n], np.int64),
          'mean': rng.normal(size=7 * P), 'm2': rng.uniform(size=7 * P),
          'ledger': store.ledger_array(runs), 'micro': None}
    if micro:
        rows = M + 1
        st['micro'] = {'count': np.array([n], np.int64),
                       'span_count': rng.integers(0, n, rows, dtype=np.int64),
                       'sum_lo': rng.integers(-2**62, 2**62, 6 * rows, dtype=np.int64),
                       'sum_hi': rng.integers(0, 5, 6 * rows, dtype=np.int64),
                       'm2': rng.uniform(size=6 * rows)}
    return st


def assert_same(a, b):
    assert a['meta'] == b['meta']
    for k in ('ps', 'count', 'mean', 'm2', 'ledger'):
        assert np.asarray(a[k]).tobytes() == np.asarray(b[k]).tobytes(), k
    if a['micro'] is None:
        assert b['micro'] is None
    else:
        for k in store.MICRO_KEYS:
            assert a['micro'][k].tobytes() == b['micro'][k].tobytes(), k


@pytest.mark.parametrize('micro', [True, False])
def test_round_trip_is_bit_exact(tmp_path, micro):
    st = fake_state(micro=micro)
    path = str(tmp_path / 'ens.npz')
    store.save_state(path, st)
    assert_same(st, store.load_state(path))
    # nothing but the checkpoint is left in the directory
    assert os.listdir(tmp_path) == ['ens.npz']


def test_failed_save_keeps_previous_checkpoint(tmp_path):
    path = str(tmp_path / 'ens.npz')
    good = fake_state(seed=1)
    store.save_state(path, good)
    bad = fake_state(seed=2)
    bad['count'] = np.array([3], np.int64)  # disagrees with the ledger
    with pytest.raises(ValueError):
        store.save_state(path, bad)
    assert_same(good, store.load_state(path))
    assert os.listdir(tmp_path) == ['ens.npz']


def test_rejects_foreign_and_inconsistent_files(tmp_path):
    other = str(tmp_path / 'other.npz')
    np.savez(other, x=np.arange(3))
    with pytest.raises(ValueError, match='not an ensemble state'):
        store.load_state(other)
    st = fake_state()
    st['mean'] = st['mean'][:-1]
    with pytest.raises(ValueError, match='probabilities'):
        store.check_state(st)
    st = fake_state()
    st['micro']['count'] = np.array([1], np.int64)
    with pytest.raises(ValueError, match='micro accumulators count'):
        store.check_state(st)
    st = fake_state()
    st['micro']['m2'] = st['micro']['m2'][:5]
    with pytest.raises(ValueError, match='micro_m2'):
        store.check_state(st)
    st = fake_state(runs=((7, 0, 30), (7, 29, 20)))
    with pytest.raises(ValueError, match='twice'):
        store.check_state(st)
    # the meta is JSON the user can read without this package
    path = str(tmp_path / 'ens.npz')
    store.save_state(path, fake_state())
    with np.load(path) as z:
        assert json.loads(str(z['meta']))['kind'] == 'grid'
        assert str(z['format']) == store.FORMAT


def test_ledger():
    L = store.ledger_array([(1, 0, 10), (1, 10, 5), (2, 0, 10)])
    assert not store.ledger_overlaps(L)
    assert store.ledger_runs(L) == 25 and store.ledger_runs(L, key=1) == 15
    assert store.ledger_next_run(L, 1) == 15
    assert store.ledger_next_run(L, 2) == 10
    assert store.ledger_next_run(L, 3) == 0
    assert store.ledger_overlaps([(1, 0, 10), (2, 5, 5), (1, 9, 1)])
    assert not store.ledger_overlaps([(1, 0, 10), (1, 10, 0), (1, 5, 0)])  # empty batches
    # keys above 2^63 survive the uint64 ledger
    assert store.ledger_next_run([(2**64 - 1, 3, 4)], 2**64 - 1) == 7


def test_compatible():
    a, b = fake_state(), fake_state(seed=5)
    assert store.compatible(a['meta'], b['meta'], a['ps'], b['ps'])
    b['meta'] = dict(b['meta'], window=4096)  # launch shape only
    assert store.compatible(a['meta'], b['meta'], a['ps'], b['ps'])
    for k, v in (('length', 4), ('precision', 'fp64'), ('precision', 'tf32x3'), ('micro', False),
                 ('cutoff', 40.0), ('model', 'site'), ('wrap', 'x')):
        c = dict(a['meta'], **{k: v})
        assert not store.compatible(a['meta'], c, a['ps'], a['ps'])
    assert not store.compatible(a['meta'], a['meta'], a['ps'], a['ps'][:-1])
    assert not store.compatible(a['meta'], a['meta'], a['ps'], a['ps'] + 1e-12)
