"""Checkpoint / resume of ensemble reduction state.

The reference's HPC workflow keeps every task's result in jug's task store
and writes the finalized curves to HDF5 (percolate/share/jugfile.py:138-156,
240-253); an interrupted job resumes by recomputing only the tasks that have
no stored result.  Here the whole state of a batched ensemble is small -- one
(count, mean, M2) per (p, statistic) and, optionally, exact per-n
microcanonical accumulators -- so a checkpoint is one ``.npz`` file:

  format        FORMAT (below)
  meta          JSON: kind, model, wrap, length, N, M, spanning, precision,
                window, cutoff, micro
  ps            float64 [P]
  count         int64 [1]; mean, m2: float64 [P * 7], statistic order
                (spanning, max, m0 .. m4)
  micro_count   int64 [1], micro_span_count int64 [M + 1],
  micro_sum_lo, micro_sum_hi  int64 [6 (M + 1)] (the two halves of exact
                128-bit sums), micro_m2 float64 [6 (M + 1)]  -- present when
                meta.micro
  ledger        uint64 [k, 3]: (key, first run id, number of runs) of every
                batch of runs the state contains

A save is atomic (a temporary file in the same directory, then
``os.replace``): a crash while saving leaves the previous checkpoint intact.
Restoring a state restores its exact bits, so a resumed job gives the same
numbers as one that was never interrupted.
"""
import json
import os
import tempfile

import numpy as np

FORMAT = 'pypercolate-gb300/ensemble-state/1'
META_KEYS = ('kind', 'model', 'wrap', 'length', 'N', 'M', 'spanning', 'precision', 'window',
             'cutoff', 'micro')
MICRO_KEYS = ('count', 'span_count', 'sum_lo', 'sum_hi', 'm2')


# ------------------------------------------------------------------ ledger
def ledger_array(entries):
    """(k, 3) uint64 array of (key, first run id, number of runs)."""
    a = np.asarray(entries, dtype=np.uint64)
    return a.reshape(-1, 3)


def ledger_overlaps(ledger):
    """True if two batches of the ledger share a run id under the same key
    (those runs would be counted twice)."""
    a = ledger_array(ledger)
    for key in np.unique(a[:, 0]):
        iv = a[a[:, 0] == key][:, 1:]
        iv = iv[iv[:, 1] > 0]
        iv = iv[np.argsort(iv[:, 0], kind='stable')]
        if np.any(iv[1:, 0] < iv[:-1, 0] + iv[:-1, 1]):
            return True
    return False


def ledger_runs(ledger, key=None):
    """Number of runs in the ledger (under `key`, or all)."""
    a = ledger_array(ledger)
    if key is not None:
        a = a[a[:, 0] == np.uint64(key)]
    return int(a[:, 2].sum())


def ledger_next_run(ledger, key):
    """First run id after every batch recorded under `key` (0 if none)."""
    a = ledger_array(ledger)
    a = a[a[:, 0] == np.uint64(key)]
    return int((a[:, 1] + a[:, 2]).max()) if len(a) else 0


# ------------------------------------------------------------------ files
def save_state(path, state):
    """Writes a state dict (as Ensemble.state() returns it) atomically."""
    meta = {k: state['meta'][k] for k in META_KEYS}
    arrays = {'format': np.array(FORMAT), 'meta': np.array(json.dumps(meta, sort_keys=True)),
              'ps': np.asarray(state['ps'], dtype=np.float64),
              'count': np.asarray(state['count'], dtype=np.int64).reshape(1),
              'mean': np.asarray(state['mean'], dtype=np.float64),
              'm2': np.asarray(state['m2'], dtype=np.float64),
              'ledger': ledger_array(state['ledger'])}
    if meta['micro']:
        for k in MICRO_KEYS:
            arrays['micro_' + k] = np.asarray(state['micro'][k])
    check_state(_as_state(arrays))
    d = os.path.dirname(os.path.abspath(path))
    fd, tmp = tempfile.mkstemp(prefix='.nzstate-', suffix='.npz', dir=d)
    try:
        with os.fdopen(fd, 'wb') as f:
            np.savez(f, **arrays)
        os.replace(tmp, path)
    except BaseException:
        if os.path.exists(tmp):
            os.unlink(tmp)
        raise


def load_state(path):
    """Reads and validates a checkpoint; returns the state dict."""
    with np.load(path, allow_pickle=False) as z:
        if 'format' not in z.files or str(z['format']) != FORMAT:
            raise ValueError('%s is not an ensemble state (format %r)'
                             % (path, str(z['format']) if 'format' in z.files else None))
        arrays = {k: z[k] for k in z.files}
    state = _as_state(arrays)
    check_state(state)
    return state


def _as_state(arrays):
    meta = json.loads(str(arrays['meta']))
    state = {'meta': meta, 'ps': arrays['ps'], 'count': arrays['count'], 'mean': arrays['mean'],
             'm2': arrays['m2'], 'ledger': ledger_array(arrays['ledger']), 'micro': None}
    if meta.get('micro'):
        state['micro'] = {k: arrays['micro_' + k] for k in MICRO_KEYS}
    return state


def check_state(state):
    """Shapes and consistency of a state dict; raises ValueError."""
    meta = state['meta']
    missing = [k for k in META_KEYS if k not in meta]
    if missing:
        raise ValueError('state meta lacks %s' % missing)
    P = len(state['ps'])
    if state['mean'].shape != (7 * P,) or state['m2'].shape != (7 * P,):
        raise ValueError('state arrays do not match %d probabilities' % P)
    n = int(state['count'][0])
    if n < 0 or n != ledger_runs(state['ledger']):
        raise ValueError('state counts %d runs but its ledger records %d'
                         % (n, ledger_runs(state['ledger'])))
    if ledger_overlaps(state['ledger']):
        raise ValueError('state ledger counts some runs twice')
    if meta['micro']:
        rows = int(meta['M']) + 1
        mc = state['micro']
        if mc is None:
            raise ValueError('state meta has micro accumulators but the file does not')
        shapes = {'count': (1,), 'span_count': (rows,), 'sum_lo': (6 * rows,),
                  'sum_hi': (6 * rows,), 'm2': (6 * rows,)}
        for k, shp in shapes.items():
            if mc[k].shape != shp:
                raise ValueError('micro_%s has shape %s, expected %s' % (k, mc[k].shape, shp))
        if int(mc['count'][0]) != n:
            raise ValueError('micro accumulators count %d runs, canonical %d'
                             % (int(mc['count'][0]), n))


def compatible(meta_a, meta_b, ps_a, ps_b):
    """True if two states describe the same lattice, p grid and arithmetic
    (and so can be merged or resumed into one another)."""
    return (all(meta_a[k] == meta_b[k] for k in META_KEYS if k != 'window')
            and len(ps_a) == len(ps_b) and np.array_equal(np.asarray(ps_a), np.asarray(ps_b)))


# ------------------------------------------------------------------ driver
def run_checkpointed(path, make_ensemble, total_runs, batch, key=0, max_batches=None):
    """Adds runs 0 .. total_runs-1 under `key` in batches of `batch` runs,
    saving the state to `path` after every batch.

    If `path` exists, its state is loaded first -- it must describe the
    ensemble that ``make_ensemble()`` builds -- and the work continues after
    the last run its ledger records, so a job killed between batches loses at
    most one batch.  `max_batches` bounds the batches done by this call (a
    scheduler's wall-clock slot).  Returns (ensemble, done) with done True
    once all total_runs runs are in the state.
    """
    from .ensemble import Ensemble
    ens = make_ensemble()
    if os.path.exists(path):
        st = load_state(path)
        if not compatible(st['meta'], ens.state_meta(), st['ps'], ens.ps):
            raise ValueError('%s holds a different ensemble' % path)
        other = set(int(k) for k in ledger_array(st['ledger'])[:, 0]) - {int(key)}
        if other:
            raise ValueError('%s holds runs under other keys %s' % (path, sorted(other)))
        ens = Ensemble.from_state(st, window=ens.window)
    done_batches = 0
    while True:
        start = ledger_next_run(ens.ledger, key)
        if start >= total_runs:
            return ens, True
        if max_batches is not None and done_batches >= max_batches:
            return ens, False
        n = min(int(batch), int(total_runs) - start)
        ens.run(n, key=key, run0=start)
        save_state(path, ens.state())
        done_batches += 1
