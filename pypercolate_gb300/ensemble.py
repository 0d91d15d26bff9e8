"""Batched ensembles: many Newman-Ziff runs of one lattice per launch sequence.

This is the fast path behind the reference's HPC workflow
(percolate/share/jugfile.py:57-135: per run ``bond_microcanonical_statistics``
-> per p ``bond_canonical_statistics`` -> ``bond_initialize_canonical_averages``
-> ``functools.reduce(bond_reduce)`` -> ``finalize_canonical_averages``).
One call of ``Ensemble.run`` performs, for all its runs at once and without
materialising per-run microcanonical arrays: Philox permutations, the
union-find, the fused microcanonical run-reductions, the banded canonical
convolution at every p, and the pairwise merge into running (n, mean, M2)
accumulators that stay on the device between calls.

The accumulated state converts to the reference's structured arrays
(``canonical_averages``, ``finalized``) and to the classic microcanonical
averages (``microcanonical_averages``, the arrays of
percolate/percolate.py:968-1064).
"""
import numpy as np

from . import _native as nat
from . import hpc

# convolution precisions, in the order of nz_ensemble's conv_precision codes
PRECISIONS = ('fp64', 'fp32', 'tf32x3')

_KINDS = {'grid': nat.GRAPH_GRID2D, 'chain': nat.GRAPH_CHAIN1D, 'torus': nat.GRAPH_TORUS2D}


def lattice_kind(kind, model='bond', wrap='either'):
    """NZ_GRAPH_* code with its model / wrapping flags."""
    if kind not in _KINDS:
        raise ValueError('unknown lattice %r' % (kind,))
    if model not in ('bond', 'site'):
        raise ValueError("model must be 'bond' or 'site'")
    if wrap not in nat.WRAP:
        raise ValueError('wrap must be one of %s' % sorted(nat.WRAP))
    if wrap != 'either' and kind != 'torus':
        raise ValueError('a wrapping criterion needs the torus')
    return _KINDS[kind] | (nat.MODEL_SITE if model == 'site' else 0) | nat.WRAP[wrap]


class Ensemble:
    """Running canonical / microcanonical averages of one lattice.

    kind      'grid' (spanning_2d_grid(length)), 'chain' (spanning_1d_chain) or
              'torus' (length x length periodic square lattice, whose
              "spanning" curves are wrapping probabilities, criterion `wrap`:
              'either', 'x', 'y' or 'both' directions)
    model     'bond' (the reference's model) or 'site' percolation; for site
              percolation M = N steps, and p is the site occupation probability
    ps        occupation probabilities of the canonical curves
    precision 'fp32' (FP32 SIMT products, FP64 accumulation over row chunks),
              'tf32x3' (tensor cores: three split TF32 products per term, FP32
              sums per 32-row chunk added into TwoSum pairs) or 'fp64'
    micro     also accumulate microcanonical run-reductions for every n
    window    rows per union-find launch (0: sized to ~32 GiB of records per window)
    tuning    launch shapes {'uf_block', 'm2_tile', 'reduce_slices', 'conv_tile', 'taper'}
              (autotune.tune_ensemble picks them; None: the library's defaults)
    """

    def __init__(self, kind='grid', length=16, ps=None, spanning=True, precision='fp32',
                 micro=True, window=0, cutoff=80.0, model='bond', wrap='either', tuning=None):
        torch = nat.torch_cuda()
        self.kind = kind
        self.model = model
        self.wrap = wrap
        self.length = int(length)
        self.spec = hpc.GraphSpec(lattice_kind(kind, model, wrap), self.length)
        self.N, self.M = self.spec.N, self.spec.M
        self.ps = np.atleast_1d(np.asarray(ps if ps is not None else np.linspace(0, 1, 101),
                                           dtype=np.float64))
        self.P = len(self.ps)
        self.spanning = bool(spanning)
        self.precision = PRECISIONS.index(precision)
        self.window = int(window)
        self.cutoff = float(cutoff)
        self.tuning = dict(tuning) if tuning else None
        self.d_ps = torch.from_numpy(self.ps.copy()).to('cuda')
        self.count = torch.zeros(1, dtype=torch.int64, device='cuda')
        self.mean = torch.zeros(self.P * 7, dtype=torch.float64, device='cuda')
        self.m2 = torch.zeros(self.P * 7, dtype=torch.float64, device='cuda')
        self.micro = None
        if micro:
            rows = self.M + 1
            self.micro = dict(
                count=torch.zeros(1, dtype=torch.int64, device='cuda'),
                span_count=torch.zeros(rows, dtype=torch.int64, device='cuda'),
                sum_lo=torch.zeros(6 * rows, dtype=torch.int64, device='cuda'),
                sum_hi=torch.zeros(6 * rows, dtype=torch.int64, device='cuda'),
                m2=torch.zeros(6 * rows, dtype=torch.float64, device='cuda'))
        self._ws = None
        self._ws_runs = 0
        self.ledger = []  # (key, first run id, number of runs) of every batch added

    # ------------------------------------------------------------------
    def _micro_struct(self):
        if self.micro is None:
            return None
        a = nat.NzMicroAccum()
        for k in ('count', 'span_count', 'sum_lo', 'sum_hi', 'm2'):
            setattr(a, k, self.micro[k].data_ptr())
        return a

    def workspace_bytes(self, n_runs):
        return nat.lib_handle().nz_ensemble_workspace_bytes(self.spec.struct(), int(n_runs),
                                                            self.P, self.window)

    def run(self, n_runs, key=0, run0=0, stream=None):
        """Add n_runs Philox runs (run ids run0 .. run0+n_runs-1 under `key`)."""
        lib = nat.lib_handle()
        n_runs = int(n_runs)
        g = self.spec.struct()
        need = lib.nz_ensemble_workspace_bytes(g, n_runs, self.P, self.window)
        if self._ws is None or self._ws.numel() < need:
            self._ws = None
            self._ws = nat.device_empty(need)
        micro = self._micro_struct()
        tune = None
        if self.tuning:
            tune = nat.NzTuning(int(self.tuning.get('uf_block', 0)), int(self.tuning.get('m2_tile', 0)),
                                int(self.tuning.get('reduce_slices', 0)),
                                int(self.tuning.get('conv_tile', 0)),
                                int(self.tuning.get('taper', 0)))
        st = lib.nz_ensemble_tuned(g, int(self.spanning), n_runs, int(key), int(run0),
                                   nat.ptr(self.d_ps), self.P, self.cutoff, self.window,
                                   self.precision, tune, nat.ptr(self._ws), self._ws.numel(),
                                   nat.ptr(self.count), nat.ptr(self.mean), nat.ptr(self.m2),
                                   micro, nat.stream_handle(stream))
        nat.check(st, 'nz_ensemble_tuned')
        self.ledger.append((int(key), int(run0), n_runs))
        self._last_runs = n_runs
        return self

    def errors(self):
        """Runs of the last `run` whose union-find state came out corrupt (a
        find over the depth bound): 0 in every valid use (synchronises)."""
        if self._ws is None:
            return 0
        torch = nat.torch_cuda()
        out = torch.zeros(1, dtype=torch.int32, device='cuda')
        st = nat.lib_handle().nz_ensemble_errors(self.spec.struct(), self._last_runs, self.P,
                                                 self.window, nat.ptr(self._ws), self._ws.numel(),
                                                 nat.ptr(out), nat.stream_handle())
        nat.check(st, 'nz_ensemble_errors')
        return int(out.cpu().numpy()[0])

    # ------------------------------------------------------------------ state
    def state_meta(self):
        return {'kind': self.kind, 'model': self.model, 'wrap': self.wrap,
                'length': self.length, 'N': self.N, 'M': self.M,
                'spanning': self.spanning, 'precision': PRECISIONS[self.precision],
                'window': self.window, 'cutoff': self.cutoff, 'micro': self.micro is not None}

    def state(self):
        """The accumulated state as host arrays (the checkpoint contents of
        pypercolate_gb300.store)."""
        from . import store
        st = {'meta': self.state_meta(), 'ps': self.ps.copy(),
              'count': self.count.cpu().numpy().copy(), 'mean': self.mean.cpu().numpy().copy(),
              'm2': self.m2.cpu().numpy().copy(), 'ledger': store.ledger_array(self.ledger),
              'micro': None}
        if self.micro is not None:
            st['micro'] = {k: v.cpu().numpy().copy() for k, v in self.micro.items()}
        return st

    @classmethod
    def from_state(cls, state, window=None):
        """An ensemble holding exactly the accumulated state `state`."""
        from . import store
        store.check_state(state)
        meta = state['meta']
        ens = cls(meta['kind'], meta['length'], state['ps'], spanning=meta['spanning'],
                  precision=meta['precision'], micro=meta['micro'],
                  window=meta['window'] if window is None else window, cutoff=meta['cutoff'],
                  model=meta['model'], wrap=meta['wrap'])
        if (ens.N, ens.M) != (meta['N'], meta['M']):
            raise ValueError('state describes N=%s, M=%s; the lattice has N=%d, M=%d'
                             % (meta['N'], meta['M'], ens.N, ens.M))
        torch = nat.torch_cuda()
        ens.count.copy_(torch.from_numpy(np.asarray(state['count'], np.int64).reshape(1)))
        ens.mean.copy_(torch.from_numpy(np.asarray(state['mean'], np.float64)))
        ens.m2.copy_(torch.from_numpy(np.asarray(state['m2'], np.float64)))
        if ens.micro is not None:
            for k, v in ens.micro.items():
                v.copy_(torch.from_numpy(np.ascontiguousarray(state['micro'][k])))
        ens.ledger = [tuple(int(x) for x in row) for row in store.ledger_array(state['ledger'])]
        return ens

    def save(self, path):
        """Atomic checkpoint of the accumulated state (a .npz file)."""
        from . import store
        store.save_state(path, self.state())

    @classmethod
    def load(cls, path, window=None):
        from . import store
        return cls.from_state(store.load_state(path), window=window)

    def merge(self, other):
        """Adds the runs of another ensemble of the same lattice and p grid
        (another GPU's shard, another process's checkpoint) to this one, on
        the device: canonical (count, mean, M2) and the microcanonical
        accumulators merge pairwise, exact sums add.  Raises ValueError if
        the two share a run (same key and run id)."""
        from . import store
        if isinstance(other, dict):
            other = Ensemble.from_state(other)
        if not store.compatible(self.state_meta(), other.state_meta(), self.ps, other.ps):
            raise ValueError('ensembles differ in lattice, p grid or arithmetic')
        ledger = store.ledger_array(list(self.ledger) + list(other.ledger))
        if store.ledger_overlaps(ledger):
            raise ValueError('ensembles share runs; merging would count them twice')
        lib = nat.lib_handle()
        s = nat.stream_handle()
        if self.micro is not None:
            nat.check(lib.nz_micro_merge(self._micro_struct(), other._micro_struct(), self.M, s),
                      'nz_micro_merge')
        nat.check(lib.nz_canonical_merge(nat.ptr(self.count), nat.ptr(self.mean), nat.ptr(self.m2),
                                         nat.ptr(other.count), nat.ptr(other.mean),
                                         nat.ptr(other.m2), 7 * self.P, s), 'nz_canonical_merge')
        self.ledger = list(self.ledger) + list(other.ledger)
        return self

    # ------------------------------------------------------------------
    def canonical_averages(self):
        """Accumulated state as the reference's canonical_averages array."""
        n = int(self.count.cpu().numpy()[0])
        mean = self.mean.cpu().numpy().reshape(self.P, 7)
        m2 = self.m2.cpu().numpy().reshape(self.P, 7)
        ret = np.empty(self.P, dtype=hpc.canonical_averages_dtype(self.spanning))
        ret['number_of_runs'] = n
        if self.spanning:
            ret['percolation_probability_mean'] = mean[:, 0]
            ret['percolation_probability_m2'] = m2[:, 0]
        ret['max_cluster_size_mean'] = mean[:, 1]
        ret['max_cluster_size_m2'] = m2[:, 1]
        ret['moments_mean'] = mean[:, 2:]
        ret['moments_m2'] = m2[:, 2:]
        return ret

    def finalized(self, alpha=0.05):
        """finalize_canonical_averages of the accumulated state (on the GPU)."""
        return hpc.finalize_canonical_averages(self.N, self.ps, self.canonical_averages(), alpha)

    def microcanonical_averages(self, alpha=0.05):
        """Classic microcanonical averages of every n (the dict of
        percolate/percolate.py:968-1064 microcanonical_averages_arrays)."""
        if self.micro is None:
            raise ValueError('ensemble was created with micro=False')
        torch = nat.torch_cuda()
        out = torch.empty((self.M + 1) * 21, dtype=torch.float64, device='cuda')
        # normalised, field-major (2 = NZ_MICRO_FIELD_MAJOR): each value's rows contiguous
        st = nat.lib_handle().nz_microcanonical_finalize(
            self._micro_struct(), self.N, self.M, int(self.spanning), float(alpha), 1 | 2,
            nat.ptr(out), nat.stream_handle())
        nat.check(st, 'nz_microcanonical_finalize')
        o = out.cpu().numpy().reshape(21, self.M + 1)
        pair = lambda j: np.stack([o[j], o[j + 1]], axis=1)  # noqa: E731
        ret = {'N': self.N, 'M': self.M}
        if self.spanning:
            ret['spanning_cluster'] = o[0].copy()
            ret['spanning_cluster_ci'] = pair(1)
        ret['max_cluster_size'] = o[3].copy()
        ret['max_cluster_size_ci'] = pair(4)
        ret['moments'] = o[6:21:3].copy()
        ret['moments_ci'] = np.stack([pair(7 + 3 * k) for k in range(5)])
        return ret

    def micro_sums(self):
        """Exact per-n sums (object array of Python ints, shape (6, M+1)),
        spanning counts and M2 -- for checking."""
        lo = self.micro['sum_lo'].cpu().numpy().view(np.uint64).reshape(6, self.M + 1)
        hi = self.micro['sum_hi'].cpu().numpy().view(np.uint64).reshape(6, self.M + 1)
        sums = np.empty(lo.shape, dtype=object)
        for idx in np.ndindex(lo.shape):
            sums[idx] = (int(hi[idx]) << 64) | int(lo[idx])
        return {'count': int(self.micro['count'].cpu().numpy()[0]),
                'span_count': self.micro['span_count'].cpu().numpy().astype(np.uint64),
                'sums': sums,
                'm2': self.micro['m2'].cpu().numpy().reshape(6, self.M + 1)}
