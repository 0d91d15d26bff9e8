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

_KINDS = {'grid': nat.GRAPH_GRID2D, 'chain': nat.GRAPH_CHAIN1D}


class Ensemble:
    """Running canonical / microcanonical averages of one lattice.

    kind      'grid' (spanning_2d_grid(length)) or 'chain' (spanning_1d_chain)
    ps        occupation probabilities of the canonical curves
    precision 'fp32' (FP32 products, FP64 accumulation over row chunks) or 'fp64'
    micro     also accumulate microcanonical run-reductions for every n
    window    rows per union-find launch (0: sized to ~8 GiB of records)
    """

    def __init__(self, kind='grid', length=16, ps=None, spanning=True, precision='fp32',
                 micro=True, window=0, cutoff=80.0):
        torch = nat.torch_cuda()
        self.kind = kind
        self.length = int(length)
        self.spec = hpc.GraphSpec(_KINDS[kind], self.length)
        self.N, self.M = self.spec.N, self.spec.M
        self.ps = np.atleast_1d(np.asarray(ps if ps is not None else np.linspace(0, 1, 101),
                                           dtype=np.float64))
        self.P = len(self.ps)
        self.spanning = bool(spanning)
        self.precision = {'fp64': 0, 'fp32': 1}[precision]
        self.window = int(window)
        self.cutoff = float(cutoff)
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
        st = lib.nz_ensemble(g, int(self.spanning), n_runs, int(key), int(run0),
                             nat.ptr(self.d_ps), self.P, self.cutoff, self.window,
                             self.precision, nat.ptr(self._ws), self._ws.numel(),
                             nat.ptr(self.count), nat.ptr(self.mean), nat.ptr(self.m2),
                             micro, nat.stream_handle(stream))
        nat.check(st, 'nz_ensemble')
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
        st = nat.lib_handle().nz_microcanonical_finalize(
            self._micro_struct(), self.N, self.M, int(self.spanning), float(alpha), 1,
            nat.ptr(out), nat.stream_handle())
        nat.check(st, 'nz_microcanonical_finalize')
        o = out.cpu().numpy().reshape(self.M + 1, 21)
        ret = {'N': self.N, 'M': self.M}
        if self.spanning:
            ret['spanning_cluster'] = o[:, 0].copy()
            ret['spanning_cluster_ci'] = o[:, 1:3].copy()
        ret['max_cluster_size'] = o[:, 3].copy()
        ret['max_cluster_size_ci'] = o[:, 4:6].copy()
        ret['moments'] = np.stack([o[:, 6 + 3 * k] for k in range(5)])
        ret['moments_ci'] = np.stack([o[:, 7 + 3 * k:9 + 3 * k] for k in range(5)])
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
