"""Batched uneven ensembles: thousands of runs of different lattices in one
persistent launch (libnzgb300 ``nz_mix``).

Each run r draws its substrate from Philox(key, r): a spanning_1d_chain(l)
with probability ``chain_share``, else a spanning_2d_grid(L), the length
log-uniform in its range and rounded to the nearest integer
(percolate/percolate.py:899-965).  The runs are reduced per lattice at
``checkpoints`` evenly spaced occupation numbers to exact sums and M2 of the
microcanonical statistics (percolate/percolate.py:450-705 at those n).

``fused=True`` reduces the runs inside the persistent union-find (each run
adds its statistics and their squares into its lattice's exact sums by
integer atomics) instead of writing per-run checkpoint records for a second
kernel; the results are identical.

``MixEnsemble.capture()`` records the whole launch sequence in a CUDA graph;
``replay(key)`` re-runs it for another key without re-launching from Python.
"""
import math

import numpy as np

from . import _native as nat

STATS = ('max', 'm0', 'm1', 'm2', 'm3', 'm4')


def log_uniform_thresholds(lo, hi):
    """thr[i] (uint32) for length lo + i: the length is the largest lo + i
    with thr[i] <= u for a uniform 32-bit u, i.e. round(exp(U)) for U uniform
    in [ln lo, ln hi] (thresholds at the half-integers, thr[0] = 0)."""
    lo, hi = int(lo), int(hi)
    n = hi - lo + 1
    thr = np.zeros(n, dtype=np.uint32)
    if n > 1:
        lens = np.arange(lo + 1, hi + 1, dtype=np.float64)
        x = np.log((lens - 0.5) / lo) / math.log(hi / lo)
        thr[1:] = np.clip(np.ceil(np.ldexp(x, 32)), 0, 2 ** 32 - 1).astype(np.uint32)
    return thr


class MixEnsemble:
    """One batched uneven ensemble configuration (sizes fixed, key varies)."""

    def __init__(self, n_runs, grid=(8, 512), chain=(1024, 65536), chain_share=0.5,
                 checkpoints=256, threads=None, block=128, smem_words=0, fused=False):
        torch = nat.torch_cuda()
        self.n_runs = int(n_runs)
        self.spec = nat.NzMixSpec()
        self.spec.grid_min, self.spec.grid_max = int(grid[0]), int(grid[1])
        self.spec.chain_min, self.spec.chain_max = int(chain[0]), int(chain[1])
        self.spec.chain_share = min(int(round(chain_share * 2 ** 32)), 2 ** 32 - 1)
        self.spec.checkpoints = int(checkpoints)
        self.spec.reduction = 1 if fused else 0
        self.fused = bool(fused)
        self.F = int(checkpoints)
        self.n_grid = grid[1] - grid[0] + 1
        self.n_chain = chain[1] - chain[0] + 1
        self.n_classes = self.n_grid + self.n_chain
        self.block = int(block)
        self.smem_words = int(smem_words)
        nmax = max(grid[1] ** 2, chain[1])
        if threads is None:
            threads = min(self.n_runs, max(1024, (48 << 30) // (4 * nmax)))
        self.threads = int(min(threads, self.n_runs))
        self.thr_grid = torch.from_numpy(log_uniform_thresholds(*grid).view(np.int32)).cuda()
        self.thr_chain = torch.from_numpy(log_uniform_thresholds(*chain).view(np.int32)).cuda()
        self.key = torch.zeros(1, dtype=torch.int64, device='cuda')
        C, F = self.n_classes, self.F
        self.count = torch.zeros(C, dtype=torch.int32, device='cuda')
        self.span = torch.zeros(C * F, dtype=torch.int32, device='cuda')
        self.sum_lo = torch.zeros(6 * C * F, dtype=torch.int64, device='cuda')
        self.sum_hi = torch.zeros(6 * C * F, dtype=torch.int64, device='cuda')
        self.m2 = torch.zeros(6 * C * F, dtype=torch.float64, device='cuda')
        self.errors = torch.zeros(1, dtype=torch.int32, device='cuda')
        ws = nat.lib_handle().nz_mix_workspace_bytes(self.spec, self.n_runs, self.threads)
        if ws == 0:
            raise ValueError('invalid mix specification')
        self.ws = nat.device_empty(ws)
        self.graph = None

    def _accum(self):
        a = nat.NzMixAccum()
        a.count = self.count.data_ptr()
        a.span = self.span.data_ptr()
        a.sum_lo = self.sum_lo.data_ptr()
        a.sum_hi = self.sum_hi.data_ptr()
        a.m2 = self.m2.data_ptr()
        a.errors = self.errors.data_ptr()
        return a

    def _launch(self):
        st = nat.lib_handle().nz_mix(self.spec, nat.ptr(self.thr_grid), nat.ptr(self.thr_chain),
                                     nat.ptr(self.key), self.n_runs, self.threads, self.block,
                                     self.smem_words, nat.ptr(self.ws), self.ws.numel(),
                                     self._accum(), nat.stream_handle())
        nat.check(st, 'nz_mix')

    def run(self, key):
        self.key.fill_(int(key))
        self._launch()
        return self

    def capture(self):
        """Record the launch sequence in a CUDA graph (key read on the device)."""
        torch = nat.torch_cuda()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self._launch()  # warm-up outside the capture
        torch.cuda.current_stream().wait_stream(s)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._launch()
        return self

    def replay(self, key):
        self.key.fill_(int(key))
        self.graph.replay()
        return self

    @property
    def additions(self):
        """Bond additions of the last run (sum over classes of runs x M)."""
        counts = self.count.cpu().numpy()
        return int((counts.astype(np.int64) * self.class_edges()).sum())

    def class_lengths(self):
        return np.concatenate([np.arange(self.spec.grid_min, self.spec.grid_max + 1),
                               np.arange(self.spec.chain_min, self.spec.chain_max + 1)])

    def class_edges(self):
        L = self.class_lengths().astype(np.int64)
        M = L - 1
        M[:self.n_grid] = 2 * L[:self.n_grid] * (L[:self.n_grid] - 1)
        return M

    def results(self):
        """Host copies: count[C], span[C, F], sums (object ints) [6, C, F], m2 [6, C, F]."""
        C, F = self.n_classes, self.F
        if int(self.errors.cpu().numpy()[0]):
            raise RuntimeError('nz_mix skipped runs (internal slot check failed)')
        lo = self.sum_lo.cpu().numpy().view(np.uint64).reshape(6, C, F)
        hi = self.sum_hi.cpu().numpy().view(np.uint64).reshape(6, C, F)
        return {'count': self.count.cpu().numpy().view(np.uint32).copy(),
                'span': self.span.cpu().numpy().view(np.uint32).reshape(C, F).copy(),
                'sum_lo': lo.copy(), 'sum_hi': hi.copy(),
                'm2': self.m2.cpu().numpy().reshape(6, C, F).copy()}
