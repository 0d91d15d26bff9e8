"""CPU oracle for the Newman-Ziff bond-percolation path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
import it.  The product package (``pypercolate_gb300``) never does.

Two layers:

* ``libnzoracle.so`` (``oracle/nz_oracle.c``): exact-integer restatement of
  ``percolate/hpc.py:195-307`` (the Newman-Ziff loop), Philox-4x32-10, the
  Philox-keyed Feistel permutation, MT19937 with numpy's legacy shuffle, the
  implicit lattices, banded FP64 canonical weights and a threaded ensemble
  pipeline used as the CPU baseline.
* numpy restatements of the FP64 stages:
  ``binomial_pmf``               percolate/percolate.py:1067-1109
  ``canonical_statistics``       percolate/hpc.py:443-515
  ``initialize_canonical_averages``  percolate/hpc.py:561-635
  ``reduce_rows``                percolate/hpc.py:638-702 (pairwise merge)
  ``finalize``                   percolate/hpc.py:752-834
  ``microcanonical_average_*``   percolate/percolate.py:450-705
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, '_build', 'libnzoracle.so')

GRID_2D = 0
CHAIN_1D = 1

_lib = None


def build(force=False):
    """Compile ``nz_oracle.c`` and ``nz_census.c`` with the committed Makefile."""
    srcs = [os.path.join(HERE, f) for f in ('nz_oracle.c', 'nz_census.c', 'Makefile')]
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(f) for f in srcs)):
        return LIB_PATH
    subprocess.check_call(['make', '-s', '-C', HERE])
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        L.nzo_philox4x32_10.argtypes = [u32p, u32p, u32p]
        L.nzo_philox_permutation.argtypes = [ctypes.c_uint64, ctypes.c_uint64,
                                             ctypes.c_uint32, u32p]
        L.nzo_mt_permutation.argtypes = [u32p, ctypes.c_int, ctypes.c_uint32, u32p]
        L.nzo_lattice_graph.argtypes = [ctypes.c_int, ctypes.c_uint32, u32p, u32p,
                                        ctypes.c_void_p]
        L.nzo_sample_states.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u32p, u32p,
                                        ctypes.c_void_p, ctypes.c_int, u32p,
                                        ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p]
        L.nzo_binomial_band.argtypes = [ctypes.c_uint32, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_uint32,
                                        u32p, u32p, ctypes.c_void_p]
        L.nzo_ensemble_canonical.argtypes = [
            ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64,
            ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.c_void_p,
            ctypes.c_void_p]
        L.nzo_ensemble_uf.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64,
                                      ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int]
        L.nzo_ensemble_uf.restype = ctypes.c_uint64
        L.nzo_lattice_census.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                                         u32p] + [ctypes.c_void_p] * 6
        _lib = L
    return _lib


def _u32p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


# --------------------------------------------------------------------------
# random numbers and permutations
# --------------------------------------------------------------------------
def philox4x32_10(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.empty(4, dtype=np.uint32)
    lib().nzo_philox4x32_10(_u32p(c), _u32p(k), _u32p(out))
    return out


def philox_permutation(key, run_id, M):
    """The project's Philox-keyed Feistel permutation of range(M)."""
    out = np.empty(max(int(M), 1), dtype=np.uint32)
    lib().nzo_philox_permutation(int(key), int(run_id), int(M), _u32p(out))
    return out[:int(M)]


def mt_permutation(seed, M):
    """np.random.RandomState(seed).permutation(M), restated (hpc.py:195,206)."""
    if np.ndim(seed) == 0:
        words = np.array([int(seed)], dtype=np.uint32)
        n_words = 0
    else:
        words = np.asarray(seed, dtype=np.int64).astype(np.uint32).ravel()
        n_words = int(words.size)
    out = np.empty(max(int(M), 1), dtype=np.uint32)
    lib().nzo_mt_permutation(_u32p(words), n_words, int(M), _u32p(out))
    return out[:int(M)]


# --------------------------------------------------------------------------
# graphs
# --------------------------------------------------------------------------
def lattice_size(kind, L):
    L = int(L)
    if kind == GRID_2D:
        return L * L, 2 * L * (L - 1)
    return L, L - 1


def lattice_graph(kind, L):
    """(N, M, edge_u, edge_v, side) of spanning_2d_grid(L) / spanning_1d_chain(L)."""
    N, M = lattice_size(kind, L)
    eu = np.empty(max(M, 1), dtype=np.uint32)
    ev = np.empty(max(M, 1), dtype=np.uint32)
    side = np.empty(N, dtype=np.uint8)
    lib().nzo_lattice_graph(kind, int(L), _u32p(eu), _u32p(ev),
                            side.ctypes.data_as(ctypes.c_void_p))
    return N, M, eu[:M], ev[:M], side


# --------------------------------------------------------------------------
# microcanonical statistics
# --------------------------------------------------------------------------
def sample_states(N, M, eu, ev, side, spanning, perm):
    """Exact per-step statistics for one run with a given permutation.

    Returns dict with ``edge`` (M+1,), ``max`` (M+1,), ``span`` (M+1,) bool,
    ``moments`` (M+1, 5) as Python-int-exact object array and ``moments_u64``
    (the reference's uint64 view, i.e. the exact value modulo 2**64).
    """
    eu = np.ascontiguousarray(eu, dtype=np.uint32)
    ev = np.ascontiguousarray(ev, dtype=np.uint32)
    side = np.ascontiguousarray(side, dtype=np.uint8)
    perm = np.ascontiguousarray(perm, dtype=np.uint32)
    if eu.size == 0:
        eu = np.zeros(1, np.uint32)
        ev = np.zeros(1, np.uint32)
    if perm.size == 0:
        perm = np.zeros(1, np.uint32)
    edge = np.empty(M + 1, dtype=np.uint32)
    mx = np.empty(M + 1, dtype=np.uint32)
    sp = np.empty(M + 1, dtype=np.uint8)
    lo = np.empty((M + 1, 5), dtype=np.uint64)
    hi = np.empty((M + 1, 5), dtype=np.uint64)
    st = lib().nzo_sample_states(
        int(N), int(M), _u32p(eu), _u32p(ev), side.ctypes.data_as(ctypes.c_void_p),
        int(bool(spanning)), _u32p(perm), edge.ctypes.data_as(ctypes.c_void_p),
        mx.ctypes.data_as(ctypes.c_void_p), sp.ctypes.data_as(ctypes.c_void_p),
        lo.ctypes.data_as(ctypes.c_void_p), hi.ctypes.data_as(ctypes.c_void_p))
    if st == 2:
        raise ValueError('Spanning cluster is to be detected, but auxiliary '
                         'nodes of less or more than 2 types (sides) given.')
    if st:
        raise RuntimeError('oracle sample_states failed: %d' % st)
    return {'edge': edge, 'max': mx, 'span': sp.astype(bool),
            'moments_u64': lo, 'moments_hi': hi,
            'moments_f64': np.ldexp(hi.astype(np.float64), 64) + lo.astype(np.float64)}


def lattice_run(kind, L, perm, spanning=True):
    N, M, eu, ev, side = lattice_graph(kind, L)
    return sample_states(N, M, eu, ev, side, spanning, perm)


# --------------------------------------------------------------------------
# canonical stages (FP64, numpy)
# --------------------------------------------------------------------------
def binomial_pmf(n, p):
    """Newman-Ziff Eq. (10) recursion from the mode, normalised
    (percolate/percolate.py:1092-1109), restated."""
    n = int(n)
    ret = np.empty(n + 1)
    nmax = int(np.round(p * n))
    ret[nmax] = 1.0
    with np.errstate(under='ignore'):
        for i in range(nmax + 1, n + 1):
            ret[i] = ret[i - 1] * (n - i + 1.0) / i * p / (1.0 - p)
        for i in range(nmax - 1, -1, -1):
            ret[i] = ret[i + 1] * (i + 1.0) / (n - i) * (1.0 - p) / p
    return ret / ret.sum()


def binomial_band(M, p, cutoff=80.0, cap=None):
    """Banded normalised weights from log B via lgamma (C restatement)."""
    if cap is None:
        cap = M + 1
    w = np.empty(cap, dtype=np.float64)
    lo = np.zeros(1, np.uint32)
    ln = np.zeros(1, np.uint32)
    st = lib().nzo_binomial_band(int(M), float(p), float(cutoff), int(cap),
                                 _u32p(lo), _u32p(ln), w.ctypes.data_as(ctypes.c_void_p))
    if st:
        raise RuntimeError('band capacity too small')
    return int(lo[0]), w[:int(ln[0])].copy()


STAT_NAMES = ('percolation_probability', 'max_cluster_size', 'm0', 'm1', 'm2', 'm3', 'm4')


def q_matrix(run, spanning=True):
    """(M+1, 7) FP64 matrix of per-step statistics in the order
    (spanning, max, m0..m4); moments from the exact integers."""
    M1 = run['max'].size
    q = np.empty((M1, 7))
    q[:, 0] = run['span'] if spanning else 0.0
    q[:, 1] = run['max']
    q[:, 2:] = run['moments_f64']
    return q


def canonical_statistics(q, weights):
    """Q(p) = sum_n w_n Q_n (percolate/hpc.py:495-512) -> 7 values."""
    return np.asarray(weights) @ q


def reduce_rows(a, b):
    """Pairwise (n, mean, M2) merge, Chan-Golub-LeVeque (hpc.py:638-702)."""
    na, ma, sa = a
    nb, mb, sb = b
    n = na + nb
    d = mb - ma
    mean = ma + d * nb / n
    m2 = sa + sb + d * d * na * nb / n
    return n, mean, m2


def finalize(number_of_nodes, n, mean, m2, alpha, normalize):
    """mean, std, Student-t CI exactly as hpc.py:782-826 computes them."""
    import scipy.stats
    with np.errstate(divide='ignore', invalid='ignore'):
        mean = np.array(mean, dtype=np.float64)
        std = np.sqrt(np.asarray(m2, dtype=np.float64) / (n - 1))
        if normalize:
            mean = mean / number_of_nodes
            std = std / number_of_nodes
        lo, hi = scipy.stats.t.interval(1 - alpha, df=n - 1, loc=mean,
                                        scale=std / np.sqrt(n))
    return mean, std, np.asarray(lo), np.asarray(hi)


def microcanonical_average_spanning(k, runs, alpha):
    """Bayesian posterior mean and Beta credible interval
    (percolate/percolate.py:450-566)."""
    import scipy.stats
    k = np.asarray(k, dtype=np.float64)
    mean = (k + 1) / (runs + 2)
    lo = scipy.stats.beta.ppf(alpha / 2, k + 1, runs - k + 1)
    hi = scipy.stats.beta.ppf(1 - alpha / 2, k + 1, runs - k + 1)
    return mean, lo, hi


def microcanonical_average_normal(mean, std, runs, alpha):
    """mean and t-CI, CI = (mean, mean) where std == 0
    (percolate/percolate.py:569-705)."""
    import scipy.stats
    mean = np.asarray(mean, dtype=np.float64)
    std = np.asarray(std, dtype=np.float64)
    with np.errstate(divide='ignore', invalid='ignore'):
        lo, hi = scipy.stats.t.interval(1 - alpha, df=runs - 1, loc=mean,
                                        scale=std / np.sqrt(runs))
    lo = np.where(std > 0, lo, mean)
    hi = np.where(std > 0, hi, mean)
    return lo, hi


# --------------------------------------------------------------------------
# ensemble pipeline on the host cores (CPU baseline / reference arm)
# --------------------------------------------------------------------------
def band_table(M, ps, cutoff=80.0):
    bands = [binomial_band(M, p, cutoff) for p in ps]
    cap = max(len(w) for _, w in bands)
    lo = np.array([b[0] for b in bands], dtype=np.uint32)
    ln = np.array([len(b[1]) for b in bands], dtype=np.uint32)
    W = np.zeros((len(ps), cap))
    for i, (_, w) in enumerate(bands):
        W[i, :len(w)] = w
    return lo, ln, W


def ensemble_canonical(kind, L, key, run0, n_runs, ps, n_threads=None, bands=None):
    """Threaded C pipeline: runs -> canonical stats -> pairwise merge.
    Returns (mean[P,7], m2[P,7])."""
    if n_threads is None:
        n_threads = os.cpu_count() or 1
    N, M = lattice_size(kind, L)
    lo, ln, W = bands if bands is not None else band_table(M, ps)
    W = np.ascontiguousarray(W)
    P = len(ps)
    mean = np.empty((P, 7))
    m2 = np.empty((P, 7))
    st = lib().nzo_ensemble_canonical(
        kind, int(L), int(key), int(run0), int(n_runs), P,
        lo.ctypes.data_as(ctypes.c_void_p), ln.ctypes.data_as(ctypes.c_void_p),
        W.ctypes.data_as(ctypes.c_void_p), int(W.shape[1]), int(n_threads),
        mean.ctypes.data_as(ctypes.c_void_p), m2.ctypes.data_as(ctypes.c_void_p))
    if st:
        raise RuntimeError('oracle ensemble failed: %d' % st)
    return mean, m2


def ensemble_uf(kind, L, key, run0, n_runs, n_threads=None):
    if n_threads is None:
        n_threads = os.cpu_count() or 1
    return int(lib().nzo_ensemble_uf(kind, int(L), int(key), int(run0), int(n_runs),
                                     int(n_threads)))


CENSUS_KINDS = {'grid': 0, 'chain': 1, 'torus': 3}
WRAP_CRITERIA = {'either': 0, 'x': 1, 'y': 2, 'both': 3}


def census_size(kind, L, site):
    """(N, number of steps) of a census lattice."""
    N = L if kind == 'chain' else L * L
    M = {'grid': 2 * L * (L - 1), 'chain': L - 1, 'torus': 2 * L * L}[kind]
    return N, (N if site else M)


def lattice_census(kind, L, perm, site=False, wrap='either'):
    """Brute-force per-step records of one run (nz_census.c): dict of
    max (with the spanning / wrapping flag in bit 31), m0, m2, m3, m4_lo,
    m4_hi, each of length steps + 1."""
    N, steps = census_size(kind, L, site)
    perm = np.ascontiguousarray(perm, dtype=np.uint32)
    assert perm.shape == (steps,)
    out = {'max_span': np.zeros(steps + 1, np.uint32), 'm0': np.zeros(steps + 1, np.uint32),
           'm2': np.zeros(steps + 1, np.uint64), 'm3': np.zeros(steps + 1, np.uint64),
           'm4_lo': np.zeros(steps + 1, np.uint64), 'm4_hi': np.zeros(steps + 1, np.uint32)}
    rc = lib().nzo_lattice_census(CENSUS_KINDS[kind], int(L), int(bool(site)), WRAP_CRITERIA[wrap],
                                  _u32p(perm), *[out[k].ctypes.data_as(ctypes.c_void_p) for k in
                                                 ('max_span', 'm0', 'm2', 'm3', 'm4_lo', 'm4_hi')])
    if rc != 0:
        raise ValueError('census failed for %s L=%d' % (kind, L))
    return out
