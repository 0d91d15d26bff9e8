"""Site percolation and wrapping on the periodic square lattice.

The reference implements bond percolation with spanning detection only and
lists site percolation and wrapping as to-do (percolate/__init__.py:68-78;
percolate/percolate.py:210-211 rejects any model but 'bond').  This module
exposes both on the GPU path, with the reference's row format:

* ``model='site'`` on 'grid' (spanning_2d_grid's L x L lattice, spanning
  between its first and last row), 'chain' or 'torus': step n occupies the
  n-th site of a random permutation of the N sites (Newman & Ziff, Phys. Rev.
  Lett. 85, 4104 (2000)); rows n = 0 .. N; moments count occupied sites only.
* ``kind='torus'``: the L x L periodic square lattice, where the
  ``has_spanning_cluster`` field means that a cluster wraps around the torus
  along x or y (``wrap='either'``), along x, along y, or along both
  (Newman & Ziff, Phys. Rev. E 64, 016706 (2001)).

Canonical curves of these models come from ``ensemble.Ensemble(kind, L, ps,
model=..., wrap=...)``; for site percolation p is the site occupation
probability and the convolution runs over B(N, n, p).
"""
import numpy as np

from . import _native as nat
from . import hpc
from .ensemble import lattice_kind


def lattice_spec(kind, length, model='bond', wrap='either'):
    """GraphSpec of an implicit lattice with its model / wrapping flags."""
    return hpc.GraphSpec(lattice_kind(kind, model, wrap), int(length))


def microcanonical_statistics(kind, length, model='site', wrap='either', seed=None, key=None,
                              run=0, spanning_cluster=True):
    """Rows n = 0 .. M of one run (microcanonical_statistics_dtype of
    percolate/hpc.py:34-70; M = N steps for site percolation).

    The order of the steps is numpy's ``RandomState(seed).permutation(M)``
    when `seed` is given (as the reference draws its bond order,
    percolate/hpc.py:195,206), else the Philox permutation of run id `run`
    under `key`."""
    spec = lattice_spec(kind, length, model, wrap)
    if seed is not None:
        rec = hpc._run_microcanonical(spec, spanning_cluster, seeds=[seed])
    else:
        rec = hpc._run_microcanonical(spec, spanning_cluster, rng='philox',
                                      key=0 if key is None else key, run0=run, n_runs=1)
    return hpc._pack_rows(rec, 0, spec, spanning_cluster)


def sample_records(kind, length, model='bond', wrap='either', perms=None, n_runs=1, key=0, run0=0,
                   spanning=True):
    """Per-step records of several runs as host planes shaped (M + 1, runs):
    max_span (bit 31 = spanning / wrapping flag), m0, m2, m3, m4_lo, m4_hi,
    edge (the bond or site of each step).  Steps follow `perms` (runs x M)
    when given, else the Philox permutations of run ids run0 .. run0+n_runs-1."""
    spec = lattice_spec(kind, length, model, wrap)
    if perms is not None:
        rec = hpc._run_microcanonical(spec, spanning, perms=perms)
    else:
        rec = hpc._run_microcanonical(spec, spanning, rng='philox', key=key, run0=run0,
                                      n_runs=n_runs)
    return rec.host()
