"""Import shim that lets the read-only reference package run in this container.

Test infrastructure only: used by ``make_golden.py`` to generate the committed
fixtures.  Nothing on the GPU side imports it (the reference tree is not present
there).

The reference (andsor/pypercolate 0.4.6) was written for Python 2/3.4,
networkx 1.x, numpy 1.9 and hypothesis 1.x.  This shim supplies, in-process:

* ``future.builtins`` -> the Python 3 ``builtins`` module;
* ``simoa.stats.online_variance`` -> the pairwise mean/M2 merge of Chan, Golub
  and LeVeque ("Updating formulae and a pairwise algorithm for computing sample
  variances", 1979), which is what ``percolate/hpc.py:677-684`` calls;
* the numpy-1 aliases ``np.float`` / ``np.bool`` / ``np.int``;
* networkx 1.x spellings used by the reference: ``Graph.nodes_iter``,
  ``Graph.node`` and a list-returning ``Graph.edges()``
  (``percolate/percolate.py:85-86,244,295``, ``percolate/hpc.py:205,246``).
"""
import builtins
import sys
import types

import numpy as np
import networkx as nx


def _online_variance(*args):
    """Chan et al. pairwise merge of (n, mean, M2) triples (restated)."""
    n_a, mean_a, m2_a = args[0]
    for n_b, mean_b, m2_b in args[1:]:
        n_a = np.asarray(n_a, dtype=np.float64)
        n_b = np.asarray(n_b, dtype=np.float64)
        n = n_a + n_b
        delta = np.asarray(mean_b) - np.asarray(mean_a)
        mean = mean_a + delta * n_b / n
        m2 = m2_a + m2_b + delta ** 2 * n_a * n_b / n
        n_a, mean_a, m2_a = n, mean, m2
    return n_a, mean_a, m2_a


def install(reference_root):
    future = types.ModuleType('future')
    future.builtins = builtins
    future_utils = types.ModuleType('future.utils')
    future_utils.iteritems = lambda d: iter(d.items())
    future.utils = future_utils
    sys.modules.setdefault('future', future)
    sys.modules.setdefault('future.builtins', builtins)
    sys.modules.setdefault('future.utils', future_utils)

    simoa = types.ModuleType('simoa')
    simoa_stats = types.ModuleType('simoa.stats')
    simoa_stats.online_variance = _online_variance
    simoa.stats = simoa_stats
    sys.modules.setdefault('simoa', simoa)
    sys.modules.setdefault('simoa.stats', simoa_stats)

    pkg_resources = types.ModuleType('pkg_resources')

    class _Dist:
        version = '0.4.6'

    pkg_resources.get_distribution = lambda name: _Dist()
    pkg_resources.DistributionNotFound = Exception
    sys.modules.setdefault('pkg_resources', pkg_resources)

    if not hasattr(nx.Graph, 'nodes_iter'):
        nx.Graph.nodes_iter = lambda self: iter(self.nodes())
        nx.Graph.node = property(lambda self: self.nodes)
        edges_view = nx.Graph.__dict__['edges'].func

        class _EdgeCaller:
            """EdgeView stand-in whose no-argument call returns a list."""

            def __init__(self, view):
                self._view = view

            def __call__(self, *a, **k):
                return self._view(*a, **k) if (a or k) else list(self._view)

            def __iter__(self):
                return iter(self._view)

            def __len__(self):
                return len(self._view)

            def __contains__(self, e):
                return e in self._view

            def __getitem__(self, e):
                return self._view[e]

            def __getattr__(self, name):
                return getattr(self._view, name)

        nx.Graph.edges = property(lambda self: _EdgeCaller(edges_view(self)))

    # numpy-1 aliases (percolate/percolate.py:433,561)
    for alias, typ in (('float', float), ('bool', bool), ('int', int)):
        if alias not in np.__dict__:
            setattr(np, alias, typ)

    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
    import percolate  # noqa: F401
    import percolate.hpc  # noqa: F401
    return percolate
