"""Generate the golden fixtures in this directory from the reference itself.

Run in a container where the reference source tree is mounted, passing
its root directory::

    python tests/golden/make_golden.py <reference source tree>

It imports andsor/pypercolate 0.4.6 read-only through ``refshim`` and records
its outputs as small ``.npz`` files.  The GPU test box never runs this
script; tests only read the committed fixtures.

Fixtures
--------
kat_3x3.npz
    The known-answer test of ``percolate/test/test_percolate.py:49-192``:
    the hand-built 3x3 grid, the permutation drawn after
    ``np.random.seed(42)``, and the per-n max cluster sizes, moments and
    spanning flags (both as produced by the reference and as literally
    written in the test file, which this script parses).
hpc_cases.npz
    ``percolate.hpc.bond_microcanonical_statistics`` rows for 2D grids,
    chains, a non-spanning grid and the 3x3 test graph, plus the
    permutation ``RandomState(seed).permutation(M)`` each run used.
hpc_injected.npz
    The same function fed the project's Philox-Feistel permutations
    (substituted for ``RandomState.permutation``).
hpc_checksums.npz
    SHA-256 digests of full reference outputs at L = 64, 128, 256.
canonical.npz
    ``_binomial_pmf``, ``bond_canonical_statistics``,
    ``bond_initialize_canonical_averages``, ``functools.reduce(bond_reduce)``
    and ``finalize_canonical_averages`` on small grids.
micro_avg.npz
    ``percolate.microcanonical_averages`` (classic API) with the per-run
    permutations it drew.
"""
import ast
import functools
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _literal(node):
    """Evaluate the literal-ish expressions used in the reference tests."""
    src = ast.unparse(node)
    return eval(src, {'np': np, '__builtins__': {}}, {})


def parse_kat(test_file):
    tree = ast.parse(open(test_file).read())
    found = {}
    for fn in tree.body:
        if not isinstance(fn, ast.FunctionDef):
            continue
        for st in fn.body:
            if isinstance(st, ast.Assign) and isinstance(st.targets[0], ast.Name):
                name = st.targets[0].id
                if fn.name == 'test_max_cluster_size' and name == 'max_cluster_sizes':
                    found['max'] = np.array(_literal(st.value))
                if fn.name == 'test_moments' and name == 'moments':
                    found['moments'] = np.array(_literal(st.value))
                if fn.name == 'test_spanning' and name == 'has_spanning_cluster':
                    found['span'] = np.array(_literal(st.value))
    return found


def clean(arr):
    """Same structured array with plain-str field names (np.save's header
    must be a Python literal; the reference names fields with np.str_)."""
    dt = np.dtype([(str(n), arr.dtype.fields[n][0]) for n in arr.dtype.names])
    out = np.empty(arr.shape, dtype=dt)
    for n in arr.dtype.names:
        out[str(n)] = arr[n]
    return out


def rows_to_arrays(rows, spanning):
    out = {
        'n': rows['n'].astype(np.uint32),
        'edge': rows['edge'].astype(np.uint32),
        'max': rows['max_cluster_size'].astype(np.uint32),
        'moments': rows['moments'].astype(np.uint64),
    }
    out['edge'][0] = 0  # undefined at n == 0 (hpc.py:212)
    if spanning:
        out['span'] = rows['has_spanning_cluster'].astype(bool)
    return out


def graph_arrays(pg):
    """Node order, edge list and side masks of a percolation_graph dict."""
    perc = pg['perc_graph']
    nodes = list(perc.nodes())
    index = {v: i for i, v in enumerate(nodes)}
    edges = list(perc.edges())
    eu = np.array([index[a] for a, b in edges], dtype=np.uint32)
    ev = np.array([index[b] for a, b in edges], dtype=np.uint32)
    side = np.zeros(len(nodes), dtype=np.uint8)
    if pg.get('spanning_cluster'):
        sides = pg['spanning_sides']
        for (a, b), s in pg['auxiliary_edge_attributes'].items():
            node = a if a in index else b
            side[index[node]] |= np.uint8(1 << sides.index(s))
    return eu, ev, side


class _PermProxy:
    """Stands in for ``percolate.hpc.np`` so that
    ``np.random.RandomState(seed).permutation(M)`` returns a given array."""

    def __init__(self, perm):
        self._perm = perm
        proxy = self

        class _RS:
            def __init__(self, seed=None):
                pass

            def permutation(self, m):
                assert m == len(proxy._perm)
                return np.array(proxy._perm, dtype=np.int64)

        class _Random:
            RandomState = _RS

        self.random = _Random()

    def __getattr__(self, name):
        return getattr(np, name)


def main(reference_root):
    sys.path.insert(0, HERE)
    sys.path.insert(0, REPO)
    import refshim
    import networkx as nx
    percolate = refshim.install(reference_root)
    hpc = percolate.hpc
    from oracle import oracle as O

    # ---------------------------------------------------------------- KAT
    test_file = os.path.join(reference_root, 'percolate', 'test', 'test_percolate.py')
    lit = parse_kat(test_file)
    g = nx.Graph()
    g.add_nodes_from(range(9))
    g.add_edges_from([(i, i + j) for i in [1, 4, 7] for j in [-1, 1]])
    g.add_edges_from([(i, i + j) for i in [3, 4, 5] for j in [-3, 3]])
    g.add_nodes_from(range(9, 12), span=0)
    g.add_nodes_from(range(12, 15), span=1)
    g.add_edges_from([(0, 9), (3, 10), (6, 11)], span=0)
    g.add_edges_from([(2, 12), (5, 13), (8, 14)], span=1)
    np.random.seed(42)
    states = list(percolate.sample_states(g, spanning_cluster=True))
    np.random.seed(42)
    kat_perm = np.random.permutation(12)
    pg = percolate.percolate.percolation_graph(g, spanning_cluster=True)
    eu, ev, side = graph_arrays(pg)
    ref_max = np.array([s['max_cluster_size'] for s in states])
    ref_mom = np.array([s['moments'] for s in states]).astype(np.int64)
    ref_span = np.array([s['has_spanning_cluster'] for s in states])
    assert np.array_equal(ref_max, lit['max'])
    assert np.array_equal(ref_mom, lit['moments'])
    assert np.array_equal(ref_span, lit['span'])
    np.savez(os.path.join(HERE, 'kat_3x3.npz'), eu=eu, ev=ev, side=side,
             perm=kat_perm.astype(np.uint32), max=ref_max.astype(np.uint32),
             moments=ref_mom.astype(np.uint64), span=ref_span,
             test_max=lit['max'], test_moments=lit['moments'], test_span=lit['span'])

    # ---------------------------------------------------------- hpc cases
    cases = []
    for L in (2, 3, 4, 8, 16):
        for seed in (0, 42, 4294967295):
            cases.append(('grid', L, seed, True))
    for L in (3, 8):
        cases.append(('grid_nospan', L, 7, False))
    for L in (1, 2, 3, 10, 100):
        cases.append(('chain', L, 5, True))
    for seed in (0, 1, 2):
        cases.append(('kat', 3, seed, True))
    store = {}
    for ci, (kind, L, seed, spanning) in enumerate(cases):
        if kind == 'grid':
            pg = percolate.percolate.percolation_graph(
                percolate.spanning_2d_grid(L), spanning_cluster=True)
        elif kind == 'grid_nospan':
            pg = percolate.percolate.percolation_graph(
                nx.grid_2d_graph(L, L), spanning_cluster=False)
        elif kind == 'chain':
            pg = percolate.percolate.percolation_graph(
                percolate.spanning_1d_chain(L), spanning_cluster=True)
        else:
            pg = percolate.percolate.percolation_graph(g, spanning_cluster=True)
        rows = hpc.bond_microcanonical_statistics(seed=seed, **pg)
        arr = rows_to_arrays(rows, spanning)
        eu, ev, side = graph_arrays(pg)
        M = pg['num_edges']
        pre = 'c%02d_' % ci
        store[pre + 'meta'] = np.array([L, seed, int(spanning), pg['num_nodes'], M],
                                       dtype=np.int64)
        store[pre + 'kind'] = np.array(kind)
        store[pre + 'eu'] = eu
        store[pre + 'ev'] = ev
        store[pre + 'side'] = side
        store[pre + 'perm'] = np.random.RandomState(seed).permutation(M).astype(np.uint32)
        for k, v in arr.items():
            store[pre + k] = v
    store['n_cases'] = np.array(len(cases))
    np.savez_compressed(os.path.join(HERE, 'hpc_cases.npz'), **store)

    # ------------------------------------------- injected Philox perms
    inj = {}
    real_np = hpc.np
    icases = [(3, 1234, 0), (8, 1234, 5), (16, 7, 123456789), (16, 1234, 99999)]
    for ci, (L, key, run) in enumerate(icases):
        pg = percolate.percolate.percolation_graph(percolate.spanning_2d_grid(L))
        perm = O.philox_permutation(key, run, pg['num_edges'])
        hpc.np = _PermProxy(perm)
        try:
            rows = hpc.bond_microcanonical_statistics(seed=0, **pg)
        finally:
            hpc.np = real_np
        arr = rows_to_arrays(rows, True)
        pre = 'i%02d_' % ci
        inj[pre + 'meta'] = np.array([L, key, run], dtype=np.int64)
        inj[pre + 'perm'] = perm
        for k, v in arr.items():
            inj[pre + k] = v
    inj['n_cases'] = np.array(len(icases))
    np.savez_compressed(os.path.join(HERE, 'hpc_injected.npz'), **inj)

    # ------------------------------------------------------- checksums
    ck = {}
    ccases = [(64, 0, 'mt'), (128, 1, 'mt'), (256, 2, 'mt'), (256, 1234, 'philox')]
    for ci, (L, seed, rng) in enumerate(ccases):
        pg = percolate.percolate.percolation_graph(percolate.spanning_2d_grid(L))
        if rng == 'philox':
            perm = O.philox_permutation(seed, 0, pg['num_edges'])
            hpc.np = _PermProxy(perm)
        try:
            rows = hpc.bond_microcanonical_statistics(seed=seed, **pg)
        finally:
            hpc.np = real_np
        arr = rows_to_arrays(rows, True)
        h = hashlib.sha256()
        for k in ('edge', 'max', 'span', 'moments'):
            h.update(np.ascontiguousarray(arr[k]).tobytes())
        pre = 'k%02d_' % ci
        ck[pre + 'meta'] = np.array([L, seed], dtype=np.int64)
        ck[pre + 'rng'] = np.array(rng)
        ck[pre + 'sha256'] = np.array(h.hexdigest())
        ck[pre + 'last_moments'] = arr['moments'][-1]
        ck[pre + 'mid_moments'] = arr['moments'][len(arr['moments']) // 2]
        ck[pre + 'max_moments'] = arr['moments'].max(axis=0)
    ck['n_cases'] = np.array(len(ccases))
    np.savez(os.path.join(HERE, 'hpc_checksums.npz'), **ck)

    # ------------------------------------------------------- canonical
    can = {}
    pmf = percolate.percolate._binomial_pmf
    pmf_cases = [(0, 0.3), (1, 0.5), (12, 0.0), (12, 1.0), (12, 0.37), (100, 0.1),
                 (1000, 0.01), (480, 0.5), (480, 0.999), (8064, 0.73)]
    for ci, (M, p) in enumerate(pmf_cases):
        can['pmf%02d_M' % ci] = np.array(M)
        can['pmf%02d_p' % ci] = np.array(p)
        can['pmf%02d_w' % ci] = pmf(M, p)
    can['n_pmf'] = np.array(len(pmf_cases))
    ccan = [(3, [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11], [0.1, 0.35, 0.5, 0.77, 1.0], 0.05),
            (8, [11, 22, 33, 44, 55, 66, 77, 88], [0.0, 0.2, 0.45, 0.5, 0.55, 0.9], 0.3173),
            (16, list(range(100, 120)), list(np.linspace(0.4, 0.6, 11)), 0.01)]
    for ci, (L, seeds, ps, alpha) in enumerate(ccan):
        pg = percolate.percolate.percolation_graph(percolate.spanning_2d_grid(L))
        M = pg['num_edges']
        facs = [pmf(M, p) for p in ps]
        inits = []
        canon = []
        for seed in seeds:
            micro = hpc.bond_microcanonical_statistics(seed=seed, **pg)
            cs = np.fromiter((hpc.bond_canonical_statistics(
                microcanonical_statistics=micro, convolution_factors=f) for f in facs),
                dtype=hpc.canonical_statistics_dtype(True))
            canon.append(cs)
            inits.append(hpc.bond_initialize_canonical_averages(canonical_statistics=cs))
        red = functools.reduce(hpc.bond_reduce, inits)
        fin = hpc.finalize_canonical_averages(number_of_nodes=pg['num_nodes'], ps=ps,
                                              canonical_averages=red, alpha=alpha)
        pre = 'can%02d_' % ci
        can[pre + 'L'] = np.array(L)
        can[pre + 'seeds'] = np.array(seeds, dtype=np.int64)
        can[pre + 'ps'] = np.array(ps)
        can[pre + 'alpha'] = np.array(alpha)
        can[pre + 'canonical'] = clean(np.stack(canon))   # structured (R, P)
        can[pre + 'reduced'] = clean(red)                  # structured (P,)
        can[pre + 'final'] = clean(fin)                    # structured (P,)
    can['n_can'] = np.array(len(ccan))
    np.savez(os.path.join(HERE, 'canonical.npz'), **can)

    # ------------------------------------------------ classic micro avg
    mic = {}
    mcases = [(3, 40, 1, percolate.percolate.alpha_1sigma), (8, 25, 2, 0.05)]
    for ci, (L, runs, seed, alpha) in enumerate(mcases):
        graph = percolate.spanning_2d_grid(L)
        M = 2 * L * (L - 1)
        np.random.seed(seed)
        perms = np.stack([np.random.permutation(M) for _ in range(runs)])
        np.random.seed(seed)
        res = percolate.microcanonical_averages_arrays(
            percolate.microcanonical_averages(graph, runs=runs, alpha=alpha))
        pre = 'm%02d_' % ci
        mic[pre + 'meta'] = np.array([L, runs, seed])
        mic[pre + 'alpha'] = np.array(alpha)
        mic[pre + 'perms'] = perms.astype(np.uint32)
        for k in ('spanning_cluster', 'spanning_cluster_ci', 'max_cluster_size',
                  'max_cluster_size_ci', 'moments', 'moments_ci'):
            mic[pre + k] = res[k]
        mic[pre + 'N'] = np.array(res['N'])
        mic[pre + 'M'] = np.array(res['M'])
    mic['n_cases'] = np.array(len(mcases))
    np.savez(os.path.join(HERE, 'micro_avg.npz'), **mic)
    print('fixtures written to', HERE)


if __name__ == '__main__':
    import warnings
    warnings.simplefilter('ignore')
    main(sys.argv[1] if len(sys.argv) > 1 else '/root/reference')
