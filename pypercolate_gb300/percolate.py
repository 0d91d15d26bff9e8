"""Substrate lattices and graph preparation, drop-in for the helpers of
``percolate.percolate`` that the HPC path uses.

* ``spanning_2d_grid``  -- percolate/percolate.py:931-965
* ``spanning_1d_chain`` -- percolate/percolate.py:899-928
* ``percolation_graph`` -- percolate/percolate.py:31-100
* ``_binomial_pmf``     -- percolate/percolate.py:1067-1109 (computed on the GPU)

The builders return networkx graphs with the same nodes, edges and ``'span'``
attributes as the reference, and tag them (``graph.graph['nz_lattice']``) so
the GPU path can number the lattice arithmetically instead of walking an edge
list.  Where networkx is not installed they return a small stand-in with the
same node and edge order, which the rest of this package accepts.
"""
import numpy as np

from . import _native as nat

try:  # networkx is optional: the GPU path never needs it
    import networkx as nx
except ImportError:  # pragma: no cover - exercised only where networkx is absent
    nx = None

alpha_1sigma = 0.31731050786291415
"""2 * Phi(-1): the alpha of the 1-sigma confidence level
(percolate/percolate.py:25)."""


class LatticeGraph:
    """networkx-free stand-in for the lattices of this module.

    Node labels and edge order are those networkx (>= 2) produces for the
    reference's builders: grid nodes (i, j) row-major, chain nodes 0..l+1;
    perc_graph.edges() node-major, the edge to the next row before the edge to
    the next column.
    """

    def __init__(self, kind, length, with_aux=True):
        self.kind = kind
        self.length = int(length)
        self.with_aux = with_aux
        self.graph = {'nz_lattice': (kind, int(length))}

    def _perc_nodes(self):
        L = self.length
        if self.kind == 'grid':
            return [(i, j) for i in range(1, L + 1) for j in range(L)]
        return list(range(1, L + 1))

    def nodes(self, data=False):
        L = self.length
        if self.kind == 'grid':
            nodes = [(i, j) for i in range(L + 2) for j in range(L)] if self.with_aux \
                else self._perc_nodes()
        else:
            nodes = list(range(L + 2)) if self.with_aux else self._perc_nodes()
        if data:
            return [(n, self.node_attrs(n)) for n in nodes]
        return nodes

    def node_attrs(self, n):
        L = self.length
        if not self.with_aux:
            return {}
        if self.kind == 'grid':
            if n[0] == 0:
                return {'span': 0}
            if n[0] == L + 1:
                return {'span': 1}
            return {}
        if n == 0:
            return {'span': 0}
        if n == L + 1:
            return {'span': 1}
        return {}

    def edges(self):
        L = self.length
        out = []
        if self.kind == 'grid':
            for i in range(1, L + 1):
                for j in range(L):
                    if i < L:
                        out.append(((i, j), (i + 1, j)))
                    if j < L - 1:
                        out.append(((i, j), (i, j + 1)))
        else:
            out = [(k, k + 1) for k in range(1, L)]
        return out

    def aux_edges(self):
        L = self.length
        if self.kind == 'grid':
            return {**{((0, j), (1, j)): 0 for j in range(L)},
                    **{((L, j), (L + 1, j)): 1 for j in range(L)}}
        return {(0, 1): 0, (L, L + 1): 1}

    def perc(self):
        return LatticeGraph(self.kind, self.length, with_aux=False)

    def number_of_nodes(self):
        return len(self.nodes())

    def number_of_edges(self):
        return len(self.edges()) + (len(self.aux_edges()) if self.with_aux else 0)


def spanning_2d_grid(length):
    """Square lattice of length x length sites with auxiliary rows 0 and
    length+1 (``'span'`` 0 and 1) for top-bottom spanning detection
    (percolate/percolate.py:931-965)."""
    length = int(length)
    if nx is None:
        return LatticeGraph('grid', length)
    ret = nx.grid_2d_graph(length + 2, length)
    for i in range(length):
        ret.nodes[(0, i)]['span'] = 0
        ret[(0, i)][(1, i)]['span'] = 0
        ret.nodes[(length + 1, i)]['span'] = 1
        ret[(length + 1, i)][(length, i)]['span'] = 1
    ret.graph['nz_lattice'] = ('grid', length)
    return ret


def spanning_1d_chain(length):
    """Chain of `length` sites with auxiliary end nodes 0 and length+1
    (percolate/percolate.py:899-928)."""
    length = int(length)
    if nx is None:
        return LatticeGraph('chain', length)
    ret = nx.grid_graph(dim=[int(length + 2)])
    ret.nodes[0]['span'] = 0
    ret[0][1]['span'] = 0
    ret.nodes[length + 1]['span'] = 1
    ret[length][length + 1]['span'] = 1
    ret.graph['nz_lattice'] = ('chain', length)
    return ret


def percolation_graph(graph, spanning_cluster=True):
    """Strip auxiliary nodes and collect N, M and the spanning attributes
    (percolate/percolate.py:31-100).  Raises ValueError like the reference
    when spanning detection is requested without two sides."""
    ret = dict()
    ret['graph'] = graph
    ret['spanning_cluster'] = bool(spanning_cluster)
    if isinstance(graph, LatticeGraph):
        if spanning_cluster:
            aux_nodes = {n: a['span'] for n, a in graph.nodes(data=True) if 'span' in a}
            ret['auxiliary_node_attributes'] = aux_nodes
            ret['spanning_sides'] = sorted(set(aux_nodes.values()))
            ret['auxiliary_edge_attributes'] = graph.aux_edges()
            perc = graph.perc()
        else:
            perc = graph
        ret['perc_graph'] = perc
        ret['num_nodes'] = perc.number_of_nodes()
        ret['num_edges'] = perc.number_of_edges()
        return ret
    if spanning_cluster:
        aux = nx.get_node_attributes(graph, 'span')
        ret['auxiliary_node_attributes'] = aux
        if not list(aux.keys()):
            raise ValueError('Spanning cluster is to be detected, but no auxiliary nodes given.')
        sides = list(set(aux.values()))
        if len(sides) != 2:
            raise ValueError('Spanning cluster is to be detected, but auxiliary nodes of less or '
                             'more than 2 types (sides) given.')
        ret['spanning_sides'] = sides
        ret['auxiliary_edge_attributes'] = nx.get_edge_attributes(graph, 'span')
        perc = graph.subgraph([n for n in graph.nodes() if 'span' not in graph.nodes[n]])
    else:
        perc = graph
    ret['perc_graph'] = perc
    ret['num_nodes'] = nx.number_of_nodes(perc)
    ret['num_edges'] = nx.number_of_edges(perc)
    return ret


def _binomial_pmf(n, p):
    """Binomial pmf B(n, k, p), k = 0..n, normalised to unit sum, as the
    reference's Newman-Ziff recursion gives it (percolate/percolate.py:
    1067-1109); computed on the GPU in FP64 (weights below exp(-745) of the
    mode, i.e. below FP64 range relative to it, are zero)."""
    torch = nat.torch_cuda()
    n = int(n)
    ps = torch.tensor([float(p)], dtype=torch.float64, device='cuda')
    out = torch.empty(n + 1, dtype=torch.float64, device='cuda')
    nat.check(nat.lib_handle().nz_binomial_pmf(n, nat.ptr(ps), 1, nat.ptr(out),
                                               nat.stream_handle()), 'nz_binomial_pmf')
    return out.cpu().numpy()


def binomial_pmfs(n, ps):
    """Full-length pmf rows for several p (one launch): shape (len(ps), n+1)."""
    torch = nat.torch_cuda()
    n = int(n)
    ps = np.atleast_1d(np.asarray(ps, dtype=np.float64))
    dps = torch.from_numpy(ps.copy()).to('cuda')
    out = torch.empty(len(ps) * (n + 1), dtype=torch.float64, device='cuda')
    nat.check(nat.lib_handle().nz_binomial_pmf(n, nat.ptr(dps), len(ps), nat.ptr(out),
                                               nat.stream_handle()), 'nz_binomial_pmf')
    return out.cpu().numpy().reshape(len(ps), n + 1)


# ---------------------------------------------------------------------------
# classic microcanonical / canonical API (percolate/percolate.py:708-1252)
# ---------------------------------------------------------------------------
_MICRO_RECORD_BUDGET = 1 << 30  # bytes of per-step records per launch


def _micro_accumulators(rows):
    torch = nat.torch_cuda()
    acc = dict(count=torch.zeros(1, dtype=torch.int64, device='cuda'),
               span_count=torch.zeros(rows, dtype=torch.int64, device='cuda'),
               sum_lo=torch.zeros(6 * rows, dtype=torch.int64, device='cuda'),
               sum_hi=torch.zeros(6 * rows, dtype=torch.int64, device='cuda'),
               m2=torch.zeros(6 * rows, dtype=torch.float64, device='cuda'))
    s = nat.NzMicroAccum()
    for k, v in acc.items():
        setattr(s, k, v.data_ptr())
    return acc, s


def _finalize_micro(acc_struct, N, M, spanning, alpha, normalize):
    torch = nat.torch_cuda()
    out = torch.empty((M + 1) * 21, dtype=torch.float64, device='cuda')
    nat.check(nat.lib_handle().nz_microcanonical_finalize(
        acc_struct, N, M, int(spanning), float(alpha), int(normalize), nat.ptr(out),
        nat.stream_handle()), 'nz_microcanonical_finalize')
    return out.cpu().numpy().reshape(M + 1, 21)


def _global_stream_perms(M, runs):
    """The next `runs` permutations np.random.permutation(M) would return
    (drawn on the GPU from numpy's global MT19937 state, which is advanced
    exactly as the draws would advance it)."""
    torch = nat.torch_cuda()
    name, keys, pos, has_gauss, gauss = np.random.get_state()
    if name != 'MT19937':
        raise ValueError('numpy global RandomState is not MT19937')
    state = np.empty(625, dtype=np.uint32)
    state[:624] = keys
    state[624] = pos
    d_in = torch.from_numpy(state.view(np.int32).copy()).cuda()
    d_out = torch.empty(625, dtype=torch.int32, device='cuda')
    perms = torch.empty(max(runs * M, 1), dtype=torch.int32, device='cuda')
    nat.check(nat.lib_handle().nz_mt_stream_permutations(
        nat.ptr(d_in), int(M), int(runs), nat.ptr(perms), nat.ptr(d_out), nat.stream_handle()),
        'nz_mt_stream_permutations')
    new = d_out.cpu().numpy().view(np.uint32)
    np.random.set_state((name, new[:624].copy(), int(new[624]), has_gauss, gauss))
    return perms


class _MicroAverages:
    """Iterator of percolate.microcanonical_averages (see that function)."""

    def __init__(self, graph, runs, spanning_cluster, model, alpha, copy_result):
        self._args = (graph, runs, spanning_cluster, model, alpha)
        self._copy = copy_result
        self._n = 0
        self._rows = None
        self._ret = {}

    def __iter__(self):
        return self

    def _validate(self):
        graph, runs, spanning_cluster, model, alpha = self._args
        try:
            runs = int(runs)
        except (TypeError, ValueError):
            raise ValueError('runs needs to be a positive integer')
        if runs <= 0:
            raise ValueError('runs needs to be a positive integer')
        try:
            alpha = float(alpha)
        except (TypeError, ValueError):
            raise ValueError('alpha needs to be a float in the interval (0, 1)')
        if alpha <= 0.0 or alpha >= 1.0:
            raise ValueError('alpha needs to be a float in the interval (0, 1)')
        if model != 'bond':
            raise ValueError('Only bond percolation supported.')
        pg = percolation_graph(graph, spanning_cluster=spanning_cluster)
        from . import hpc
        self._spec = hpc.graph_spec(**pg)
        self._runs, self._alpha, self._spanning = runs, alpha, bool(spanning_cluster)

    def _initial_row(self):
        """n = 0 for every run: no permutation is drawn yet (as in the
        reference, whose runs draw theirs at their second step)."""
        torch = nat.torch_cuda()
        N, R = self._spec.N, self._runs
        acc, s = _micro_accumulators(1)
        acc['count'].fill_(R)
        # max = 1, and every moment (m1 = N - max included) is N - 1
        vals = torch.tensor([1, N - 1, N - 1, N - 1, N - 1, N - 1], dtype=torch.int64,
                            device='cuda') * R
        acc['sum_lo'].copy_(vals)
        return _finalize_micro(s, N, 0, self._spanning, self._alpha, 0)[0]

    def _all_rows(self, normalize=0):
        from . import hpc
        spec, R = self._spec, self._runs
        N, M = spec.N, spec.M
        perms = _global_stream_perms(M, R)
        acc, s = _micro_accumulators(M + 1)
        chunk = max(1, min(R, _MICRO_RECORD_BUDGET // (36 * (M + 1))))
        for r0 in range(0, R, chunk):
            rc = min(chunk, R - r0)
            p = perms[r0 * M:(r0 + rc) * M].cpu().numpy().view(np.uint32).reshape(rc, M)
            rec = hpc._run_microcanonical(spec, self._spanning, perms=p if M else None,
                                          seeds=None if M else [0] * rc, with_edge=False)
            nat.check(nat.lib_handle().nz_microcanonical_reduce(
                rec.struct(), N, M, rc, 0, M + 1, s, nat.stream_handle()),
                'nz_microcanonical_reduce')
        return _finalize_micro(s, N, M, self._spanning, self._alpha, normalize)

    def _row_dict(self, n, o):
        spec = self._spec
        ret = dict() if self._copy else self._ret
        ret['n'] = n
        ret['N'] = spec.N
        ret['M'] = spec.M
        ret['max_cluster_size'] = float(o[3])
        ret['max_cluster_size_ci'] = np.array(o[4:6])
        ret['moments'] = np.array(o[6:21:3])
        ret['moments_ci'] = np.stack([o[7 + 3 * k:9 + 3 * k] for k in range(5)])
        if self._spanning:
            ret['spanning_cluster'] = float(o[0])
            ret['spanning_cluster_ci'] = np.array(o[1:3])
        return ret

    def __next__(self):
        if self._n == 0:
            self._validate()
            row = self._initial_row()
        else:
            if self._n > self._spec.M:
                raise StopIteration
            if self._rows is None:
                self._rows = self._all_rows()
            row = self._rows[self._n]
        out = self._row_dict(self._n, row)
        self._n += 1
        return out

    def arrays(self):
        """microcanonical_averages_arrays of a fresh iterator, normalised on the GPU."""
        if self._n != 0:
            raise ValueError('iterator already advanced')
        self._validate()
        self._n = self._spec.M + 1
        o = self._all_rows(normalize=1)
        ret = {'N': self._spec.N, 'M': self._spec.M}
        ret['max_cluster_size'] = o[:, 3].copy()
        ret['max_cluster_size_ci'] = o[:, 4:6].copy()
        if self._spanning:
            ret['spanning_cluster'] = o[:, 0].copy()
            ret['spanning_cluster_ci'] = o[:, 1:3].copy()
        ret['moments'] = np.stack([o[:, 6 + 3 * k] for k in range(5)])
        ret['moments_ci'] = np.stack([o[:, 7 + 3 * k:9 + 3 * k] for k in range(5)])
        return ret


def microcanonical_averages(graph, runs=40, spanning_cluster=True, model='bond',
                            alpha=alpha_1sigma, copy_result=True):
    """Microcanonical ensemble averages over `runs` runs for n = 0..M
    (percolate/percolate.py:708-896).  Yields one dict per n (absolute units,
    like the reference).  The runs draw np.random.permutation(M) in turn from
    numpy's global RandomState (continued on the GPU), so a given
    np.random.seed reproduces the reference's averages; the whole ensemble is
    computed by the union-find and run-reduction kernels when n = 1 is
    requested.  ValueErrors are raised at the first next()."""
    return _MicroAverages(graph, runs, spanning_cluster, model, alpha, copy_result)


def microcanonical_averages_arrays(microcanonical_averages):
    """Arrays over n of the microcanonical averages, max and moments divided
    by N (percolate/percolate.py:968-1064)."""
    if isinstance(microcanonical_averages, _MicroAverages):
        return microcanonical_averages.arrays()
    ret = dict()
    for n, avg in enumerate(microcanonical_averages):
        assert n == avg['n']
        if n == 0:
            M, N = avg['M'], avg['N']
            spanning = 'spanning_cluster' in avg
            ret['max_cluster_size'] = np.empty(M + 1)
            ret['max_cluster_size_ci'] = np.empty((M + 1, 2))
            if spanning:
                ret['spanning_cluster'] = np.empty(M + 1)
                ret['spanning_cluster_ci'] = np.empty((M + 1, 2))
            ret['moments'] = np.empty((5, M + 1))
            ret['moments_ci'] = np.empty((5, M + 1, 2))
        ret['max_cluster_size'][n] = avg['max_cluster_size']
        ret['max_cluster_size_ci'][n] = avg['max_cluster_size_ci']
        if spanning:
            ret['spanning_cluster'][n] = avg['spanning_cluster']
            ret['spanning_cluster_ci'][n] = avg['spanning_cluster_ci']
        ret['moments'][:, n] = avg['moments']
        ret['moments_ci'][:, n] = avg['moments_ci']
    for key in list(ret):
        if 'spanning_cluster' not in key:
            ret[key] = ret[key] / N
    ret['M'], ret['N'] = M, N
    return ret


def canonical_averages(ps, microcanonical_averages_arrays):
    """Canonical averages at each p: binomial weights (FP64, GPU) times every
    microcanonical array, confidence bounds included, as the reference does
    (percolate/percolate.py:1112-1221).  The weights are computed over the
    band where the pmf does not underflow (nz_binomial_weights, cutoff 745)
    and contracted with the arrays by nz_band_dot (FP64, one CTA per p)."""
    torch = nat.torch_cuda()
    lib = nat.lib_handle()
    arr = microcanonical_averages_arrays
    N, M = arr['N'], arr['M']
    ps = np.asarray(ps, dtype=np.float64)
    flat = np.ascontiguousarray(ps.ravel())
    P = flat.size
    spanning = 'spanning_cluster' in arr
    cols = [arr['max_cluster_size'][:, None], arr['max_cluster_size_ci'],
            arr['moments'].T, arr['moments_ci'].transpose(1, 0, 2).reshape(M + 1, 10)]
    if spanning:
        cols += [arr['spanning_cluster'][:, None], arr['spanning_cluster_ci']]
    V = torch.from_numpy(np.ascontiguousarray(np.hstack(cols), dtype=np.float64)).cuda()
    ncols = int(V.shape[1])
    cutoff = 745.0  # FP64 underflow: the range of the reference's pmf
    cap = int(lib.nz_binomial_band_cap(M, cutoff))
    d_ps = torch.from_numpy(flat.copy()).cuda()
    lo = torch.empty(P, dtype=torch.int32, device='cuda')
    ln = torch.empty(P, dtype=torch.int32, device='cuda')
    w = torch.empty(P * cap, dtype=torch.float64, device='cuda')
    s = nat.stream_handle()
    nat.check(lib.nz_binomial_weights(M, nat.ptr(d_ps), P, cutoff, cap, nat.ptr(lo), nat.ptr(ln),
                                      nat.ptr(w), s), 'nz_binomial_weights')
    out = torch.empty(P * ncols, dtype=torch.float64, device='cuda')
    nat.check(lib.nz_band_dot(nat.ptr(lo), nat.ptr(ln), nat.ptr(w), cap, P, nat.ptr(V), M + 1,
                              ncols, nat.ptr(out), s), 'nz_band_dot')
    C = out.cpu().numpy().reshape(P, ncols)
    ret = {'ps': ps, 'N': N, 'M': M}
    ret['max_cluster_size'] = C[:, 0]
    ret['max_cluster_size_ci'] = C[:, 1:3]
    ret['moments'] = C[:, 3:8].T.copy()
    ret['moments_ci'] = C[:, 8:18].reshape(-1, 5, 2).transpose(1, 0, 2).copy()
    if spanning:
        ret['spanning_cluster'] = C[:, 18]
        ret['spanning_cluster_ci'] = C[:, 19:21]
    return ret


def statistics(graph, ps, spanning_cluster=True, model='bond', alpha=alpha_1sigma, runs=40):
    """Canonical statistics of `graph` (percolate/percolate.py:1226-1252)."""
    return canonical_averages(ps, microcanonical_averages_arrays(microcanonical_averages(
        graph=graph, runs=runs, spanning_cluster=spanning_cluster, model=model, alpha=alpha)))
