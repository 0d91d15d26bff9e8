"""Drop-in replacement of ``percolate.hpc`` (andsor/pypercolate 0.4.6) whose
work runs in libnzgb300.so on a GB300.

Same functions, signatures, structured dtypes and error behaviour as the
reference module:

=======================================  ====================================
this module                              reference
=======================================  ====================================
``microcanonical_statistics_dtype``      percolate/hpc.py:34-70
``bond_sample_states``                   percolate/hpc.py:73-307
``bond_microcanonical_statistics``       percolate/hpc.py:310-404
``canonical_statistics_dtype``           percolate/hpc.py:407-440
``bond_canonical_statistics``            percolate/hpc.py:443-515
``canonical_averages_dtype``             percolate/hpc.py:518-558
``bond_initialize_canonical_averages``   percolate/hpc.py:561-635
``bond_reduce``                          percolate/hpc.py:638-702
``finalized_canonical_averages_dtype``   percolate/hpc.py:705-749
``finalize_canonical_averages``          percolate/hpc.py:752-834
=======================================  ====================================

``bond_finalize_canonical_averages`` is an alias of
``finalize_canonical_averages``.

Random permutations: with an integer / array / None ``seed`` the runs use
``np.random.RandomState(seed).permutation(M)`` exactly as the reference does
(hpc.py:195,206), generated on the GPU by an MT19937 restatement, so results
are bit-identical to the reference's for the same seed.  The keyword
``rng='philox'`` (swallowed by the reference's ``**kwargs``) selects the
project's Philox-keyed permutation instead, with ``seed`` as the Philox key.
"""
import os

import numpy as np

from . import _native as nat


# ---------------------------------------------------------------------------
# structured dtypes (field names and types as in the reference)
# ---------------------------------------------------------------------------
def _ndarray_dtype(fields):
    """List of (name, type) pairs usable as a numpy structured dtype."""
    return [(str(key), values) for key, values in fields]


def microcanonical_statistics_dtype(spanning_cluster=True):
    fields = [('n', 'uint32'), ('edge', 'uint32')]
    if spanning_cluster:
        fields.append(('has_spanning_cluster', 'bool'))
    fields += [('max_cluster_size', 'uint32'), ('moments', '(5,)uint64')]
    return _ndarray_dtype(fields)


def canonical_statistics_dtype(spanning_cluster=True):
    fields = []
    if spanning_cluster:
        fields.append(('percolation_probability', 'float64'))
    fields += [('max_cluster_size', 'float64'), ('moments', '(5,)float64')]
    return _ndarray_dtype(fields)


def canonical_averages_dtype(spanning_cluster=True):
    fields = [('number_of_runs', 'uint32')]
    if spanning_cluster:
        fields += [('percolation_probability_mean', 'float64'),
                   ('percolation_probability_m2', 'float64')]
    fields += [('max_cluster_size_mean', 'float64'), ('max_cluster_size_m2', 'float64'),
               ('moments_mean', '(5,)float64'), ('moments_m2', '(5,)float64')]
    return _ndarray_dtype(fields)


def finalized_canonical_averages_dtype(spanning_cluster=True):
    fields = [('number_of_runs', 'uint32'), ('p', 'float64'), ('alpha', 'float64')]
    if spanning_cluster:
        fields += [('percolation_probability_mean', 'float64'),
                   ('percolation_probability_std', 'float64'),
                   ('percolation_probability_ci', '(2,)float64')]
    fields += [('percolation_strength_mean', 'float64'),
               ('percolation_strength_std', 'float64'),
               ('percolation_strength_ci', '(2,)float64'),
               ('moments_mean', '(5,)float64'), ('moments_std', '(5,)float64'),
               ('moments_ci', '(5,2)float64')]
    return _ndarray_dtype(fields)


# ---------------------------------------------------------------------------
# graphs
# ---------------------------------------------------------------------------
class GraphSpec:
    """What the library needs to know about a percolation graph: either an
    implicit lattice (kind, length) or an explicit edge list over nodes
    numbered in ``perc_graph.nodes()`` order, edges in ``perc_graph.edges()``
    order (so that ``edge`` indices match the reference's)."""

    def __init__(self, kind, length=0, num_nodes=0, num_edges=0, eu=None, ev=None, side=None):
        self.kind = int(kind)  # NZ_GRAPH_* with the NZ_MODEL_SITE / NZ_WRAP_* flags
        self.base = self.kind & nat.KIND_MASK
        self.site = bool(self.kind & nat.MODEL_SITE)
        self.length = int(length)
        self.eu, self.ev, self.side = eu, ev, side
        self._dev = None
        if self.base == nat.GRAPH_GRID2D:
            self.N, self.M = self.length ** 2, 2 * self.length * (self.length - 1)
        elif self.base == nat.GRAPH_CHAIN1D:
            self.N, self.M = self.length, self.length - 1
        elif self.base == nat.GRAPH_TORUS2D:
            self.N, self.M = self.length ** 2, 2 * self.length ** 2
        else:
            self.N, self.M = int(num_nodes), int(num_edges)
        if self.site:
            self.M = self.N  # one step per site

    def struct(self):
        """NzGraph descriptor (uploads an explicit edge list once)."""
        if self.base != nat.GRAPH_EDGES:
            return nat.make_graph(self.kind, self.length)
        if self._dev is None:
            self._dev = (nat.to_device(self.eu.astype(np.uint32)),
                         nat.to_device(self.ev.astype(np.uint32)),
                         nat.to_device(self.side.astype(np.uint8)))
        eu, ev, side = self._dev
        return nat.make_graph(nat.GRAPH_EDGES, 0, self.N, self.M, eu, ev, side)


def _lattice_tag(perc_graph, kwargs):
    tag = kwargs.get('nz_lattice')
    if tag is None:
        tag = getattr(perc_graph, 'graph', {}).get('nz_lattice') if hasattr(perc_graph, 'graph') else None
    return tag


def graph_spec(perc_graph, num_nodes, num_edges, spanning_cluster=True,
               auxiliary_node_attributes=None, auxiliary_edge_attributes=None,
               spanning_sides=None, **kwargs):
    """Resolve the reference's graph keyword arguments into a GraphSpec."""
    tag = _lattice_tag(perc_graph, kwargs)
    if tag is not None and spanning_cluster:
        kind = nat.GRAPH_GRID2D if tag[0] == 'grid' else nat.GRAPH_CHAIN1D
        spec = GraphSpec(kind, tag[1])
        if spec.N == num_nodes and spec.M == num_edges:
            return spec
    nodes = list(perc_graph.nodes())
    index = {v: i for i, v in enumerate(nodes)}
    edges = list(perc_graph.edges())
    if len(nodes) != num_nodes or len(edges) != num_edges:
        raise ValueError('num_nodes / num_edges do not match perc_graph')
    eu = np.fromiter((index[a] for a, b in edges), dtype=np.uint32, count=len(edges))
    ev = np.fromiter((index[b] for a, b in edges), dtype=np.uint32, count=len(edges))
    side = np.zeros(max(len(nodes), 1), dtype=np.uint8)
    if spanning_cluster:
        side[:] = _side_masks(index, auxiliary_node_attributes or {},
                              auxiliary_edge_attributes or {}, list(spanning_sides))
    return GraphSpec(nat.GRAPH_EDGES, 0, len(nodes), len(edges), eu, ev, side[:len(nodes)])


def _side_masks(index, aux_nodes, aux_edges, sides):
    """Per perc node the set of sides it is attached to (bit 0: sides[0],
    bit 1: sides[1]), following the auxiliary union-find of
    percolate/hpc.py:224-243.  If the auxiliary structure alone already joins
    both sides, node 0 is marked as touching both (the reference then reports
    a spanning cluster from its first union on)."""
    side = np.zeros(max(len(index), 1), dtype=np.uint8)
    parent = {}

    def find(x):
        parent.setdefault(x, x)
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    def union(a, b):
        ra, rb = find(a), find(b)
        if ra != rb:
            parent[ra] = rb

    roots = {}
    for s in sides:
        members = [n for n, ns in aux_nodes.items() if ns == s]
        roots[s] = ('side', s)
        for n in members:
            union(('aux', n), roots[s])
    for edge, es in aux_edges.items():
        if es not in roots:
            continue
        for node in edge:
            if node in index:
                side[index[node]] |= np.uint8(1 << sides.index(es))
            else:
                union(('aux', node), roots[es])
    if len(sides) == 2 and find(roots[sides[0]]) == find(roots[sides[1]]) and len(index):
        side[0] |= 3
    return side


# ---------------------------------------------------------------------------
# permutations
# ---------------------------------------------------------------------------
def _mt_seed_words(seed):
    """numpy legacy seeding: (words uint32, length) with length 0 for a
    scalar seed (init_genrand) and k >= 1 for an array seed (init_by_array)."""
    if seed is None:
        words = np.frombuffer(os.urandom(4 * 624), dtype=np.uint32).copy()
        return words, len(words)
    if np.ndim(seed) == 0 and not isinstance(seed, (list, tuple)):
        try:
            s = int(seed)
        except TypeError:
            raise TypeError('Cannot cast seed to an integer')
        if s < 0 or s > 2 ** 32 - 1:
            raise ValueError('Seed must be between 0 and 2**32 - 1')
        return np.array([s], dtype=np.uint32), 0
    arr = np.asarray(seed)
    if arr.size == 0:
        raise ValueError('Seed must be non-empty')
    arr = arr.astype(np.int64).ravel()
    if ((arr > 2 ** 32 - 1) | (arr < 0)).any():
        raise ValueError('Seed must be between 0 and 2**32 - 1')
    return arr.astype(np.uint32), int(arr.size)


def _run_microcanonical(spec, spanning, seeds=None, rng='numpy', key=0, run0=0, n_runs=None,
                        perms=None, with_edge=True):
    """Run the union-find kernel for several runs; returns device Records."""
    torch = nat.torch_cuda()
    lib = nat.lib_handle()
    g = spec.struct()
    if perms is not None:
        perms = np.ascontiguousarray(perms, dtype=np.uint32).reshape(-1, max(spec.M, 1) if spec.M else 0)
        n_runs = perms.shape[0]
        mode = nat.PERM_GIVEN
    elif rng == 'philox':
        mode = nat.PERM_PHILOX
        n_runs = int(n_runs if n_runs is not None else 1)
    else:
        mode = nat.PERM_MT19937
        n_runs = len(seeds)
    rec = nat.Records(spec.M + 1, n_runs, with_edge=with_edge, site=getattr(spec, 'site', False))
    ws_bytes = lib.nz_microcanonical_workspace_bytes(g, n_runs, mode)
    ws = nat.device_empty(ws_bytes)
    d_perm = d_words = d_len = None
    stride = 1
    if mode == nat.PERM_GIVEN:
        d_perm = nat.to_device(perms)
    elif mode == nat.PERM_MT19937:
        ws_list = [_mt_seed_words(s) for s in seeds]
        stride = max(max(len(w) for w, _ in ws_list), 1)
        words = np.zeros((n_runs, stride), dtype=np.uint32)
        lens = np.zeros(n_runs, dtype=np.int32)
        for i, (w, ln) in enumerate(ws_list):
            words[i, :len(w)] = w
            lens[i] = ln
        d_words = nat.to_device(words)
        d_len = nat.to_device(lens)
    recs = rec.struct()
    st = lib.nz_microcanonical(g, int(bool(spanning)), n_runs, mode, int(key), int(run0),
                               nat.ptr(d_perm), nat.ptr(d_words), nat.ptr(d_len), stride,
                               nat.ptr(ws), ws_bytes, recs, nat.stream_handle())
    nat.check(st, 'nz_microcanonical')
    rec._keep = (ws, d_perm, d_words, d_len, torch)
    return rec


def _pack_rows(rec, run, spec, spanning):
    lib = nat.lib_handle()
    dt = np.dtype(microcanonical_statistics_dtype(spanning))
    out = nat.device_empty(dt.itemsize * (spec.M + 1))
    st = lib.nz_pack_microcanonical_rows(rec.struct(), run, spec.N, spec.M, int(bool(spanning)),
                                         nat.ptr(out), nat.stream_handle())
    nat.check(st, 'nz_pack_microcanonical_rows')
    return nat.to_host(out, dt, (spec.M + 1,))


def _check_sides(spanning_cluster, spanning_sides):
    if spanning_cluster:
        if spanning_sides is None or len(spanning_sides) != 2:
            raise ValueError('Spanning cluster is to be detected, but auxiliary nodes '
                             'of less or more than 2 types (sides) given.')


# ---------------------------------------------------------------------------
# microcanonical statistics
# ---------------------------------------------------------------------------
def bond_microcanonical_statistics(
    perc_graph, num_nodes, num_edges, seed, spanning_cluster=True,
    auxiliary_node_attributes=None, auxiliary_edge_attributes=None,
    spanning_sides=None, **kwargs
):
    """Cluster statistics of every microstate n = 0..M of one run
    (percolate/hpc.py:310-404): a fresh structured array of M+1 rows with
    dtype ``microcanonical_statistics_dtype(spanning_cluster)``."""
    _check_sides(spanning_cluster, spanning_sides)
    spec = graph_spec(perc_graph, num_nodes, num_edges, spanning_cluster,
                      auxiliary_node_attributes, auxiliary_edge_attributes,
                      spanning_sides, **kwargs)
    rng = kwargs.get('rng', 'numpy')
    if rng == 'philox':
        rec = _run_microcanonical(spec, spanning_cluster, rng='philox', key=int(seed),
                                  run0=int(kwargs.get('run_id', 0)), n_runs=1)
    else:
        rec = _run_microcanonical(spec, spanning_cluster, seeds=[seed])
    return _pack_rows(rec, 0, spec, spanning_cluster)


def bond_sample_states(
    perc_graph, num_nodes, num_edges, seed, spanning_cluster=True,
    auxiliary_node_attributes=None, auxiliary_edge_attributes=None,
    spanning_sides=None, **kwargs
):
    """Generator of successive sample states (percolate/hpc.py:73-307).

    Like the reference it yields a reference to ONE internal 1-row array that
    is updated in place for every n = 0..M; the ValueError for a graph
    without two spanning sides is raised at the first ``next()``.  The whole
    run is computed by one kernel launch at that first step."""
    _check_sides(spanning_cluster, spanning_sides)
    rows = bond_microcanonical_statistics(
        perc_graph, num_nodes, num_edges, seed, spanning_cluster=spanning_cluster,
        auxiliary_node_attributes=auxiliary_node_attributes,
        auxiliary_edge_attributes=auxiliary_edge_attributes,
        spanning_sides=spanning_sides, **kwargs)
    ret = np.empty(1, dtype=rows.dtype)
    for n in range(rows.shape[0]):
        ret[0] = rows[n]
        yield ret


def bond_microcanonical_statistics_batch(
    perc_graph, num_nodes, num_edges, seeds, spanning_cluster=True,
    auxiliary_node_attributes=None, auxiliary_edge_attributes=None,
    spanning_sides=None, **kwargs
):
    """Several runs in one launch: list of structured arrays, one per seed
    (each equal to ``bond_microcanonical_statistics(seed=s, ...)``)."""
    _check_sides(spanning_cluster, spanning_sides)
    spec = graph_spec(perc_graph, num_nodes, num_edges, spanning_cluster,
                      auxiliary_node_attributes, auxiliary_edge_attributes,
                      spanning_sides, **kwargs)
    seeds = list(seeds)
    rec = _run_microcanonical(spec, spanning_cluster, seeds=seeds)
    return [_pack_rows(rec, r, spec, spanning_cluster) for r in range(len(seeds))]


# ---------------------------------------------------------------------------
# canonical statistics and averages
# ---------------------------------------------------------------------------
def bond_canonical_statistics(microcanonical_statistics, convolution_factors, **kwargs):
    """Canonical statistics of one run at one p (percolate/hpc.py:443-515):
    FP64 sums over n of factor * statistic.  A 2-D ``convolution_factors``
    (one row per p) returns one row per p from a single launch."""
    micro = microcanonical_statistics
    spanning = 'has_spanning_cluster' in micro.dtype.names
    rows = np.ascontiguousarray(micro, dtype=microcanonical_statistics_dtype(spanning)).ravel()
    M = rows.shape[0] - 1
    f = np.asarray(convolution_factors, dtype=np.float64)
    single = f.ndim == 1
    f = np.ascontiguousarray(f.reshape(-1, f.shape[-1]))
    if f.shape[1] != M + 1:
        raise ValueError('convolution_factors must have num_edges + 1 entries')
    torch = nat.torch_cuda()
    d_rows = nat.to_device(rows)
    d_f = nat.to_device(f)
    out = torch.empty(f.shape[0] * 7, dtype=torch.float64, device='cuda')
    st = nat.lib_handle().nz_canonical_statistics_rows(
        nat.ptr(d_rows), M, int(spanning), nat.ptr(d_f), f.shape[0], nat.ptr(out),
        nat.stream_handle())
    nat.check(st, 'nz_canonical_statistics_rows')
    vals = out.cpu().numpy().reshape(-1, 7)
    ret = np.empty(f.shape[0], dtype=canonical_statistics_dtype(spanning))
    if spanning:
        ret['percolation_probability'] = vals[:, 0]
    ret['max_cluster_size'] = vals[:, 1]
    ret['moments'] = vals[:, 2:]
    return ret[:1] if single else ret


def bond_initialize_canonical_averages(canonical_statistics, **kwargs):
    """(number_of_runs = 1, mean = statistic, M2 = 0) rows
    (percolate/hpc.py:561-635), same shape as the input."""
    cs = canonical_statistics
    spanning = 'percolation_probability' in cs.dtype.names
    arr = np.ascontiguousarray(cs, dtype=canonical_statistics_dtype(spanning))
    dt = np.dtype(canonical_averages_dtype(spanning))
    P = arr.size
    d_in = nat.to_device(arr)
    out = nat.device_empty(dt.itemsize * max(P, 1))
    st = nat.lib_handle().nz_initialize_canonical_averages(nat.ptr(d_in), P, int(spanning),
                                                           nat.ptr(out), nat.stream_handle())
    nat.check(st, 'nz_initialize_canonical_averages')
    return nat.to_host(out, dt, arr.shape)


def bond_reduce(row_a, row_b):
    """Merge two canonical-averages arrays (percolate/hpc.py:638-702):
    number_of_runs add, means and M2 combine by the pairwise formula.
    Associative and commutative."""
    spanning = (
        'percolation_probability_mean' in row_a.dtype.names and
        'percolation_probability_mean' in row_b.dtype.names and
        'percolation_probability_m2' in row_a.dtype.names and
        'percolation_probability_m2' in row_b.dtype.names
    )
    dt = np.dtype(canonical_averages_dtype(spanning))
    a = np.ascontiguousarray(row_a, dtype=dt)
    b = np.ascontiguousarray(row_b, dtype=dt)
    if a.shape != b.shape:
        raise ValueError('bond_reduce: shapes differ')
    d_a, d_b = nat.to_device(a), nat.to_device(b)
    out = nat.device_empty(dt.itemsize * max(a.size, 1))
    st = nat.lib_handle().nz_bond_reduce(nat.ptr(d_a), nat.ptr(d_b), a.size, int(spanning),
                                         nat.ptr(out), nat.stream_handle())
    nat.check(st, 'nz_bond_reduce')
    return nat.to_host(out, dt, a.shape)


def finalize_canonical_averages(number_of_nodes, ps, canonical_averages, alpha):
    """Means (normalised by N for strength and moments), standard deviations
    sqrt(M2 / (n - 1)) and Student-t confidence intervals at level 1 - alpha
    (percolate/hpc.py:752-834), computed on the GPU in FP64."""
    ca = canonical_averages
    spanning = ('percolation_probability_mean' in ca.dtype.names and
                'percolation_probability_m2' in ca.dtype.names)
    dt_in = np.dtype(canonical_averages_dtype(spanning))
    dt = np.dtype(finalized_canonical_averages_dtype(spanning))
    arr = np.ascontiguousarray(ca, dtype=dt_in)
    P = arr.size
    ps_arr = np.ascontiguousarray(np.broadcast_to(np.asarray(ps, dtype=np.float64), arr.shape)).ravel()
    d_in, d_ps = nat.to_device(arr), nat.to_device(ps_arr)
    out = nat.device_empty(dt.itemsize * max(P, 1))
    st = nat.lib_handle().nz_finalize_canonical_averages(
        nat.ptr(d_in), P, int(spanning), float(number_of_nodes), nat.ptr(d_ps), float(alpha),
        nat.ptr(out), nat.stream_handle())
    nat.check(st, 'nz_finalize_canonical_averages')
    return nat.to_host(out, dt, arr.shape)


bond_finalize_canonical_averages = finalize_canonical_averages
