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
