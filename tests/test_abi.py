"""CPU checks of the C ABI library and the host-side logic (no GPU calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import REPO


def _declared_functions():
    src = open(os.path.join(REPO, 'include', 'nz_gb300.h')).read()
    src = re.sub(r'/\*.*?\*/', '', src, flags=re.S)
    names = re.findall(r'\b(nz_[a-z0-9_]+)\s*\(', src)
    return sorted(set(names))


@pytest.fixture(scope='module')
def lib():
    from pypercolate_gb300 import build
    build.build()
    return ctypes.CDLL(build.LIB)


def test_library_exports_every_declared_symbol(lib):
    names = _declared_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name


def test_bindings_cover_header():
    from pypercolate_gb300 import _native
    assert set(_declared_functions()) == set(_native.EXPORTED)


def test_host_only_entry_points(lib):
    from pypercolate_gb300 import _native as nat
    L = nat.lib_handle()
    assert b'sm_103a' in L.nz_version()
    assert nat.graph_size(nat.make_graph(nat.GRAPH_GRID2D, 256)) == (65536, 130560)
    assert nat.graph_size(nat.make_graph(nat.GRAPH_CHAIN1D, 1)) == (1, 0)
    with pytest.raises(ValueError):
        nat.graph_size(nat.make_graph(nat.GRAPH_CHAIN1D, 0))
    with pytest.raises(nat.NzError):
        nat.graph_size(nat.make_graph(nat.GRAPH_GRID2D, 2048))
    g = nat.make_graph(nat.GRAPH_GRID2D, 256)
    assert L.nz_microcanonical_workspace_bytes(g, 10, nat.PERM_PHILOX) >= 10 * 65536 * 4
    assert L.nz_ensemble_workspace_bytes(g, 100, 1001, 0) > 100 * 65536 * 4
    # the bench's ensemble: node words (26.2 GB), two record windows sized
    # for at most ~32 GiB each (rows counted at 36 B per record; 26 B at
    # L = 256: narrow m0 and m2, no m4 high words) and the per-run canonical
    # accumulators (5.6 GB) -- about 81 GB of HBM
    ws = L.nz_ensemble_workspace_bytes(g, 100000, 1001, 0)
    records = ws - 100000 * 65536 * 4 - 100000 * 1001 * 7 * 8
    assert 2 * 32 * 2**30 * 26 / 36 * 0.99 < records < 2 * 32 * 2**30 * 26 / 36 * 1.01
    assert L.nz_binomial_band_cap(130560, 80.0) > 2 * 12 * 181


def test_lattice_extension_kinds(lib):
    """Kind flags: torus sizes, site model (one step per site), rejected mixes."""
    from pypercolate_gb300 import _native as nat
    from pypercolate_gb300.ensemble import lattice_kind
    L = nat.lib_handle()
    size = lambda kind, n: nat.graph_size(nat.make_graph(kind, n))  # noqa: E731
    assert size(nat.GRAPH_TORUS2D, 5) == (25, 50)
    assert size(nat.GRAPH_TORUS2D | nat.WRAP['both'], 1) == (1, 2)
    assert size(nat.GRAPH_GRID2D | nat.MODEL_SITE, 5) == (25, 25)
    assert size(nat.GRAPH_CHAIN1D | nat.MODEL_SITE, 7) == (7, 7)
    assert size(nat.GRAPH_TORUS2D | nat.MODEL_SITE | nat.WRAP['x'], 4) == (16, 16)
    for bad in (nat.GRAPH_GRID2D | nat.WRAP['x'], nat.GRAPH_CHAIN1D | nat.WRAP['y'],
                nat.GRAPH_TORUS2D | 0x800, nat.GRAPH_GRID2D | 0x1000):
        with pytest.raises(ValueError):
            size(bad, 4)
    with pytest.raises(ValueError):  # site percolation needs an implicit lattice
        nat.graph_size(nat.make_graph(nat.GRAPH_EDGES | nat.MODEL_SITE, 0, 3, 2))
    with pytest.raises(nat.NzError):
        size(nat.GRAPH_TORUS2D, 1449)  # 1449^2 > 2^21 nodes
    # torus cells are 16 bytes per site
    g = nat.make_graph(nat.GRAPH_TORUS2D, 64)
    assert L.nz_microcanonical_workspace_bytes(g, 10, nat.PERM_PHILOX) >= 10 * 4096 * 16
    assert lattice_kind('torus', 'site', 'both') == nat.GRAPH_TORUS2D | nat.MODEL_SITE | 0x600
    with pytest.raises(ValueError):
        lattice_kind('grid', 'bond', 'x')
    with pytest.raises(ValueError):
        lattice_kind('torus', 'sites')


def test_dtypes_match_reference_layout():
    from pypercolate_gb300 import hpc
    assert np.dtype(hpc.microcanonical_statistics_dtype(True)).itemsize == 53
    assert np.dtype(hpc.microcanonical_statistics_dtype(False)).itemsize == 52
    assert np.dtype(hpc.canonical_statistics_dtype(True)).itemsize == 56
    assert np.dtype(hpc.canonical_averages_dtype(True)).itemsize == 116
    assert np.dtype(hpc.canonical_averages_dtype(False)).itemsize == 100
    assert np.dtype(hpc.finalized_canonical_averages_dtype(True)).itemsize == 244
    assert np.dtype(hpc.finalized_canonical_averages_dtype(False)).itemsize == 212
    for sc in (True, False):
        names = np.dtype(hpc.finalized_canonical_averages_dtype(sc)).names
        assert ('percolation_probability_ci' in names) == sc
    assert hpc.bond_finalize_canonical_averages is hpc.finalize_canonical_averages


def test_seed_parsing_matches_numpy_rules():
    from pypercolate_gb300 import hpc
    w, n = hpc._mt_seed_words(42)
    assert n == 0 and w[0] == 42
    w, n = hpc._mt_seed_words([1, 2, 3])
    assert n == 3 and list(w) == [1, 2, 3]
    with pytest.raises(ValueError):
        hpc._mt_seed_words(-1)
    with pytest.raises(ValueError):
        hpc._mt_seed_words(2 ** 32)
    with pytest.raises(ValueError):
        hpc._mt_seed_words([])


def test_lattice_standin_matches_networkx():
    nx = pytest.importorskip('networkx')
    from pypercolate_gb300.percolate import LatticeGraph, percolation_graph
    from pypercolate_gb300 import percolate as P
    for L in (1, 2, 3, 5):
        g = P.spanning_2d_grid(L)
        pg = percolation_graph(g)
        sg = LatticeGraph('grid', L)
        assert list(pg['perc_graph'].edges()) == sg.edges()
        assert list(pg['perc_graph'].nodes()) == sg.perc().nodes()
        assert pg['num_edges'] == 2 * L * (L - 1)
    for L in (1, 2, 7):
        pg = percolation_graph(P.spanning_1d_chain(L))
        assert list(pg['perc_graph'].edges()) == LatticeGraph('chain', L).edges()


def test_graph_spec_side_masks():
    nx = pytest.importorskip('networkx')
    from pypercolate_gb300 import hpc
    from pypercolate_gb300.percolate import percolation_graph
    from conftest import load_golden
    z = load_golden('kat_3x3.npz')
    g = nx.Graph()
    g.add_nodes_from(range(9))
    g.add_edges_from([(i, i + j) for i in [1, 4, 7] for j in [-1, 1]])
    g.add_edges_from([(i, i + j) for i in [3, 4, 5] for j in [-3, 3]])
    g.add_nodes_from(range(9, 12), span=0)
    g.add_nodes_from(range(12, 15), span=1)
    g.add_edges_from([(0, 9), (3, 10), (6, 11)], span=0)
    g.add_edges_from([(2, 12), (5, 13), (8, 14)], span=1)
    pg = percolation_graph(g)
    spec = hpc.graph_spec(**pg)
    assert spec.kind == 2
    assert np.array_equal(spec.eu, z['eu']) and np.array_equal(spec.ev, z['ev'])
    assert np.array_equal(spec.side, z['side'])
    # implicit lattice for the package's own builders
    from pypercolate_gb300 import percolate as P
    spec = hpc.graph_spec(**percolation_graph(P.spanning_2d_grid(8)))
    assert spec.kind == 0 and spec.M == 112
    # non-spanning on the same graph falls back to the explicit (L+2) x L grid
    spec = hpc.graph_spec(**percolation_graph(P.spanning_2d_grid(4), spanning_cluster=False))
    assert spec.kind == 2 and spec.N == 24


def test_log_uniform_thresholds():
    from pypercolate_gb300.mix import log_uniform_thresholds
    thr = log_uniform_thresholds(8, 512)
    assert thr[0] == 0 and len(thr) == 505
    assert np.all(np.diff(thr.astype(np.int64)) >= 0)
    rng = np.random.default_rng(0)
    u = rng.integers(0, 2 ** 32, size=400000, dtype=np.uint64)
    L = 8 + np.searchsorted(thr.astype(np.uint64), u, side='right') - 1
    assert L.min() == 8 and L.max() == 512
    # log-uniform: median at sqrt(8 * 512) = 64, quartiles at 22.6 and 181
    assert abs(np.mean(L <= 64) - 0.5) < 0.01
    assert abs(np.mean(L <= 22) - 0.25) < 0.02
    assert np.array_equal(log_uniform_thresholds(5, 5), [0])


def test_surrogate_features():
    """Host-side inputs of the surrogate: (p, 1/L, one-hot, scaling variable)."""
    from pypercolate_gb300 import surrogate as S
    ps = np.array([0.0, 0.5, 0.6, 1.0])
    x = S.features(ps, 16, 'grid')
    assert x.shape == (4, S.WIDTHS[0]) and x.dtype == np.float32
    np.testing.assert_allclose(x[:, 0], ps)
    np.testing.assert_allclose(x[:, 1], 1 / 16)
    assert np.all(x[:, 2] == 1) and np.all(x[:, 3] == 0)
    np.testing.assert_allclose(x[:, 4], np.arcsinh((ps - 0.5) * 8.0), rtol=1e-6)  # 16^(3/4) = 8
    # the same (p - p_c) L^(1/nu) at two sizes gives the same scaling input
    a = S.features([0.5 + 0.1 / 8], 16, 'grid')[0, 4]
    b = S.features([0.5 + 0.1 / 64], 256, 'grid')[0, 4]
    assert abs(a - b) < 1e-6
    c = S.features([1.0 - 3.0 / 1024], 1024, 'chain')
    assert c[0, 3] == 1 and abs(c[0, 4] - np.arcsinh(-3.0)) < 1e-6


def test_surrogate_target_transforms():
    """The units the surrogate learns in: logit spanning probability (clipped
    to [1e-6, 1 - 1e-6]), log strength, log susceptibility as is; `curves`
    inverts them, and `train_se` carries the standard errors over to first
    order (at most one logit unit where pi is within its error of 0 or 1)."""
    from pypercolate_gb300 import surrogate as S
    y = np.array([[0.0, 1e-3, 1.0], [0.5, 0.2, 2.0], [1.0, 0.9, -3.0], [0.25, 1e-13, 0.5]])
    se = np.array([[1e-4, 1e-6, 1e-3], [5e-3, 1e-3, 1e-3], [1e-4, 1e-4, 1e-2], [1e-2, 1e-6, 1e-3]])
    t = S.train_targets(y)
    np.testing.assert_allclose(t[:, 0], [np.log(1e-6 / (1 - 1e-6)), 0.0, np.log((1 - 1e-6) / 1e-6),
                                         np.log(1 / 3)], rtol=1e-9)
    np.testing.assert_allclose(t[:, 1], np.log([1e-3, 0.2, 0.9, S.STRENGTH_FLOOR]), rtol=1e-12)
    np.testing.assert_array_equal(t[:, 2], y[:, 2])
    back = S.curves(t)
    np.testing.assert_allclose(back[[1, 3], 0], y[[1, 3], 0], rtol=1e-12)
    np.testing.assert_allclose(back[[0, 2], 0], [1e-6, 1 - 1e-6], rtol=1e-9)  # clipped
    np.testing.assert_allclose(back[:3, 1], y[:3, 1], rtol=1e-12)
    s = S.train_se(y, se)
    np.testing.assert_allclose(s[:, 0], [1.0, 0.02, 1.0, 1e-2 / 0.1875], rtol=1e-12)
    np.testing.assert_allclose(s[:, 1], [1e-3, 5e-3, 1e-4 / 0.9, 1e-6 / S.STRENGTH_FLOOR], rtol=1e-12)
    np.testing.assert_array_equal(s[:, 2], se[:, 2])
    # large logits do not overflow on the way back
    assert np.all(np.isfinite(S.curves(np.array([[800.0, 0.0, 0.0], [-800.0, 0.0, 0.0]]))))


def test_precision_codes():
    """Ensemble precision names in the order of nz_ensemble's conv_precision
    codes (0 FP64, 1 FP32 SIMT, 2 3xTF32 tensor cores)."""
    from pypercolate_gb300.ensemble import PRECISIONS
    assert PRECISIONS == ('fp64', 'fp32', 'tf32x3')


def test_mix_workspace_by_reduction(lib):
    """The two reductions of nz_mix need different scratch: per-run
    checkpoint records (36 B per run and checkpoint) or per-lattice sums
    (27 words per lattice and checkpoint); an unknown reduction is refused."""
    from pypercolate_gb300 import _native as nat
    L = nat.lib_handle()
    spec = nat.NzMixSpec()
    spec.grid_min, spec.grid_max, spec.chain_min, spec.chain_max = 8, 64, 100, 2000
    spec.chain_share, spec.checkpoints = 2 ** 31, 64
    runs, threads = 50000, 4096
    classes = (64 - 8 + 1) + (2000 - 100 + 1)
    spec.reduction = 0
    rec = L.nz_mix_workspace_bytes(ctypes.byref(spec), runs, threads)
    spec.reduction = 1
    fused = L.nz_mix_workspace_bytes(ctypes.byref(spec), runs, threads)
    assert rec - fused == pytest.approx(runs * 64 * 36 - classes * 64 * 27 * 8, abs=4096)
    spec.reduction = 2
    assert L.nz_mix_workspace_bytes(ctypes.byref(spec), runs, threads) == 0


def test_beta_quantile_host_restatement_matches_scipy():
    """The Beta quantiles of the microcanonical spanning bounds
    (csrc/nz_math.cuh, host-compiled here): closed forms for Beta(1, b) and
    Beta(a, 1), Newton from the skewness-corrected start elsewhere -- against
    scipy.stats.beta.ppf over the run counts and k an ensemble produces."""
    import shutil
    import subprocess
    import tempfile
    st = pytest.importorskip('scipy.stats')
    cxx = shutil.which('g++')
    if cxx is None:
        pytest.skip('no host C++ compiler')
    src = ('#include <cmath>\n#define __host__\n#define __device__\nusing std::isfinite;\n'
           '#include "%s"\n'
           'extern "C" void bq(const double *q, const double *a, const double *b, double *o, int n)'
           ' { for (int i = 0; i < n; ++i) o[i] = nz::beta_quantile(q[i], a[i], b[i]); }\n'
           % os.path.join(REPO, 'pypercolate_gb300', 'csrc', 'nz_math.cuh'))
    with tempfile.TemporaryDirectory() as d:
        with open(os.path.join(d, 'bq.cpp'), 'w') as f:
            f.write(src)
        so = os.path.join(d, 'bq.so')
        subprocess.run([cxx, '-O2', '-std=c++17', '-shared', '-fPIC', os.path.join(d, 'bq.cpp'), '-o', so],
                       check=True)
        fn = ctypes.CDLL(so).bq
        rng = np.random.default_rng(5)
        q, a, b = [], [], []
        for R in (1, 2, 60, 1000, 100000):
            ks = np.unique(np.concatenate([np.arange(0, min(R, 20) + 1), R - np.arange(0, min(R, 20) + 1),
                                           rng.integers(0, R + 1, 400)]))
            for qq in (0.025, 0.975, 0.15865, 0.84135):
                q += [qq] * len(ks)
                a += list(ks + 1.0)
                b += list(R - ks + 1.0)
        q, a, b = (np.array(v, dtype=np.float64) for v in (q, a, b))
        out = np.empty_like(q)
        P = ctypes.POINTER(ctypes.c_double)
        fn(q.ctypes.data_as(P), a.ctypes.data_as(P), b.ctypes.data_as(P), out.ctypes.data_as(P),
           ctypes.c_int(len(q)))
    np.testing.assert_allclose(out, st.beta.ppf(q, a, b), rtol=1e-9)


def test_ensemble_tuner_candidates():
    """The main path's autotuner: the library's defaults first, then one
    launch-shape change at a time (no duplicates, windows within [256, M+1]),
    and the combination of every change that beat the defaults."""
    from pypercolate_gb300 import autotune as A
    M, runs = 130560, 100000
    w = A.default_window(M, runs)
    assert w == int(32.0 * 2 ** 30 / (runs * 36))
    assert A.default_window(100, runs) == 101 and A.default_window(10 ** 7, 10 ** 8) == 256
    cands = A.ensemble_candidates(M, runs)
    base = cands[0]
    assert base == {'uf_block': 128, 'm2_tile': 8, 'conv_tile': 8, 'taper': 0, 'reduce_slices': 64,
                    'window': w}
    assert len(cands) == len({tuple(sorted(c.items())) for c in cands})
    for c in cands[1:]:
        assert sum(c[k] != base[k] for k in base) == 1
        assert 256 <= c['window'] <= M + 1
    table = [(base, 100.0), (dict(base, uf_block=64), 99.0), (dict(base, m2_tile=16), 101.0),
             (dict(base, window=w // 2), 98.0), (dict(base, window=3 * w // 2), 99.5)]
    combo = A.combined_candidate(table)
    assert combo == dict(base, uf_block=64, window=w // 2)
    assert A.combined_candidate([(base, 1.0), (dict(base, taper=1), 2.0)]) == base
    # a lattice with fewer rows than the smallest window: every window is M + 1
    small = A.ensemble_candidates(180, runs)
    assert {c['window'] for c in small} == {181}
