"""GPU ensemble path (batched runs, fused reductions, banded convolution)
against the CPU oracle on the same Philox runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from pypercolate_gb300 import _native as nat
    nat.lib_handle()
    return nat


def _oracle_canonical(oracle, kind, L, key, run0, R, ps):
    """Per-run canonical values with the same banded FP64 weights the GPU
    computes, merged by the pairwise formula (exact oracle pipeline)."""
    return oracle.ensemble_canonical(kind, L, key, run0, R, ps, n_threads=8)


@pytest.mark.parametrize('kind,L', [(0, 8), (0, 24), (1, 500)])
def test_ensemble_fp64_matches_oracle(gpu, oracle, kind, L):
    from pypercolate_gb300.ensemble import Ensemble
    ps = np.linspace(0.0, 1.0, 41)
    R = 300
    ens = Ensemble('grid' if kind == 0 else 'chain', L, ps, precision='fp64', micro=False)
    ens.run(R, key=77, run0=0)
    ca = ens.canonical_averages()
    mean, m2 = _oracle_canonical(oracle, kind, L, 77, 0, R, ps)
    assert np.all(ca['number_of_runs'] == R)
    np.testing.assert_allclose(ca['percolation_probability_mean'], mean[:, 0], rtol=1e-9, atol=1e-13)
    np.testing.assert_allclose(ca['max_cluster_size_mean'], mean[:, 1], rtol=1e-9)
    np.testing.assert_allclose(ca['moments_mean'], mean[:, 2:], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(ca['max_cluster_size_m2'], m2[:, 1], rtol=1e-7, atol=1e-6)
    np.testing.assert_allclose(ca['moments_m2'], m2[:, 2:], rtol=1e-7, atol=1e-6)


@pytest.mark.parametrize('precision', ['fp32', 'tf32x3'])
def test_ensemble_fp32_error_budget(gpu, oracle, precision):
    """FP32 convolution (SIMT, or 3xTF32 on the tensor cores): spanning
    probability and percolation strength within 1e-6 absolute of the FP64
    oracle pipeline; moments within 2e-6 relative."""
    from pypercolate_gb300.ensemble import Ensemble
    ps = np.linspace(0.0, 1.0, 101)
    L, R = 32, 256
    ens = Ensemble('grid', L, ps, precision=precision, micro=False)
    ens.run(R, key=3, run0=0)
    ca = ens.canonical_averages()
    mean, _ = _oracle_canonical(oracle, 0, L, 3, 0, R, ps)
    N = L * L
    assert np.max(np.abs(ca['percolation_probability_mean'] - mean[:, 0])) < 1e-6
    assert np.max(np.abs(ca['max_cluster_size_mean'] - mean[:, 1]) / N) < 1e-6
    rel = np.abs(ca['moments_mean'] - mean[:, 2:]) / np.maximum(np.abs(mean[:, 2:]), 1e-30)
    assert np.max(rel) < 2e-6


def test_ensemble_accumulates_across_calls(gpu):
    from pypercolate_gb300.ensemble import Ensemble
    ps = np.linspace(0.2, 0.8, 13)
    a = Ensemble('grid', 12, ps, precision='fp64', micro=True)
    a.run(100, key=1, run0=0).run(150, key=1, run0=100)
    b = Ensemble('grid', 12, ps, precision='fp64', micro=True)
    b.run(250, key=1, run0=0)
    ca, cb = a.canonical_averages(), b.canonical_averages()
    assert np.all(ca['number_of_runs'] == 250)
    for k in ('percolation_probability_mean', 'max_cluster_size_mean', 'moments_mean'):
        np.testing.assert_allclose(ca[k], cb[k], rtol=1e-12, atol=1e-14)
    for k in ('max_cluster_size_m2', 'moments_m2'):
        np.testing.assert_allclose(ca[k], cb[k], rtol=1e-9, atol=1e-9)
    sa, sb = a.micro_sums(), b.micro_sums()
    assert sa['count'] == sb['count'] == 250
    assert np.array_equal(sa['span_count'], sb['span_count'])
    assert (sa['sums'] == sb['sums']).all()
    np.testing.assert_allclose(sa['m2'], sb['m2'], rtol=1e-9, atol=1e-6)


@pytest.mark.parametrize('L,R,window', [(10, 97, 0), (10, 97, 37), (128, 9, 0)])
def test_fused_micro_reductions_exact(gpu, oracle, L, R, window):
    """Exact per-n sums over runs of max and every moment (Python ints), the
    spanning counts, and M2 within 1e-9, against the oracle's exact integers
    (L = 128: the m3 and m4 squares run scaled by 2^-5 and 2^-20)."""
    from pypercolate_gb300.ensemble import Ensemble
    ens = Ensemble('grid', L, [0.5], precision='fp64', micro=True, window=window)
    ens.run(R, key=11, run0=5)
    assert ens.errors() == 0  # no run's union-find state came out corrupt
    got = ens.micro_sums()
    M = 2 * L * (L - 1)
    N = L * L
    vals = np.zeros((6, R, M + 1), dtype=object)
    span = np.zeros(M + 1, dtype=np.int64)
    for r in range(R):
        run = oracle.lattice_run(0, L, oracle.philox_permutation(11, 5 + r, M))
        lo = run['moments_u64'].astype(object)
        hi = run['moments_hi'].astype(object)
        exact = lo + hi * (1 << 64)
        vals[0, r] = run['max'].astype(object)
        vals[1, r] = exact[:, 0]
        vals[2, r] = N - run['max'].astype(object)
        vals[3, r] = exact[:, 2]
        vals[4, r] = exact[:, 3]
        vals[5, r] = exact[:, 4]
        span += run['span']
    assert got['count'] == R
    assert np.array_equal(got['span_count'], span.astype(np.uint64))
    assert (got['sums'] == vals.sum(axis=1)).all()
    fl = vals.astype(np.float64)
    m2 = ((fl - fl.mean(axis=1, keepdims=True)) ** 2).sum(axis=1)
    np.testing.assert_allclose(got['m2'], m2, rtol=1e-9, atol=1e-6)


def test_microcanonical_averages_semantics(gpu, oracle):
    """Classic microcanonical averages (percolate/percolate.py:450-705)."""
    from pypercolate_gb300.ensemble import Ensemble
    L, R, alpha = 6, 60, 0.3173
    ens = Ensemble('grid', L, [0.5], precision='fp64', micro=True)
    ens.run(R, key=2, run0=0)
    got = ens.microcanonical_averages(alpha)
    M, N = 2 * L * (L - 1), L * L
    mx, sp, mom = [], [], []
    for r in range(R):
        run = oracle.lattice_run(0, L, oracle.philox_permutation(2, r, M))
        mx.append(run['max'].astype(np.float64))
        sp.append(run['span'])
        mom.append(run['moments_f64'])
    mx, sp, mom = np.array(mx), np.array(sp), np.array(mom)
    mean, lo, hi = oracle.microcanonical_average_spanning(sp.sum(0), R, alpha)
    np.testing.assert_allclose(got['spanning_cluster'], mean, rtol=1e-12)
    np.testing.assert_allclose(got['spanning_cluster_ci'][:, 0], lo, rtol=1e-8, atol=1e-14)
    np.testing.assert_allclose(got['spanning_cluster_ci'][:, 1], hi, rtol=1e-8)
    mlo, mhi = oracle.microcanonical_average_normal(mx.mean(0), mx.std(0, ddof=1), R, alpha)
    np.testing.assert_allclose(got['max_cluster_size'], mx.mean(0) / N, rtol=1e-12)
    np.testing.assert_allclose(got['max_cluster_size_ci'][:, 0], mlo / N, rtol=1e-9)
    np.testing.assert_allclose(got['max_cluster_size_ci'][:, 1], mhi / N, rtol=1e-9)
    for k in range(5):
        np.testing.assert_allclose(got['moments'][k], mom[:, :, k].mean(0) / N, rtol=1e-12)
        klo, khi = oracle.microcanonical_average_normal(mom[:, :, k].mean(0),
                                                        mom[:, :, k].std(0, ddof=1), R, alpha)
        np.testing.assert_allclose(got['moments_ci'][k][:, 0], klo / N, rtol=1e-8, atol=1e-12)


def test_finalized_ensemble(gpu):
    """Ensemble.finalized() == finalize_canonical_averages(canonical_averages())."""
    from pypercolate_gb300.ensemble import Ensemble
    from pypercolate_gb300 import hpc
    import scipy.stats
    ps = np.linspace(0.3, 0.7, 9)
    ens = Ensemble('grid', 16, ps, precision='fp64', micro=False)
    ens.run(200, key=9)
    fin = ens.finalized(0.05)
    ca = ens.canonical_averages()
    n = ca['number_of_runs'].astype(np.float64)
    std = np.sqrt(ca['max_cluster_size_m2'] / (n - 1)) / 256
    np.testing.assert_allclose(fin['percolation_strength_std'], std, rtol=1e-12)
    lo, hi = scipy.stats.t.interval(0.95, df=n - 1, loc=fin['percolation_strength_mean'],
                                    scale=std / np.sqrt(n))
    np.testing.assert_allclose(fin['percolation_strength_ci'][:, 0], lo, rtol=1e-10)
    np.testing.assert_allclose(fin['percolation_strength_ci'][:, 1], hi, rtol=1e-10)
    assert np.all(fin['p'] == ps)


@pytest.mark.parametrize('kind,L,model,wrap,R,window', [
    ('grid', 32, 'bond', 'either', 300, 0),
    ('grid', 32, 'bond', 'either', 300, 97),     # 21 windows, ragged last one
    ('grid', 340, 'bond', 'either', 3, 0),       # m4 with its high-word plane
    ('grid', 20, 'site', 'either', 257, 0),
    ('torus', 24, 'bond', 'both', 129, 0),
    ('torus', 16, 'site', 'x', 130, 0),
    ('chain', 3000, 'bond', 'either', 200, 0),
    ('chain', 1, 'bond', 'either', 5, 0),        # M = 0: one row
])
def test_tensor_core_convolution_matches_fp64(gpu, kind, L, model, wrap, R, window):
    """The tcgen05 3xTF32 convolution against the FP64 convolution of the
    same records (same Philox runs): spanning and max / N within 1e-6
    absolute, moments within 2e-6 relative; run counts that are not a
    multiple of the 128-run tile, 41 probabilities (a ragged 32-p tile), and
    windows that cut the bands."""
    from pypercolate_gb300.ensemble import Ensemble
    ps = np.linspace(0.0, 1.0, 41)
    got = {}
    for prec in ('fp64', 'tf32x3'):
        ens = Ensemble(kind, L, ps, precision=prec, micro=False, model=model, wrap=wrap, window=window)
        ens.run(R, key=5, run0=11)
        assert ens.errors() == 0
        ca = ens.canonical_averages()
        assert np.all(ca['number_of_runs'] == R)
        got[prec] = (ca['percolation_probability_mean'], ca['max_cluster_size_mean'], ca['moments_mean'])
    N = ens.N
    (s64, x64, m64), (s32, x32, m32) = got['fp64'], got['tf32x3']
    assert np.max(np.abs(s32 - s64)) < 1e-6
    assert np.max(np.abs(x32 - x64)) / N < 1e-6
    big = np.abs(m64) > 1e-12
    assert np.all(np.abs(m32 - m64)[~big] < 1e-12)
    if big.any():
        assert np.max(np.abs(m32 - m64)[big] / np.abs(m64[big])) < 2e-6


@pytest.mark.parametrize('precision', ['fp32', 'tf32x3'])
def test_convolution_without_spanning_statistic(gpu, precision):
    """spanning=False: no spanning fields, and the max and moment curves of
    the FP32 paths (the tcgen05 kernel skips its spanning CTAs) within the
    error budget of the FP64 path on the same runs."""
    from pypercolate_gb300.ensemble import Ensemble
    ps = np.linspace(0.0, 1.0, 37)
    got = {}
    for prec in ('fp64', precision):
        ens = Ensemble('grid', 24, ps, spanning=False, precision=prec, micro=False)
        ens.run(150, key=9, run0=3)
        ca = ens.canonical_averages()
        assert 'percolation_probability_mean' not in ca.dtype.names
        got[prec] = (ca['max_cluster_size_mean'], ca['moments_mean'])
    (x64, m64), (x32, m32) = got['fp64'], got[precision]
    assert np.max(np.abs(x32 - x64)) / (24 * 24) < 1e-6
    big = np.abs(m64) > 1e-12
    assert np.max(np.abs(m32 - m64)[big] / np.abs(m64[big])) < 2e-6


@pytest.mark.parametrize('L', [339, 340])
def test_m4_high_plane_either_side_of_its_bound(gpu, oracle, L):
    """Up to N = 115,000 sites the ensemble leaves out the m4 high-word
    plane (sum' s^4 < 2^64 there); L = 339 (N = 114,921) runs without it,
    L = 340 (N = 115,600) with it.  Both give the oracle's exact sums, and
    the M2 of m3 and m4 -- squared as scaled FP32 pairs, scale 2^-11 and
    2^-28 at these sizes -- within 1e-9 of the exact integer M2."""
    from pypercolate_gb300.ensemble import Ensemble
    R = 3
    ens = Ensemble('grid', L, [0.5], precision='fp64', micro=True)
    ens.run(R, key=21, run0=0)
    got = ens.micro_sums()
    M = 2 * L * (L - 1)
    runs = [oracle.lattice_run(0, L, oracle.philox_permutation(21, r, M)) for r in range(R)]
    exact = {k: [run['moments_u64'][:, k].astype(object) + run['moments_hi'][:, k].astype(object) * (1 << 64)
                 for run in runs] for k in (3, 4)}
    assert (got['sums'][5] == sum(exact[4])).all()
    for k, stat in ((3, 4), (4, 5)):
        xs = exact[k]
        s1 = sum(xs)
        s2 = sum(x * x for x in xs)
        # R * M2 = R * sum x^2 - (sum x)^2, exact in integers
        m2 = np.array([float(a * R - b * b) / R for a, b in zip(s2, s1)])
        np.testing.assert_allclose(got['m2'][stat], m2, rtol=1e-9, atol=1e-6, err_msg='m%d' % k)


def test_chain_spanning_is_exactly_p_to_the_bonds(gpu):
    """A chain spans only once every bond is in, so each run's canonical
    spanning value is the binomial weight of n = M: p^M, with zero spread."""
    from pypercolate_gb300.ensemble import Ensemble
    l = 100
    ps = np.array([0.9, 0.97, 0.999])
    ens = Ensemble('chain', l, ps, precision='fp64', micro=False)
    ens.run(500, key=3, run0=0)
    ca = ens.canonical_averages()
    np.testing.assert_allclose(ca['percolation_probability_mean'], ps ** (l - 1), rtol=1e-12)
    assert np.all(np.abs(ca['percolation_probability_m2']) < 1e-20)


def test_square_grid_spans_half_the_time_at_one_half(gpu):
    """Bond percolation on the square lattice is self-dual at p = 1/2, so the
    top-to-bottom spanning probability of an L x L grid tends to 1/2; at
    L = 128 over 20,000 runs it lies within 5 standard errors plus 0.02 of
    it.  (A biased bond order -- e.g. a permutation over-representing some
    rows early -- moves it well away.)"""
    from pypercolate_gb300.ensemble import Ensemble
    R = 20000
    ens = Ensemble('grid', 128, np.array([0.5]), precision='fp64', micro=False)
    ens.run(R, key=99, run0=0)
    got = float(ens.canonical_averages()['percolation_probability_mean'][0])
    assert abs(got - 0.5) < 5 * np.sqrt(0.25 / R) + 0.02, got


@pytest.mark.parametrize('precision', ['fp32', 'tf32x3'])
def test_tuned_launch_shapes_give_the_same_results(gpu, precision):
    """Every launch shape the autotuner can pick (runs per union-find CTA,
    probability tiles of the two FP32 convolutions, run-reduction slices,
    record window and its tapered schedule) gives the same ensemble: exact micro sums equal, canonical
    curves equal to FP32 rounding of the per-run sums (1e-6 relative)."""
    from pypercolate_gb300.ensemble import Ensemble
    ps = np.linspace(0.0, 1.0, 61)
    L, R = 20, 700
    ref = Ensemble('grid', L, ps, precision=precision, micro=True)
    ref.run(R, key=21, run0=3)
    want = ref.canonical_averages()
    for tuning, window in (({'uf_block': 64, 'conv_tile': 16, 'm2_tile': 8, 'reduce_slices': 256}, 97),
                           ({'uf_block': 32, 'conv_tile': 16, 'm2_tile': 16, 'reduce_slices': 1,
                             'taper': 1}, 0),
                           ({'taper': 1}, 300)):
        ens = Ensemble('grid', L, ps, precision=precision, micro=True, window=window, tuning=tuning)
        ens.run(R, key=21, run0=3)
        assert ens.errors() == 0
        got = ens.canonical_averages()
        for k in ('percolation_probability_mean', 'max_cluster_size_mean', 'moments_mean'):
            np.testing.assert_allclose(got[k], want[k], rtol=1e-6, atol=1e-9)
        a, b = ens.micro_sums(), ref.micro_sums()
        assert a['count'] == b['count'] == R
        assert (a['sums'] == b['sums']).all()
        assert np.array_equal(a['span_count'], b['span_count'])
