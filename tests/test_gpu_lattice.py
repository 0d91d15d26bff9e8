"""Site percolation and wrapping on the torus: GPU records against the
brute-force census (oracle/nz_census.c), bit for bit; canonical and
microcanonical reductions of the new models against the census; and the
exactly known wrapping probabilities of the square lattice at p_c."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PLANES = ('max_span', 'm0', 'm2', 'm3', 'm4_lo', 'm4_hi')


@pytest.fixture(scope='module')
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from pypercolate_gb300 import _native as nat
    nat.lib_handle()
    return nat


CASES = ([('grid', 'site', 'either', L) for L in (1, 2, 3, 8, 17)]
         + [('chain', 'site', 'either', L) for L in (1, 2, 50)]
         + [('torus', 'bond', w, L) for w in ('either', 'x', 'y', 'both') for L in (1, 2, 3, 8, 13)]
         + [('torus', 'site', w, L) for w in ('either', 'both') for L in (1, 2, 5, 11)])


@pytest.mark.parametrize('kind,model,wrap,L', CASES)
def test_records_match_census(gpu, oracle, kind, model, wrap, L):
    from pypercolate_gb300 import lattice
    site = model == 'site'
    N, steps = oracle.census_size(kind, L, site)
    runs = 6
    perms = np.stack([oracle.philox_permutation(31, r, steps) for r in range(runs)]) if steps else \
        np.zeros((runs, 0), np.uint32)
    given = lattice.sample_records(kind, L, model, wrap, perms=perms)
    philox = lattice.sample_records(kind, L, model, wrap, n_runs=runs, key=31, run0=0)
    for r in range(runs):
        want = oracle.lattice_census(kind, L, perms[r], site=site, wrap=wrap)
        for k in PLANES:
            np.testing.assert_array_equal(given[k][:, r], want[k], err_msg='%s run %d' % (k, r))
            np.testing.assert_array_equal(philox[k][:, r], want[k], err_msg='%s run %d' % (k, r))
        if steps:
            np.testing.assert_array_equal(given['edge'][1:, r], perms[r])


def test_packed_rows_of_a_site_run(gpu, oracle):
    """Reference-format rows: moments[1] counts occupied sites (n - max)."""
    from pypercolate_gb300 import lattice
    rows = lattice.microcanonical_statistics('grid', 6, model='site', key=4, run=2)
    perm = oracle.philox_permutation(4, 2, 36)
    want = oracle.lattice_census('grid', 6, perm, site=True)
    n = np.arange(37)
    mx = want['max_span'] & 0x7FFFFFFF
    np.testing.assert_array_equal(rows['n'], n)
    np.testing.assert_array_equal(rows['edge'][1:], perm)
    np.testing.assert_array_equal(rows['max_cluster_size'], mx)
    np.testing.assert_array_equal(rows['has_spanning_cluster'], want['max_span'] >> 31)
    np.testing.assert_array_equal(rows['moments'][:, 0], want['m0'])
    np.testing.assert_array_equal(rows['moments'][:, 1], n - mx)
    np.testing.assert_array_equal(rows['moments'][:, 2], want['m2'])
    # numpy-seeded order, as the reference draws its bonds
    seeded = lattice.microcanonical_statistics('torus', 5, model='site', seed=123)
    want = oracle.lattice_census('torus', 5, np.random.RandomState(123).permutation(25), site=True)
    np.testing.assert_array_equal(seeded['max_cluster_size'], want['max_span'] & 0x7FFFFFFF)
    np.testing.assert_array_equal(seeded['has_spanning_cluster'], want['max_span'] >> 31)


@pytest.mark.parametrize('kind,model,wrap,L', [('grid', 'site', 'either', 9),
                                               ('torus', 'bond', 'both', 7),
                                               ('torus', 'site', 'x', 8)])
def test_ensemble_reductions_match_census(gpu, oracle, kind, model, wrap, L):
    """Fused microcanonical sums (exact) and canonical means (FP64
    convolution) of an ensemble of the new models against the census."""
    from pypercolate_gb300.ensemble import Ensemble
    site = model == 'site'
    N, steps = oracle.census_size(kind, L, site)
    R = 40
    ps = np.linspace(0.05, 0.95, 19)
    ens = Ensemble(kind, L, ps, precision='fp64', micro=True, model=model, wrap=wrap)
    ens.run(R, key=8, run0=100)
    assert ens.errors() == 0
    q = np.zeros((R, steps + 1, 7))
    sums = np.zeros((6, steps + 1), dtype=object)
    n = np.arange(steps + 1)
    held = n if site else N
    span = np.zeros(steps + 1, np.int64)
    for r in range(R):
        c = oracle.lattice_census(kind, L, oracle.philox_permutation(8, 100 + r, steps), site=site,
                                  wrap=wrap)
        mx = (c['max_span'] & 0x7FFFFFFF).astype(np.int64)
        m4 = [(int(h) << 64) | int(lo) for h, lo in zip(c['m4_hi'], c['m4_lo'])]
        cols = [mx, c['m0'].astype(np.int64), held - mx, c['m2'], c['m3'], m4]
        for k in range(6):
            sums[k] += np.array([int(x) for x in cols[k]], dtype=object)
        span += (c['max_span'] >> 31).astype(np.int64)
        q[r, :, 0] = c['max_span'] >> 31
        q[r, :, 1] = mx
        q[r, :, 2] = c['m0']
        q[r, :, 3] = held - mx
        q[r, :, 4] = c['m2'].astype(np.float64)
        q[r, :, 5] = c['m3'].astype(np.float64)
        q[r, :, 6] = np.array([float(x) for x in m4])
    got = ens.micro_sums()
    assert got['count'] == R
    np.testing.assert_array_equal(got['span_count'], span)
    for k in range(6):
        assert list(got['sums'][k]) == list(sums[k]), k
    W = np.stack([oracle.binomial_pmf(steps, p) for p in ps])  # (P, steps+1)
    stats = np.einsum('pn,rns->rps', W, q)
    ca = ens.canonical_averages()
    assert np.all(ca['number_of_runs'] == R)
    np.testing.assert_allclose(ca['percolation_probability_mean'], stats[:, :, 0].mean(0),
                               rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(ca['max_cluster_size_mean'], stats[:, :, 1].mean(0), rtol=1e-9)
    np.testing.assert_allclose(ca['moments_mean'], stats[:, :, 2:].mean(0), rtol=1e-9, atol=1e-9)


# Wrapping probabilities of critical bond percolation on the square torus
# (L -> infinity): Pinson, J. Stat. Phys. 75, 1167 (1994); the values quoted
# by Newman & Ziff, Phys. Rev. E 64, 016706 (2001), Table I.
R_EXACT = {'either': 0.690473725, 'x': 0.521058290, 'both': 0.351642855}


@pytest.mark.parametrize('model,p_c', [('bond', 0.5), ('site', 0.59274621)])
def test_critical_wrapping_probabilities(gpu, model, p_c):
    """Universal wrapping probabilities at p_c on a 128 x 128 torus, 40,000
    runs: within 5 standard errors plus a finite-size allowance of 0.01
    (NZ 2001 find corrections of order L^-2 for bond and small ones for site)."""
    from pypercolate_gb300.ensemble import Ensemble
    R = 40000
    for wrap, exact in R_EXACT.items():
        ens = Ensemble('torus', 128, np.array([p_c]), precision='fp64', micro=False,
                       model=model, wrap=wrap)
        ens.run(R, key=2024, run0=0)
        got = float(ens.canonical_averages()['percolation_probability_mean'][0])
        se = np.sqrt(exact * (1 - exact) / R)
        assert abs(got - exact) < 5 * se + 0.01, (model, wrap, got, exact)
