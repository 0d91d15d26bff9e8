"""The CPU oracle against the reference's own golden vectors and against
fixtures recorded from the reference (tests/golden/make_golden.py)."""
import hashlib

import numpy as np
import pytest

from conftest import golden_cases, load_golden


def test_philox_known_answers(oracle):
    # Random123 known-answer vectors for philox4x32-10 (Salmon et al. 2011)
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
        ([0xffffffff] * 4, [0xffffffff] * 2,
         [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
        ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
         [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
    ]
    for ctr, key, want in kat:
        assert list(oracle.philox4x32_10(ctr, key)) == want


@pytest.mark.parametrize('M', [0, 1, 2, 3, 5, 12, 480, 8064, 130560])
def test_philox_permutation_is_bijection(oracle, M):
    p = oracle.philox_permutation(1234, 17, M)
    assert np.array_equal(np.sort(p), np.arange(M))


def test_philox_permutation_uniformity(oracle):
    # positions of each element over many runs: chi-square against uniform
    M, R = 12, 6000
    counts = np.zeros((M, M))
    before = 0
    for r in range(R):
        p = oracle.philox_permutation(99, r, M)
        counts[np.arange(M), p] += 1
        before += int(np.argmax(p == 3) < np.argmax(p == 7))
    exp = R / M
    chi2 = ((counts - exp) ** 2 / exp).sum()
    dof = (M - 1) ** 2
    assert chi2 < dof + 6 * np.sqrt(2 * dof)
    assert abs(before / R - 0.5) < 4 * 0.5 / np.sqrt(R)


@pytest.mark.parametrize('seed', [0, 1, 42, 4294967295, [1, 2, 3], [7]])
@pytest.mark.parametrize('M', [0, 1, 2, 12, 480, 1984])
def test_mt_permutation_matches_numpy(oracle, seed, M):
    want = np.random.RandomState(seed).permutation(M)
    assert np.array_equal(oracle.mt_permutation(seed, M), want)


def test_kat_3x3(oracle):
    """percolate/test/test_percolate.py:132-192 known-answer vectors."""
    z = load_golden('kat_3x3.npz')
    assert np.array_equal(oracle.mt_permutation(42, 12), z['perm'])
    run = oracle.sample_states(9, 12, z['eu'], z['ev'], z['side'], True, z['perm'])
    assert np.array_equal(run['max'], z['test_max'])
    assert np.array_equal(run['moments_u64'].astype(np.int64), z['test_moments'])
    assert np.array_equal(run['span'], z['test_span'])


@pytest.mark.parametrize('case', golden_cases(), ids=lambda c: '%s-L%d-s%d' % (
    c['kind'], c['L'], c['seed']))
def test_reference_rows(oracle, case):
    if case['kind'] in ('grid', 'chain'):
        kind = oracle.GRID_2D if case['kind'] == 'grid' else oracle.CHAIN_1D
        N, M, eu, ev, side = oracle.lattice_graph(kind, case['L'])
        # implicit lattice numbering == networkx's perc_graph.edges() order
        assert (N, M) == (case['N'], case['M'])
        assert np.array_equal(eu, case['eu']) and np.array_equal(ev, case['ev'])
        assert np.array_equal(side, case['side'])
    assert np.array_equal(oracle.mt_permutation(case['seed'], case['M']), case['perm'])
    run = oracle.sample_states(case['N'], case['M'], case['eu'], case['ev'],
                               case['side'], case['spanning'], case['perm'])
    assert np.array_equal(run['edge'][1:], case['edge'][1:])
    assert np.array_equal(run['max'], case['max'])
    assert np.array_equal(run['moments_u64'], case['moments'])
    if case['spanning']:
        assert np.array_equal(run['span'], case['span'])


def test_injected_philox_permutations(oracle):
    z = load_golden('hpc_injected.npz')
    for ci in range(int(z['n_cases'])):
        pre = 'i%02d_' % ci
        L, key, run_id = (int(x) for x in z[pre + 'meta'])
        perm = oracle.philox_permutation(key, run_id, 2 * L * (L - 1))
        assert np.array_equal(perm, z[pre + 'perm'])
        run = oracle.lattice_run(oracle.GRID_2D, L, perm)
        assert np.array_equal(run['max'], z[pre + 'max'])
        assert np.array_equal(run['moments_u64'], z[pre + 'moments'])
        assert np.array_equal(run['span'], z[pre + 'span'])
        assert np.array_equal(run['edge'][1:], z[pre + 'edge'][1:])


def _digest(edge, mx, span, mom):
    edge = edge.copy()
    edge[0] = 0
    h = hashlib.sha256()
    for a in (edge.astype(np.uint32), mx.astype(np.uint32), span.astype(bool),
              mom.astype(np.uint64)):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_reference_checksums_large(oracle):
    """Full reference outputs up to L=256, where sum s^4 wraps modulo 2**64."""
    z = load_golden('hpc_checksums.npz')
    for ci in range(int(z['n_cases'])):
        pre = 'k%02d_' % ci
        L, seed = (int(x) for x in z[pre + 'meta'])
        M = 2 * L * (L - 1)
        if str(z[pre + 'rng']) == 'philox':
            perm = oracle.philox_permutation(seed, 0, M)
        else:
            perm = oracle.mt_permutation(seed, M)
        run = oracle.lattice_run(oracle.GRID_2D, L, perm)
        assert np.array_equal(run['moments_u64'][-1], z[pre + 'last_moments'])
        assert _digest(run['edge'], run['max'], run['span'],
                       run['moments_u64']) == str(z[pre + 'sha256'])


def test_binomial_pmf(oracle):
    z = load_golden('canonical.npz')
    for ci in range(int(z['n_pmf'])):
        M, p = int(z['pmf%02d_M' % ci]), float(z['pmf%02d_p' % ci])
        ref = z['pmf%02d_w' % ci]
        np.testing.assert_array_equal(oracle.binomial_pmf(M, p), ref)
        lo, w = oracle.binomial_band(M, p)
        full = np.zeros(M + 1)
        full[lo:lo + len(w)] = w
        # the band drops weights below exp(-80) of the mode
        np.testing.assert_allclose(full, ref, rtol=1e-9, atol=1e-33)


def test_canonical_pipeline(oracle):
    """bond_canonical_statistics / initialize / reduce / finalize fixtures."""
    z = load_golden('canonical.npz')
    for ci in range(int(z['n_can'])):
        pre = 'can%02d_' % ci
        L = int(z[pre + 'L'])
        ps = z[pre + 'ps']
        alpha = float(z[pre + 'alpha'])
        canon = z[pre + 'canonical']
        red = z[pre + 'reduced']
        fin = z[pre + 'final']
        M = 2 * L * (L - 1)
        W = np.stack([oracle.binomial_pmf(M, p) for p in ps])
        acc = None
        for r, seed in enumerate(z[pre + 'seeds']):
            run = oracle.lattice_run(oracle.GRID_2D, L,
                                     oracle.mt_permutation(int(seed), M))
            q = oracle.q_matrix(run)
            cs = W @ q
            np.testing.assert_allclose(cs[:, 0], canon[r]['percolation_probability'],
                                       rtol=1e-12, atol=1e-15)
            np.testing.assert_allclose(cs[:, 1], canon[r]['max_cluster_size'], rtol=1e-12)
            np.testing.assert_allclose(cs[:, 2:], canon[r]['moments'], rtol=1e-12,
                                       atol=1e-12)
            row = (1.0, cs, np.zeros_like(cs))
            acc = row if acc is None else oracle.reduce_rows(acc, row)
        n, mean, m2 = acc
        assert np.all(red['number_of_runs'] == n)
        np.testing.assert_allclose(mean[:, 0], red['percolation_probability_mean'],
                                   rtol=1e-12)
        np.testing.assert_allclose(mean[:, 2:], red['moments_mean'], rtol=1e-12)
        np.testing.assert_allclose(m2[:, 1], red['max_cluster_size_m2'], rtol=1e-9,
                                   atol=1e-9)
        N = L * L
        fm, fs, flo, fhi = oracle.finalize(N, n, mean[:, 1], m2[:, 1], alpha, True)
        np.testing.assert_allclose(fm, fin['percolation_strength_mean'], rtol=1e-12)
        np.testing.assert_allclose(fs, fin['percolation_strength_std'], rtol=1e-9,
                                   atol=1e-15)
        np.testing.assert_allclose(flo, fin['percolation_strength_ci'][:, 0], rtol=1e-9)
        np.testing.assert_allclose(fhi, fin['percolation_strength_ci'][:, 1], rtol=1e-9)


def test_classic_microcanonical_averages(oracle):
    """percolate.microcanonical_averages (percolate/percolate.py:708-896)."""
    z = load_golden('micro_avg.npz')
    for ci in range(int(z['n_cases'])):
        pre = 'm%02d_' % ci
        L, runs, seed = (int(x) for x in z[pre + 'meta'])
        alpha = float(z[pre + 'alpha'])
        N = L * L
        mx, sp, mom = [], [], []
        for perm in z[pre + 'perms']:
            run = oracle.lattice_run(oracle.GRID_2D, L, perm)
            mx.append(run['max'])
            sp.append(run['span'])
            mom.append(run['moments_f64'])
        mx = np.array(mx, dtype=np.float64)
        sp = np.array(sp)
        mom = np.array(mom)
        mean, lo, hi = oracle.microcanonical_average_spanning(sp.sum(0), runs, alpha)
        np.testing.assert_allclose(mean, z[pre + 'spanning_cluster'], rtol=1e-12)
        np.testing.assert_allclose(lo, z[pre + 'spanning_cluster_ci'][:, 0], rtol=1e-9)
        mlo, mhi = oracle.microcanonical_average_normal(mx.mean(0), mx.std(0, ddof=1),
                                                        runs, alpha)
        np.testing.assert_allclose(mx.mean(0) / N, z[pre + 'max_cluster_size'], rtol=1e-12)
        np.testing.assert_allclose(mlo / N, z[pre + 'max_cluster_size_ci'][:, 0],
                                   rtol=1e-9)
        np.testing.assert_allclose(mom.mean(0).T / N, z[pre + 'moments'], rtol=1e-12)


# ---------------------------------------------------------------------------
# brute-force census (oracle/nz_census.c): the checker of site percolation and
# of wrapping on the torus, pinned here by reproducing the pinned restatement
# of the reference's bond path
@pytest.mark.parametrize('kind,L', [('grid', 2), ('grid', 5), ('grid', 16), ('chain', 2),
                                    ('chain', 40)])
def test_census_reproduces_bond_oracle(oracle, kind, L):
    for run in range(4):
        N, M = oracle.census_size(kind, L, False)
        perm = oracle.philox_permutation(77, run, M)
        c = oracle.lattice_census(kind, L, perm)
        r = oracle.lattice_run(0 if kind == 'grid' else 1, L, perm)
        lo, hi = r['moments_u64'], r['moments_hi']
        np.testing.assert_array_equal(c['max_span'] & 0x7FFFFFFF, r['max'])
        np.testing.assert_array_equal((c['max_span'] >> 31).astype(bool), r['span'])
        np.testing.assert_array_equal(c['m0'], lo[:, 0])
        for k, name in ((2, 'm2'), (3, 'm3'), (4, 'm4_lo')):
            np.testing.assert_array_equal(c[name], lo[:, k])
        np.testing.assert_array_equal(c['m4_hi'].astype(np.uint64), hi[:, 4])


def test_census_known_configurations(oracle):
    # torus: the bonds of row 0 close a horizontal loop at the L-th bond
    c = oracle.lattice_census('torus', 4, np.arange(32), wrap='x')
    assert list(c['max_span'][:6] >> 31) == [0, 0, 0, 0, 1, 1]
    c = oracle.lattice_census('torus', 4, np.arange(32), wrap='y')
    # vertical bonds start at index 16; column 0's loop closes at bond 16 + 12
    flags = c['max_span'] >> 31
    assert flags[28] == 0 and flags[29] == 1
    both = oracle.lattice_census('torus', 4, np.arange(32), wrap='both')['max_span'] >> 31
    assert np.array_equal(both, flags)  # x wraps first here, so both == y
    # everything open / occupied: one cluster of N, nothing else
    for kind, L, site in (('torus', 5, False), ('torus', 5, True), ('grid', 6, True),
                          ('chain', 9, True)):
        N, S = oracle.census_size(kind, L, site)
        c = oracle.lattice_census(kind, L, np.arange(S), site=site)
        assert (c['max_span'][-1] & 0x7FFFFFFF) == N and c['m0'][-1] == 0 and c['m2'][-1] == 0
        assert c['max_span'][-1] >> 31 == 1
    # site model: nothing occupied at n = 0
    c = oracle.lattice_census('grid', 3, np.arange(9), site=True)
    assert c['max_span'][0] == 0 and c['m0'][0] == 0 and c['m2'][0] == 0
    # one site on a 1 x 1 torus is its own neighbour in both directions
    c = oracle.lattice_census('torus', 1, np.arange(1), site=True, wrap='both')
    assert list(c['max_span'] >> 31) == [0, 1]


def test_philox_permutation_is_statistically_uniform(oracle):
    """The keyed Feistel permutation behaves like a uniform random one where
    an affine-like round function fails: on a 32 x 32 torus (M = 2048 bonds,
    the first N horizontal) the share of horizontal bonds among the first M/2
    has the hypergeometric spread; position and value are independent
    (16 x 16 chi-square); consecutive elements are uncorrelated."""
    L = 32
    N, M = L * L, 2 * L * L
    runs = 400
    P = np.stack([oracle.philox_permutation(99, r, M) for r in range(runs)]).astype(np.int64)
    for r in range(0, runs, 50):
        assert np.array_equal(np.sort(P[r]), np.arange(M))
    share = (P[:, :M // 2] < N).mean(1)
    sd_hyper = np.sqrt(M / 16.0 / (M - 1) * M) / (M / 2)  # = 0.0111
    assert abs(share.mean() - 0.5) < 4 * sd_hyper / np.sqrt(runs)
    assert 0.8 < share.std() / sd_hyper < 1.25
    pos = np.broadcast_to(np.arange(M) * 16 // M, P.shape).ravel()
    table = np.bincount(pos * 16 + (P * 16 // M).ravel(), minlength=256).astype(float)
    expected = P.size / 256.0
    chi2 = ((table - expected) ** 2 / expected).sum()
    assert chi2 < 225 + 5 * np.sqrt(2 * 225)
    step = np.abs(np.diff(P, axis=1)).mean()
    assert abs(step / (M / 3.0) - 1) < 0.01   # E|U - V| = M/3 for independent uniforms
    # and the permutation depends on the key and the run id
    assert not np.array_equal(P[0], P[1])
    assert not np.array_equal(oracle.philox_permutation(98, 0, M), P[0])
