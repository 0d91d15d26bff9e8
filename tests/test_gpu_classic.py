"""Classic microcanonical / canonical API (percolate/percolate.py:708-1252)
against the reference's outputs recorded with the same np.random.seed."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from pypercolate_gb300 import _native as nat
    nat.lib_handle()
    return nat


def _case(z, ci):
    pre = 'm%02d_' % ci
    L, runs, seed = (int(x) for x in z[pre + 'meta'])
    return pre, L, runs, seed, float(z[pre + 'alpha'])


def test_microcanonical_averages_arrays_match_reference(gpu):
    from pypercolate_gb300 import percolate as P
    z = load_golden('micro_avg.npz')
    for ci in range(int(z['n_cases'])):
        pre, L, runs, seed, alpha = _case(z, ci)
        np.random.seed(seed)
        res = P.microcanonical_averages_arrays(
            P.microcanonical_averages(P.spanning_2d_grid(L), runs=runs, alpha=alpha))
        for k in ('spanning_cluster', 'max_cluster_size', 'moments'):
            np.testing.assert_allclose(res[k], z[pre + k], rtol=1e-12, err_msg=k)
        for k in ('spanning_cluster_ci', 'max_cluster_size_ci', 'moments_ci'):
            np.testing.assert_allclose(res[k], z[pre + k], rtol=1e-8, atol=1e-12, err_msg=k)
        assert res['N'] == int(z[pre + 'N']) and res['M'] == int(z[pre + 'M'])
        # numpy's global stream advanced exactly as the reference's runs advance it
        after = np.random.get_state()
        np.random.seed(seed)
        for _ in range(runs):
            np.random.permutation(res['M'])
        want = np.random.get_state()
        assert np.array_equal(after[1], want[1]) and after[2] == want[2]


def test_microcanonical_averages_generator(gpu):
    from pypercolate_gb300 import percolate as P
    z = load_golden('micro_avg.npz')
    pre, L, runs, seed, alpha = _case(z, 0)
    np.random.seed(seed)
    it = P.microcanonical_averages(P.spanning_2d_grid(L), runs=runs, alpha=alpha)
    first = next(it)
    # n = 0 draws no permutation (the reference's runs draw at their second step)
    state = np.random.get_state()
    np.random.seed(seed)
    assert np.array_equal(state[1], np.random.get_state()[1])
    assert first['n'] == 0 and first['max_cluster_size'] == 1.0
    assert first['spanning_cluster'] == 1 / (runs + 2)
    rows = [first] + list(it)
    N = int(z[pre + 'N'])
    assert [r['n'] for r in rows] == list(range(int(z[pre + 'M']) + 1))
    mx = np.array([r['max_cluster_size'] for r in rows]) / N
    np.testing.assert_allclose(mx, z[pre + 'max_cluster_size'], rtol=1e-12)


def test_microcanonical_averages_errors(gpu):
    from pypercolate_gb300 import percolate as P
    g = P.spanning_2d_grid(3)
    for kw in ({'runs': 'many'}, {'runs': 0}, {'alpha': 'huge'}, {'alpha': 0.0},
               {'model': 'site'}):
        with pytest.raises(ValueError):
            next(P.microcanonical_averages(g, **kw))


def test_canonical_averages_and_statistics(gpu, oracle):
    from pypercolate_gb300 import percolate as P
    z = load_golden('micro_avg.npz')
    pre, L, runs, seed, alpha = _case(z, 1)
    ps = np.linspace(0.3, 0.7, 9)
    arr = {k: z[pre + k] for k in ('spanning_cluster', 'spanning_cluster_ci', 'max_cluster_size',
                                   'max_cluster_size_ci', 'moments', 'moments_ci')}
    arr['N'], arr['M'] = int(z[pre + 'N']), int(z[pre + 'M'])
    got = P.canonical_averages(ps, arr)
    W = np.stack([oracle.binomial_pmf(arr['M'], p) for p in ps])
    np.testing.assert_allclose(got['spanning_cluster'], W @ arr['spanning_cluster'], rtol=1e-10)
    np.testing.assert_allclose(got['max_cluster_size_ci'], W @ arr['max_cluster_size_ci'],
                               rtol=1e-10)
    np.testing.assert_allclose(got['moments'], arr['moments'] @ W.T, rtol=1e-10)
    np.testing.assert_allclose(got['moments_ci'][2], W @ arr['moments_ci'][2], rtol=1e-10)
    np.random.seed(seed)
    st = P.statistics(P.spanning_2d_grid(L), ps, runs=runs, alpha=alpha)
    np.testing.assert_allclose(st['max_cluster_size'], got['max_cluster_size'], rtol=1e-10)
