"""GPU parity: the CUDA path (through the C ABI) against the reference's golden
vectors, reference-generated fixtures and the exact CPU oracle."""
import hashlib

import numpy as np
import pytest

from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from pypercolate_gb300 import _native as nat
    nat.lib_handle()
    return nat


def _spec_for_case(case, nat, hpc):
    if case['kind'] == 'grid':
        return hpc.GraphSpec(nat.GRAPH_GRID2D, case['L'])
    if case['kind'] == 'chain':
        return hpc.GraphSpec(nat.GRAPH_CHAIN1D, case['L'])
    return hpc.GraphSpec(nat.GRAPH_EDGES, 0, case['N'], case['M'], case['eu'], case['ev'],
                         case['side'])


def _rows_equal(rows, case):
    assert np.array_equal(rows['n'], np.arange(case['M'] + 1))
    assert np.array_equal(rows['edge'][1:], case['edge'][1:])
    assert np.array_equal(rows['max_cluster_size'], case['max'])
    assert np.array_equal(rows['moments'], case['moments'])
    if case['spanning']:
        assert np.array_equal(rows['has_spanning_cluster'], case['span'])


def test_kat_3x3(gpu):
    """percolate/test/test_percolate.py:132-192, fed the test's permutation."""
    from pypercolate_gb300 import hpc
    z = load_golden('kat_3x3.npz')
    spec = hpc.GraphSpec(gpu.GRAPH_EDGES, 0, 9, 12, z['eu'], z['ev'], z['side'])
    rec = hpc._run_microcanonical(spec, True, perms=z['perm'][None, :])
    rows = hpc._pack_rows(rec, 0, spec, True)
    assert np.array_equal(rows['max_cluster_size'], z['test_max'])
    assert np.array_equal(rows['moments'].astype(np.int64), z['test_moments'])
    assert np.array_equal(rows['has_spanning_cluster'], z['test_span'])
    # same run drawn by the GPU's MT19937 from seed 42 (np.random.seed(42) in the test)
    rec = hpc._run_microcanonical(spec, True, seeds=[42])
    rows2 = hpc._pack_rows(rec, 0, spec, True)
    assert np.array_equal(rows2['max_cluster_size'], z['test_max'])


@pytest.mark.parametrize('case', golden_cases(), ids=lambda c: '%s-L%d-s%d' % (
    c['kind'], c['L'], c['seed']))
def test_reference_rows_same_seed(gpu, case):
    """Same seed -> same rows as percolate.hpc.bond_microcanonical_statistics."""
    from pypercolate_gb300 import hpc
    spec = _spec_for_case(case, gpu, hpc)
    rec = hpc._run_microcanonical(spec, case['spanning'], seeds=[case['seed']])
    _rows_equal(hpc._pack_rows(rec, 0, spec, case['spanning']), case)


def test_reference_rows_batched(gpu):
    """Many seeds in one launch, each run equal to its reference fixture."""
    from pypercolate_gb300 import hpc
    cases = [c for c in golden_cases() if c['kind'] == 'grid' and c['L'] == 16]
    spec = hpc.GraphSpec(gpu.GRAPH_GRID2D, 16)
    rec = hpc._run_microcanonical(spec, True, seeds=[c['seed'] for c in cases])
    for r, case in enumerate(cases):
        _rows_equal(hpc._pack_rows(rec, r, spec, True), case)


def test_injected_philox_permutations(gpu):
    from pypercolate_gb300 import hpc
    z = load_golden('hpc_injected.npz')
    for ci in range(int(z['n_cases'])):
        pre = 'i%02d_' % ci
        L, key, run_id = (int(x) for x in z[pre + 'meta'])
        spec = hpc.GraphSpec(gpu.GRAPH_GRID2D, L)
        rec = hpc._run_microcanonical(spec, True, rng='philox', key=key, run0=run_id, n_runs=1)
        rows = hpc._pack_rows(rec, 0, spec, True)
        assert np.array_equal(rows['edge'][1:], z[pre + 'edge'][1:])
        assert np.array_equal(rows['max_cluster_size'], z[pre + 'max'])
        assert np.array_equal(rows['moments'], z[pre + 'moments'])
        assert np.array_equal(rows['has_spanning_cluster'], z[pre + 'span'])


def test_reference_checksums_up_to_L256(gpu):
    """Full reference outputs at L = 64, 128, 256 (uint64 wrap of sum s^4)."""
    from pypercolate_gb300 import hpc
    z = load_golden('hpc_checksums.npz')
    for ci in range(int(z['n_cases'])):
        pre = 'k%02d_' % ci
        L, seed = (int(x) for x in z[pre + 'meta'])
        spec = hpc.GraphSpec(gpu.GRAPH_GRID2D, L)
        if str(z[pre + 'rng']) == 'philox':
            rec = hpc._run_microcanonical(spec, True, rng='philox', key=seed, run0=0, n_runs=1)
        else:
            rec = hpc._run_microcanonical(spec, True, seeds=[seed])
        rows = hpc._pack_rows(rec, 0, spec, True)
        h = hashlib.sha256()
        edge = rows['edge'].copy()
        edge[0] = 0
        for a in (edge, rows['max_cluster_size'], rows['has_spanning_cluster'],
                  rows['moments']):
            h.update(np.ascontiguousarray(a).tobytes())
        assert h.hexdigest() == str(z[pre + 'sha256'])


@pytest.mark.parametrize('M', [1, 2, 12, 480, 130560])
def test_permutations_match_oracle(gpu, oracle, M):
    import torch
    lib = gpu.lib_handle()
    R = 7
    out = torch.empty(R * M, dtype=torch.int32, device='cuda')
    gpu.check(lib.nz_permutations(M, R, gpu.PERM_PHILOX, 1234, 10, None, None, 1,
                                  gpu.ptr(out), gpu.stream_handle()), 'perm')
    got = out.cpu().numpy().view(np.uint32).reshape(R, M)
    for r in range(R):
        assert np.array_equal(got[r], oracle.philox_permutation(1234, 10 + r, M))
    seeds = np.array([[0], [1], [42], [7], [99], [2 ** 32 - 1], [5]], dtype=np.uint32)
    lens = np.zeros(R, dtype=np.int32)
    d_s, d_l = gpu.to_device(seeds), gpu.to_device(lens)
    gpu.check(lib.nz_permutations(M, R, gpu.PERM_MT19937, 0, 0, gpu.ptr(d_s), gpu.ptr(d_l), 1,
                                  gpu.ptr(out), gpu.stream_handle()), 'perm')
    got = out.cpu().numpy().view(np.uint32).reshape(R, M)
    for r in range(R):
        assert np.array_equal(got[r], np.random.RandomState(int(seeds[r, 0])).permutation(M))


@pytest.mark.parametrize('kind,L,R', [(0, 32, 64), (0, 100, 9), (1, 3000, 17), (0, 2, 5)])
def test_exact_records_vs_oracle(gpu, oracle, kind, L, R):
    """Every per-step integer (incl. the high word of sum s^4) of Philox runs."""
    from pypercolate_gb300 import hpc
    spec = hpc.GraphSpec(kind, L)
    rec = hpc._run_microcanonical(spec, True, rng='philox', key=99, run0=1000, n_runs=R)
    h = rec.host()
    for r in range(R):
        ref = oracle.lattice_run(kind, L, oracle.philox_permutation(99, 1000 + r, spec.M))
        assert np.array_equal(h['max_span'][:, r] & 0x7fffffff, ref['max'])
        assert np.array_equal((h['max_span'][:, r] >> 31).astype(bool), ref['span'])
        assert np.array_equal(h['m0'][:, r], ref['moments_u64'][:, 0])
        assert np.array_equal(h['m2'][:, r], ref['moments_u64'][:, 2])
        assert np.array_equal(h['m3'][:, r], ref['moments_u64'][:, 3])
        assert np.array_equal(h['m4_lo'][:, r], ref['moments_u64'][:, 4])
        assert np.array_equal(h['m4_hi'][:, r].astype(np.uint64), ref['moments_hi'][:, 4])
        assert np.array_equal(h['edge'][1:, r], ref['edge'][1:])


def test_full_occupancy_launch_matches_oracle(gpu, oracle):
    """One union-find launch with 16,384 runs of spanning_2d_grid(128) (every
    SM full of resident warps, 19 GB of records): sampled runs across the
    launch equal the oracle row for row."""
    from pypercolate_gb300 import hpc
    spec = hpc.GraphSpec(gpu.GRAPH_GRID2D, 128)
    R = 16384
    rec = hpc._run_microcanonical(spec, True, rng='philox', key=77, run0=5000, n_runs=R,
                                  with_edge=False)
    for r in (0, 1, 31, 4097, 9999, R - 1):
        ref = oracle.lattice_run(0, 128, oracle.philox_permutation(77, 5000 + r, spec.M))
        col = {k: getattr(rec, k)[r::R].cpu().numpy() for k in ('max_span', 'm2', 'm4_lo')}
        assert np.array_equal(col['max_span'].view(np.uint32) & 0x7fffffff, ref['max']), r
        assert np.array_equal((col['max_span'].view(np.uint32) >> 31).astype(bool), ref['span']), r
        assert np.array_equal(col['m2'].view(np.uint64), ref['moments_u64'][:, 2]), r
        assert np.array_equal(col['m4_lo'].view(np.uint64), ref['moments_u64'][:, 4]), r
    del rec


def test_exact_beyond_uint64_L724(gpu, oracle):
    """At L=724 sum' s^4 exceeds 2**64 in some runs (run 0 of key 5 here):
    the high word is exact."""
    from pypercolate_gb300 import hpc
    spec = hpc.GraphSpec(gpu.GRAPH_GRID2D, 724)
    rec = hpc._run_microcanonical(spec, True, rng='philox', key=5, run0=0, n_runs=3,
                                  with_edge=False)
    h = rec.host()
    wrapped = 0
    for r in range(3):
        ref = oracle.lattice_run(0, 724, oracle.philox_permutation(5, r, spec.M))
        wrapped += int(ref['moments_hi'][:, 4].max() > 0)
        assert np.array_equal(h['m4_hi'][:, r].astype(np.uint64), ref['moments_hi'][:, 4])
        assert np.array_equal(h['m4_lo'][:, r], ref['moments_u64'][:, 4])
        assert np.array_equal(h['m3'][:, r], ref['moments_u64'][:, 3])
        assert np.array_equal(h['max_span'][:, r] & 0x7fffffff, ref['max'])
    assert wrapped >= 1


def test_edge_cases(gpu):
    from pypercolate_gb300 import hpc
    # chain of one node: M = 0, a single row
    spec = hpc.GraphSpec(gpu.GRAPH_CHAIN1D, 1)
    rows = hpc._pack_rows(hpc._run_microcanonical(spec, True, seeds=[3]), 0, spec, True)
    assert rows.shape == (1,) and rows['max_cluster_size'][0] == 1
    assert list(rows['moments'][0]) == [0] * 5 and not rows['has_spanning_cluster'][0]
    # L = 1 grid
    spec = hpc.GraphSpec(gpu.GRAPH_GRID2D, 1)
    rows = hpc._pack_rows(hpc._run_microcanonical(spec, True, seeds=[3]), 0, spec, True)
    assert rows.shape == (1,)
    # explicit graph with a self-loop and a node touching both sides
    eu = np.array([0, 1, 1], np.uint32)
    ev = np.array([1, 1, 2], np.uint32)
    side = np.array([3, 0, 0], np.uint8)
    spec = hpc.GraphSpec(gpu.GRAPH_EDGES, 0, 3, 3, eu, ev, side)
    rec = hpc._run_microcanonical(spec, True, perms=np.array([[1, 0, 2]], np.uint32))
    rows = hpc._pack_rows(rec, 0, spec, True)
    # n=1 adds the self-loop: no union, spanning stays False
    assert list(rows['has_spanning_cluster']) == [False, False, True, True]
    assert list(rows['max_cluster_size']) == [1, 1, 2, 3]


def test_binomial_pmf(gpu):
    from pypercolate_gb300 import percolate as P
    z = load_golden('canonical.npz')
    for ci in range(int(z['n_pmf'])):
        M, p = int(z['pmf%02d_M' % ci]), float(z['pmf%02d_p' % ci])
        np.testing.assert_allclose(P._binomial_pmf(M, p), z['pmf%02d_w' % ci],
                                   rtol=1e-11, atol=1e-300)


def test_canonical_pipeline_rows(gpu):
    """bond_canonical_statistics / initialize / reduce / finalize on the GPU
    against the reference's outputs."""
    import functools
    from pypercolate_gb300 import hpc
    from pypercolate_gb300 import percolate as P
    z = load_golden('canonical.npz')
    for ci in range(int(z['n_can'])):
        pre = 'can%02d_' % ci
        L = int(z[pre + 'L'])
        ps = z[pre + 'ps']
        alpha = float(z[pre + 'alpha'])
        spec = hpc.GraphSpec(gpu.GRAPH_GRID2D, L)
        facs = P.binomial_pmfs(spec.M, ps)
        inits = []
        for r, seed in enumerate(z[pre + 'seeds']):
            rows = hpc._pack_rows(hpc._run_microcanonical(spec, True, seeds=[int(seed)]), 0,
                                  spec, True)
            cs = hpc.bond_canonical_statistics(rows, facs)
            ref = z[pre + 'canonical'][r]
            np.testing.assert_allclose(cs['percolation_probability'],
                                       ref['percolation_probability'], rtol=1e-10, atol=1e-14)
            np.testing.assert_allclose(cs['max_cluster_size'], ref['max_cluster_size'],
                                       rtol=1e-10)
            np.testing.assert_allclose(cs['moments'], ref['moments'], rtol=1e-10, atol=1e-10)
            init = hpc.bond_initialize_canonical_averages(cs)
            assert np.all(init['number_of_runs'] == 1)
            assert np.all(init['moments_m2'] == 0)
            np.testing.assert_array_equal(init['moments_mean'], cs['moments'])
            inits.append(init)
        red = functools.reduce(hpc.bond_reduce, inits)
        zr = z[pre + 'reduced']
        assert np.all(red['number_of_runs'] == zr['number_of_runs'])
        for k in ('percolation_probability_mean', 'max_cluster_size_mean', 'moments_mean'):
            np.testing.assert_allclose(red[k], zr[k], rtol=1e-9)
        for k in ('percolation_probability_m2', 'max_cluster_size_m2', 'moments_m2'):
            np.testing.assert_allclose(red[k], zr[k], rtol=1e-7, atol=1e-6)
        fin = hpc.finalize_canonical_averages(spec.N, ps, red, alpha)
        zf = z[pre + 'final']
        for k in zf.dtype.names:
            np.testing.assert_allclose(fin[k], zf[k], rtol=1e-7, atol=1e-12, err_msg=k)


def test_student_t_quantile(gpu):
    import scipy.stats
    import torch
    qs = np.array([0.025, 0.975, 0.1, 0.5, 0.9, 1e-6, 1 - 1e-6, 0.3, 0.15865525393145707])
    dfs = np.array([1.0, 2.0, 3.0, 5.0, 10.0, 99.0, 1000.0, 99999.0, 7.0])
    q, d = np.meshgrid(qs, dfs)
    q, d = q.ravel(), d.ravel()
    out = torch.empty(q.size, dtype=torch.float64, device='cuda')
    d_q, d_d = torch.from_numpy(q.copy()).cuda(), torch.from_numpy(d.copy()).cuda()
    gpu.check(gpu.lib_handle().nz_student_t_quantile(gpu.ptr(d_q), gpu.ptr(d_d), q.size,
                                                     gpu.ptr(out), gpu.stream_handle()), 'tq')
    np.testing.assert_allclose(out.cpu().numpy(), scipy.stats.t.ppf(q, d), rtol=1e-10,
                               atol=1e-12)


def test_banded_weights_and_record_convolution(gpu, oracle):
    """nz_binomial_weights (banded FP64) and nz_canonical_statistics_records
    (FP64 convolution of record planes) against the oracle."""
    import torch
    from pypercolate_gb300 import hpc
    lib = gpu.lib_handle()
    L, R = 16, 5
    spec = hpc.GraphSpec(gpu.GRAPH_GRID2D, L)
    ps = np.array([0.0, 0.31, 0.5, 0.77, 1.0])
    P = ps.size
    cap = lib.nz_binomial_band_cap(spec.M, 80.0)
    d_ps = torch.from_numpy(ps.copy()).cuda()
    lo = torch.empty(P, dtype=torch.int32, device='cuda')
    ln = torch.empty(P, dtype=torch.int32, device='cuda')
    w = torch.empty(P * cap, dtype=torch.float64, device='cuda')
    gpu.check(lib.nz_binomial_weights(spec.M, gpu.ptr(d_ps), P, 80.0, cap, gpu.ptr(lo),
                                      gpu.ptr(ln), gpu.ptr(w), gpu.stream_handle()), 'weights')
    W = w.cpu().numpy().reshape(P, cap)
    lo_h, ln_h = lo.cpu().numpy(), ln.cpu().numpy()
    for i, p in enumerate(ps):
        full = np.zeros(spec.M + 1)
        full[lo_h[i]:lo_h[i] + ln_h[i]] = W[i, :ln_h[i]]
        np.testing.assert_allclose(full, oracle.binomial_pmf(spec.M, p), rtol=1e-11, atol=1e-33)
    rec = hpc._run_microcanonical(spec, True, rng='philox', key=3, run0=0, n_runs=R,
                                  with_edge=False)
    out = torch.empty(R * P * 7, dtype=torch.float64, device='cuda')
    gpu.check(lib.nz_canonical_statistics_records(rec.struct(), spec.N, spec.M, R, 1,
                                                  gpu.ptr(lo), gpu.ptr(ln), gpu.ptr(w), cap, P,
                                                  gpu.ptr(out), gpu.stream_handle()), 'conv')
    got = out.cpu().numpy().reshape(R, P, 7)
    Wfull = np.stack([oracle.binomial_pmf(spec.M, p) for p in ps])
    for r in range(R):
        q = oracle.q_matrix(oracle.lattice_run(0, L, oracle.philox_permutation(3, r, spec.M)))
        np.testing.assert_allclose(got[r], Wfull @ q, rtol=1e-11, atol=1e-12)
