"""MLP surrogate: forward/backward kernels against the FP64 CPU oracle,
training, the Monte Carlo acceptance rule, and what the surrogate gains when
it places the p-grid of a held-out lattice size."""
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


def test_forward_and_gradients_match_fp64_oracle(gpu):
    import torch
    from oracle import mlp_oracle as MO
    from pypercolate_gb300.surrogate import MLP, WIDTHS
    rng = np.random.default_rng(3)
    model = MLP(seed=5)
    B = 96
    x = rng.normal(size=(B, WIDTHS[0])).astype(np.float32)
    t = rng.normal(size=(B, 3)).astype(np.float32)
    w = rng.uniform(0.5, 2.0, size=(B, 3)).astype(np.float32)
    dx, dt, dw = (torch.from_numpy(a).cuda() for a in (x, t, w))
    loss = float(model.loss_and_grads(dx, dt, dw))
    y = model.forward_device(dx).cpu().numpy()
    params = model.params.cpu().numpy()
    y_ref, _, _ = MO.forward(params, WIDTHS, x)
    # the oracle rounds to BF16 at the same points; an FP32-accumulated value
    # that lands next to a BF16 rounding boundary can round one BF16 ulp
    # (0.4 %) away from the FP64 one, so agreement is to ~1e-3, not bitwise
    np.testing.assert_allclose(y, y_ref, rtol=5e-3, atol=2e-3)
    loss_ref, g_ref = MO.loss_and_grads(params, WIDTHS, x, t, w)
    assert abs(loss - loss_ref) <= 2e-3 * abs(loss_ref)
    g = model.grads.cpu().numpy()
    assert g.shape == g_ref.shape
    assert np.linalg.norm(g - g_ref) <= 5e-3 * np.linalg.norm(g_ref)
    cos = g @ g_ref / (np.linalg.norm(g) * np.linalg.norm(g_ref))
    assert cos > 0.99999
    scale = np.abs(g_ref).max()
    np.testing.assert_allclose(g, g_ref, rtol=5e-2, atol=2e-3 * scale)
    assert model.take_errors() == 0  # no tensor-core wait gave up


def test_adam_matches_reference_update(gpu):
    from pypercolate_gb300.surrogate import MLP
    model = MLP(widths=(4, 8, 3), seed=1)
    p0 = model.params.cpu().numpy().astype(np.float64)
    model.grads.copy_(model.params * 0.5 + 0.1)
    g = model.grads.cpu().numpy().astype(np.float64)
    model.adam(lr=1e-3)
    m = 0.1 * g
    v = 0.001 * g * g
    want = p0 - 1e-3 * (m / 0.1) / (np.sqrt(v / 0.001) + 1e-8)
    np.testing.assert_allclose(model.params.cpu().numpy(), want, rtol=1e-5, atol=1e-7)


def test_training_fits_a_smooth_function(gpu):
    from pypercolate_gb300.surrogate import MLP
    rng = np.random.default_rng(0)
    X = rng.uniform(0, 1, size=(20000, 5)).astype(np.float32)
    Y = np.column_stack([np.tanh(8 * (X[:, 0] - 0.5)), X[:, 1] ** 2, np.sin(3 * X[:, 2])])
    model = MLP(seed=2)
    trace = model.fit(X, Y, steps=400, batch=4096, lr=1e-3, log_every=100)
    assert trace[-1][1] < 0.1 * trace[0][1]
    pred = model.predict(X[:2000])
    assert np.sqrt(np.mean((pred - Y[:2000]) ** 2)) < 0.1


def test_standard_error_weights(gpu):
    """Loss weights 1 / (se^2 + floor^2), normalised to mean 1: equal errors
    reproduce the unweighted training exactly; a half of the rows with small
    errors is then fitted better than without weights."""
    from pypercolate_gb300.surrogate import MLP
    rng = np.random.default_rng(3)
    X = rng.uniform(0, 1, size=(8192, 5)).astype(np.float32)
    Y = np.column_stack([np.sin(6 * X[:, 0]) * X[:, 1], np.cos(5 * X[:, 2]), X[:, 3] * X[:, 4]])
    a = MLP(seed=4).fit(X, Y, steps=200, batch=4096, log_every=50)
    b = MLP(seed=4).fit(X, Y, steps=200, batch=4096, log_every=50, se=np.full(Y.shape, 0.2))
    assert a == b
    precise = X[:, 0] < 0.5
    se = np.where(precise[:, None], 1e-3, 1.0) * np.ones_like(Y)
    plain, weighted = MLP(seed=5), MLP(seed=5)
    plain.fit(X, Y, steps=600, batch=4096)
    weighted.fit(X, Y, steps=600, batch=4096, se=se)
    err = lambda m: np.sqrt(np.mean((m.predict(X[precise]) - Y[precise]) ** 2))  # noqa: E731
    assert err(weighted) < err(plain)


def test_surrogate_pipeline_small(gpu):
    """Train on square lattices L in {8..48} minus 28, judge at L=28 by Monte
    Carlo, and check that surrogate-placed p-grids interpolate the held-out
    spanning curve better than a uniform grid of the same size."""
    from pypercolate_gb300 import surrogate as S
    ps = np.linspace(0.0, 1.0, 401)
    X, Y = [], []
    for L in (8, 12, 16, 20, 24, 32, 40, 48):
        y, _ = S.ensemble_targets('grid', L, ps, 1500, key=L)
        X.append(S.features(ps, L, 'grid'))
        Y.append(S.train_targets(y))
    model = S.MLP(seed=0)
    model.fit(np.concatenate(X), np.concatenate(Y), steps=1500, batch=4096, lr=1e-3)
    dense = np.linspace(0.0, 1.0, 1001)
    truth, truth_se = S.ensemble_targets('grid', 28, dense, 4000, key=2828)
    pred = S.curves(model.predict(S.features(dense, 28, 'grid')))
    values, ok = S.judged(pred[:, 0], truth[:, 0], truth_se[:, 0])
    # the Monte Carlo estimate is the fallback wherever the surrogate is rejected
    assert np.array_equal(values[~ok], truth[~ok, 0])
    assert np.array_equal(values[ok], pred[ok, 0])
    assert np.all(np.abs(values - truth[:, 0]) < 2 * truth_se[:, 0] + 1e-12)
    # a cheaper judge (fewer runs, larger error bars) accepts more of the curve
    cheap, cheap_se = S.ensemble_targets('grid', 28, dense, 200, key=2829)
    _, ok_cheap = S.judged(pred[:, 0], cheap[:, 0], cheap_se[:, 0])
    assert ok_cheap.mean() >= ok.mean() - 0.05
    k = 16
    uni = np.linspace(0.0, 1.0, k)
    placed = S.place_p_grid(model, 28, 'grid', k)
    err_uni = np.max(np.abs(np.interp(dense, uni, np.interp(uni, dense, truth[:, 0])) - truth[:, 0]))
    err_placed = np.max(np.abs(np.interp(dense, placed, np.interp(placed, dense, truth[:, 0]))
                               - truth[:, 0]))
    assert err_placed < err_uni


def test_pick_next_length_prefers_the_lattice_the_surrogate_knows_least(gpu):
    """Trained on square lattices L in {8..32}, the surrogate is judged by
    cheap pilot ensembles at three candidate lengths; the one far outside the
    training range (L = 128) disagrees most with it, in Monte Carlo standard
    errors, and is the one to simulate next."""
    from pypercolate_gb300 import surrogate as S
    ps = np.linspace(0.0, 1.0, 401)
    X, Y = [], []
    for L in (8, 12, 16, 20, 24, 28, 32):
        y, _ = S.ensemble_targets('grid', L, ps, 1500, key=L)
        X.append(S.features(ps, L, 'grid'))
        Y.append(S.train_targets(y))
    model = S.MLP(seed=1)
    model.fit(np.concatenate(X), np.concatenate(Y), steps=1500, batch=4096, lr=1e-3)
    cands = [16, 24, 128]
    choice, scores = S.pick_next_length(model, cands, 'grid', pilot_runs=400)
    assert len(scores) == 3 and all(np.isfinite(scores))
    assert choice == 128
    assert scores[2] > max(scores[0], scores[1])
