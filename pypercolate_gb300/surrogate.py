"""Learned surrogate of the canonical curves, judged by Monte Carlo.

An MLP (4 hidden layers of width 128, GELU) maps (p, 1/L, lattice type
one-hot [square 2D, chain 1D]) -- plus the finite-size-scaling variable
asinh((p - p_c) L^(1/nu)) derived from them (p_c = 1/2, nu = 4/3 for bond
percolation on the square lattice; p_c = 1, nu = 1 for the chain), on which
the curves of different L collapse -- to (spanning probability, percolation
strength, log-susceptibility), where susceptibility = m2 / N (the mean size
of the non-largest clusters, sum' s^2 / N); the spanning probability is
learned as its logit and the strength as its logarithm (``train_targets``,
``curves``).  It is trained with the library's
own forward, backward and Adam kernels (libnzgb300 ``nz_mlp_*``: tcgen05
GEMMs with BF16 operands and FP32 accumulation) on ensembles that this
package's GPU path generates.

The Monte Carlo estimate stays the judge and the fallback: a surrogate value
is accepted only where it lies within ``accept_sigma`` Monte Carlo standard
errors of an ensemble estimate; elsewhere the ensemble estimate is used.
The surrogate is used to place p-grids (points where the curves change
fastest) and to pick the next lattice size to simulate.
"""
import numpy as np

from . import _native as nat

WIDTHS = (5, 128, 128, 128, 128, 3)
OUTPUTS = ('spanning_probability', 'percolation_strength', 'log_susceptibility')
KIND_2D, KIND_CHAIN = 'grid', 'chain'


# (p_c, 1/nu) of the two lattice families
SCALING = {KIND_2D: (0.5, 0.75), KIND_CHAIN: (1.0, 1.0)}


def features(ps, L, kind):
    """Input rows (p, 1/L, is_square_2d, is_chain_1d, asinh((p - p_c) L^(1/nu)))."""
    ps = np.asarray(ps, dtype=np.float64)
    out = np.zeros((ps.size, WIDTHS[0]), dtype=np.float32)
    out[:, 0] = ps
    out[:, 1] = 1.0 / float(L)
    out[:, 2 if kind == KIND_2D else 3] = 1.0
    p_c, inv_nu = SCALING[kind]
    out[:, 4] = np.arcsinh((ps - p_c) * float(L) ** inv_nu)
    return out


def training_grid(kind, L, n):
    """n probabilities for one lattice: half uniform in [0, 1], half inside
    the finite-size transition window (square lattice: p_c = 1/2 +- 8 L^-3/4,
    from nu = 4/3; chain: the last 8/l below p = 1), where the curves change
    and a uniform grid puts almost no points."""
    uni = np.linspace(0.0, 1.0, n - n // 2)
    if kind == KIND_2D:
        w = 8.0 * float(L) ** -0.75
        win = np.linspace(max(0.0, 0.5 - w), min(1.0, 0.5 + w), n // 2)
    else:
        win = np.linspace(max(0.0, 1.0 - 8.0 / L), 1.0, n // 2)
    return np.unique(np.concatenate([uni, win]))


def ensemble_targets(kind, L, ps, runs, key=11, run0=0, precision='fp32'):
    """Monte Carlo estimates and standard errors of the three curves at ps,
    from one GPU ensemble (canonical averages of `runs` runs)."""
    from .ensemble import Ensemble
    ens = Ensemble(kind, L, ps, precision=precision, micro=False)
    ens.run(runs, key=key, run0=run0)
    ca = ens.canonical_averages()
    N = ens.N
    n = ca['number_of_runs'].astype(np.float64)
    se = lambda m2: np.sqrt(np.maximum(m2, 0.0) / np.maximum(n - 1, 1)) / np.sqrt(n)  # noqa: E731
    span = ca['percolation_probability_mean']
    # where every run agrees the sample error is 0; floor it at the binomial
    # error of the Bayesian estimate (k+1)/(R+2) (one run's worth of doubt)
    pb = (span * n + 1.0) / (n + 2.0)
    span_se = np.maximum(se(ca['percolation_probability_m2']), np.sqrt(pb * (1 - pb) / n))
    strength = ca['max_cluster_size_mean'] / N
    strength_se = np.maximum(se(ca['max_cluster_size_m2']) / N, 1.0 / (N * np.sqrt(n)))
    chi = ca['moments_mean'][:, 2] / N
    chi_se = np.maximum(se(ca['moments_m2'][:, 2]) / N, 1.0 / (N * np.sqrt(n)))
    floor = 1.0 / N ** 2
    log_chi = np.log(np.maximum(chi, floor))
    log_chi_se = chi_se / np.maximum(chi, floor)
    y = np.column_stack([span, strength, log_chi])
    s = np.column_stack([span_se, strength_se, log_chi_se])
    return y, s


STRENGTH_FLOOR = 1e-12
SPAN_EPS = 1e-6


def train_targets(y):
    """The curves as the network learns them: the logit of the spanning
    probability (clipped to [1e-6, 1 - 1e-6]), log strength and log
    susceptibility.  Away from the threshold the spanning probability is 0
    or 1 to within its Monte Carlo error (~1/runs), and below it the
    strength is ~log(N)/N with an error ~1e-6: in logit and log units the
    network's error is relative there, so it can come within the judge's
    error bars."""
    out = np.array(y, dtype=np.float64, copy=True)
    pi = np.clip(out[:, 0], SPAN_EPS, 1.0 - SPAN_EPS)
    out[:, 0] = np.log(pi) - np.log1p(-pi)
    out[:, 1] = np.log(np.maximum(out[:, 1], STRENGTH_FLOOR))
    return out


def train_se(y, se):
    """Standard errors of the curves (``ensemble_targets``) in the units the
    network learns (``train_targets``), to first order: the spanning error
    divided by pi (1 - pi) (at most one logit unit where pi is within its
    error of 0 or 1), the strength's error relative."""
    y = np.asarray(y, dtype=np.float64)
    out = np.array(se, dtype=np.float64, copy=True)
    pi = y[:, 0]
    out[:, 0] = out[:, 0] / np.maximum(pi * (1.0 - pi), out[:, 0])
    out[:, 1] = out[:, 1] / np.maximum(y[:, 1], STRENGTH_FLOOR)
    return out


def curves(pred):
    """Network outputs back to (spanning probability, strength, log
    susceptibility)."""
    out = np.array(pred, dtype=np.float64, copy=True)
    out[:, 0] = 0.5 * (1.0 + np.tanh(0.5 * out[:, 0]))  # the logistic function, overflow-free
    out[:, 1] = np.exp(out[:, 1])
    return out


class MLP:
    """Parameters and optimizer state on the GPU; all arithmetic in the library."""

    def __init__(self, widths=WIDTHS, seed=0):
        torch = nat.torch_cuda()
        self.widths = np.asarray(widths, dtype=np.int32)
        self.n_layers = len(widths) - 1
        lib = nat.lib_handle()
        self.count = int(lib.nz_mlp_param_count(self.widths.ctypes.data, self.n_layers))
        rng = np.random.default_rng(seed)
        host = np.empty(self.count, dtype=np.float32)
        o = 0
        for i in range(self.n_layers):
            fan_in, fan_out = widths[i], widths[i + 1]
            bound = np.sqrt(6.0 / fan_in) / np.sqrt(2.0)
            host[o:o + fan_in * fan_out] = rng.uniform(-bound, bound, fan_in * fan_out)
            o += fan_in * fan_out
            host[o:o + fan_out] = 0.0
            o += fan_out
        self.params = torch.from_numpy(host).cuda()
        self.params_bf16 = torch.empty(self.count, dtype=torch.int16, device='cuda')
        self.grads = torch.zeros(self.count, dtype=torch.float32, device='cuda')
        self.m = torch.zeros(self.count, dtype=torch.float32, device='cuda')
        self.v = torch.zeros(self.count, dtype=torch.float32, device='cuda')
        self.step_count = 0
        nat.check(lib.nz_mlp_params_to_bf16(nat.ptr(self.params), self.count,
                                            nat.ptr(self.params_bf16), nat.stream_handle()),
                  'nz_mlp_params_to_bf16')
        self.x_mean = np.zeros(int(widths[0]), np.float32)
        self.x_std = np.ones(int(widths[0]), np.float32)
        self.y_mean = np.zeros(3, np.float32)
        self.y_std = np.ones(3, np.float32)
        self._buf = {}

    def _buffers(self, batch):
        torch = nat.torch_cuda()
        if batch not in self._buf:
            acts = int(nat.lib_handle().nz_mlp_activation_count(self.widths.ctypes.data,
                                                                self.n_layers, batch))
            self._buf[batch] = dict(
                z=torch.empty(acts, dtype=torch.float32, device='cuda'),
                h=torch.empty(acts, dtype=torch.float32, device='cuda'),
                y=torch.empty(batch * int(self.widths[-1]), dtype=torch.float32, device='cuda'),
                dy=torch.empty(batch * int(self.widths[-1]), dtype=torch.float32, device='cuda'),
                scratch=torch.empty(2 * batch * int(self.widths.max()), dtype=torch.float32,
                                    device='cuda'),
                loss=torch.empty(64, dtype=torch.float32, device='cuda'))
        return self._buf[batch]

    def forward_device(self, x):
        """x: device float32 [batch, widths[0]] (already standardised) -> device y."""
        batch = x.shape[0]
        b = self._buffers(batch)
        nat.check(nat.lib_handle().nz_mlp_forward(
            self.widths.ctypes.data, self.n_layers, batch, nat.ptr(x), nat.ptr(self.params),
            nat.ptr(self.params_bf16), nat.ptr(b['z']), nat.ptr(b['h']), nat.ptr(b['y']),
            nat.stream_handle()), 'nz_mlp_forward')
        return b['y'][:batch * int(self.widths[-1])].view(batch, -1)

    def loss_and_grads(self, x, t, w=None):
        """Forward + weighted squared error + backward; returns the loss (device)."""
        lib = nat.lib_handle()
        batch = x.shape[0]
        b = self._buffers(batch)
        self.forward_device(x)
        nout = int(self.widths[-1])
        nat.check(lib.nz_mlp_loss(nat.ptr(b['y']), nat.ptr(t), nat.ptr(w), batch, nout,
                                  nat.ptr(b['dy']), nat.ptr(b['loss']), 64, nat.stream_handle()),
                  'nz_mlp_loss')
        nat.check(lib.nz_mlp_backward(
            self.widths.ctypes.data, self.n_layers, batch, nat.ptr(x), nat.ptr(self.params_bf16),
            nat.ptr(b['z']), nat.ptr(b['h']), nat.ptr(b['dy']), nat.ptr(self.grads),
            nat.ptr(b['scratch']), nat.stream_handle()), 'nz_mlp_backward')
        return b['loss'].sum()

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step_count += 1
        nat.check(nat.lib_handle().nz_mlp_adam(
            nat.ptr(self.params), nat.ptr(self.grads), nat.ptr(self.m), nat.ptr(self.v),
            nat.ptr(self.params_bf16), self.count, lr, beta1, beta2, eps, self.step_count,
            nat.stream_handle()), 'nz_mlp_adam')

    @staticmethod
    def take_errors():
        """Tensor-core GEMM tiles whose waits gave up since the last call
        (0 in every valid use; such tiles hold NaN)."""
        import ctypes
        v = ctypes.c_uint32(0)
        nat.check(nat.lib_handle().nz_mlp_take_errors(ctypes.byref(v)), 'nz_mlp_take_errors')
        return int(v.value)

    def fit(self, X, Y, steps=3000, batch=4096, lr=1e-3, seed=0, log_every=0, decay=0.0,
            se=None, se_floor=0.01):
        """Standardise, then Adam on random mini-batches; the learning rate
        stays `lr`, then (decay > 0) falls geometrically to lr * decay over
        the last third of the steps.  With `se` (the targets' Monte Carlo
        standard errors, same shape and units as Y) the squared errors are
        weighted by 1 / (se^2 + se_floor^2) in standardised units, normalised
        to mean 1 per output: precisely known points count more, points the
        ensembles hardly determine less.  Returns the loss trace."""
        torch = nat.torch_cuda()
        X = np.asarray(X, np.float32)
        Y = np.asarray(Y, np.float32)
        self.x_mean, self.x_std = X.mean(0), X.std(0) + 1e-6
        self.y_mean, self.y_std = Y.mean(0), Y.std(0) + 1e-6
        dX = torch.from_numpy((X - self.x_mean) / self.x_std).cuda()
        dY = torch.from_numpy((Y - self.y_mean) / self.y_std).cuda()
        dW = None
        if se is not None:
            s = np.asarray(se, np.float64) / self.y_std
            w = 1.0 / (s * s + se_floor * se_floor)
            w /= w.mean(0)
            dW = torch.from_numpy(w.astype(np.float32)).cuda()
        gen = torch.Generator(device='cuda')
        gen.manual_seed(seed)
        n = dX.shape[0]
        batch = min(batch, n)
        trace = []
        for k in range(steps):
            idx = torch.randint(0, n, (batch,), device='cuda', generator=gen)
            loss = self.loss_and_grads(dX[idx].contiguous(), dY[idx].contiguous(),
                                       None if dW is None else dW[idx].contiguous())
            rate = lr
            if decay > 0.0 and k > 2 * steps // 3:
                rate = lr * decay ** ((k - 2 * steps // 3) / max(1, steps - 2 * steps // 3))
            self.adam(rate)
            if log_every and (k % log_every == 0 or k == steps - 1):
                trace.append((k, float(loss)))
        if self.take_errors():
            raise RuntimeError('MLP tensor-core GEMM waits gave up during training')
        return trace

    def predict(self, X):
        torch = nat.torch_cuda()
        X = (np.asarray(X, np.float32) - self.x_mean) / self.x_std
        out = []
        for i in range(0, X.shape[0], 65536):
            dx = torch.from_numpy(np.ascontiguousarray(X[i:i + 65536])).cuda()
            out.append(self.forward_device(dx).cpu().numpy().copy())
        return np.concatenate(out) * self.y_std + self.y_mean


def judged(pred, mc, mc_se, accept_sigma=2.0):
    """Surrogate values where |pred - mc| < accept_sigma * se, Monte Carlo
    elsewhere.  Returns (values, accepted mask)."""
    ok = np.abs(pred - mc) < accept_sigma * np.maximum(mc_se, 1e-12)
    return np.where(ok, pred, mc), ok


def place_p_grid(model, L, kind, k, lo=0.0, hi=1.0, dense=4001, floor=0.05):
    """k probabilities placed where the surrogate's spanning curve changes
    fastest: quantiles of the density |dPi/dp| + floor * mean|dPi/dp|."""
    p = np.linspace(lo, hi, dense)
    pi = curves(model.predict(features(p, L, kind)))[:, 0]
    d = np.abs(np.gradient(pi, p))
    d = d + floor * d.mean() + 1e-12
    cdf = np.concatenate([[0.0], np.cumsum(0.5 * (d[1:] + d[:-1]) * np.diff(p))])
    cdf /= cdf[-1]
    return np.interp(np.linspace(0.0, 1.0, k), cdf, p)


def pick_next_length(model, candidates, kind, pilot_runs=200, ps=None, key=99):
    """Among candidate lengths, the one where a cheap pilot ensemble disagrees
    most with the surrogate (in Monte Carlo standard errors): the lattice the
    surrogate knows least, hence the most useful one to simulate next."""
    if ps is None:
        ps = np.linspace(0.3, 0.7, 41)
    scores = []
    for L in candidates:
        y, s = ensemble_targets(kind, L, ps, pilot_runs, key=key)
        pred = curves(model.predict(features(ps, L, kind)))
        z = np.abs(pred[:, 0] - y[:, 0]) / np.maximum(s[:, 0], 1e-6)
        scores.append(float(np.mean(z)))
    return candidates[int(np.argmax(scores))], scores
