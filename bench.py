"""Benchmark: bond additions per second of the Newman-Ziff ensemble at L=256.

One step = one batch of R independent runs on spanning_2d_grid(256)
(N = 65,536 sites, M = 130,560 bonds) through the whole hot path: Philox
permutations, union-find with per-step statistics, fused microcanonical
run-reductions, banded canonical convolution at 1001 uniform p in [0, 1],
and the pairwise merge into the running (n, mean, M2) averages.
value = R * M * n_gpus / step time (bond additions per second).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the CPU restatement of the reference pipeline
(oracle/, threaded over all host cores) on the same lattice and p-grid.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

L_DEFAULT = 256
P_DEFAULT = 1001
KEY = 1234
# algorithmic DRAM bytes per bond addition of the union-find kernel: four
# random 32-byte sectors (find(u), find(v), the child pointer and the root
# word written on a union) plus the per-step record it streams


def uf_bytes_per_add(N):
    """4 x 32 B plus the record the ensemble writes per step: 26 B up to
    N = 65,536 nodes (m0 and m2 narrow), 32 B up to 115,000 (no m4 high
    words), 36 B above."""
    return 4 * 32 + (26 if N <= 65536 else 32 if N <= 115000 else 36)
# measured DRAM bytes (read + write) per bond addition of uf_window_kernel:
# ncu capture of spanning_2d_grid(256), 12,288 runs, one 1,024-row window at
# p ~ 0.5; a full launch's traffic is this figure times the additions it
# makes
UF_TRAFFIC_PER_ADD = 177.3
UF_READ_PER_ADD = 90.6  # of which read (the scattered finds)


def bench_window(M, R, window):
    """Record-window rows of an ensemble of R runs (as nz_ensemble picks
    them: ~32 GiB of 36-byte records per window, 256 .. M + 1 rows)."""
    if window > 0:
        return min(window, M + 1)
    return int(max(256, min(M + 1, 32.0 * (1 << 30) / (R * 36))))


def curve_errors_vs_fp64(L, ps, precision, sample, run0, window):
    """Max absolute and relative error per canonical curve (as finalised:
    spanning as is, the rest / N) of `precision` against the FP64
    convolution of the same runs (the timed runs run0 .. run0 + sample - 1,
    same record windows), for the mean and the standard deviation."""
    import torch
    from pypercolate_gb300.ensemble import Ensemble
    got = {}
    for prec in (precision, 'fp64'):
        e = Ensemble('grid', L, ps, precision=prec, micro=False, window=window)
        e.run(sample, key=KEY, run0=run0)
        ca = e.canonical_averages()
        got[prec] = (np.column_stack([ca['percolation_probability_mean'], ca['max_cluster_size_mean'],
                                      ca['moments_mean']]),
                     np.column_stack([ca['percolation_probability_m2'], ca['max_cluster_size_m2'],
                                      ca['moments_m2']]))
        N = e.N
        del e
        torch.cuda.empty_cache()
    (gm, g2), (rm, r2) = got[precision], got['fp64']
    norm = np.array([1.0] + [float(N)] * 6)
    out = {}
    for j, name in enumerate(STAT_NAMES):
        a, b = gm[:, j] / norm[j], rm[:, j] / norm[j]
        sa = np.sqrt(np.maximum(g2[:, j], 0) / (sample - 1)) / norm[j]
        sb = np.sqrt(np.maximum(r2[:, j], 0) / (sample - 1)) / norm[j]
        nz = np.abs(b) > 1e-12 * np.max(np.abs(b))  # relative error above the far tails
        out[name] = {'max_abs': float(np.max(np.abs(a - b))),
                     'max_rel': float(np.max(np.abs(a - b)[nz] / np.abs(b[nz]))) if nz.any() else 0.0,
                     'std_max_abs': float(np.max(np.abs(sa - sb))),
                     'curve_max': float(np.max(np.abs(b)))}
    return {'sample_runs': sample, 'precision': precision, 'window_rows': window,
            'criterion': 'spanning, max/N, m0/N, m1/N, m2/N: max_abs < 1e-6; m3/N, m4/N: '
                         'max_rel < 1e-6 (relative errors where the value is >= 1e-12 of the '
                         'curve maximum)',
            'curves': out}


def plain_mix_leg(counts, stream, fused=False, grid=(8, 512), chain=(1024, 65536), grid_step=32,
                  chain_step=512):
    """The uneven workload the plain way: one lattice size per launch
    sequence (class draw, queue, union-find with the same 256 checkpoints,
    exact reduction, the batched leg's choice of reduction), back to back on
    one stream, each class with the runs
    the batched ensemble gave it (`counts`, grid classes then chain
    classes).  Timed on a stratified sample -- every grid_step-th grid
    length and every chain_step-th chain length -- and scaled by the strata
    sizes into whole-workload additions and time."""
    import torch
    from pypercolate_gb300.mix import MixEnsemble
    n_grid = grid[1] - grid[0] + 1
    legs = []
    for c in range(0, n_grid, grid_step):
        if counts[c]:
            L = grid[0] + c
            legs.append(('grid', grid_step, MixEnsemble(int(counts[c]), grid=(L, L), chain=chain[:1] * 2,
                                                        chain_share=0.0, threads=int(counts[c]),
                                                        fused=fused)))
    for c in range(0, chain[1] - chain[0] + 1, chain_step):
        k = int(counts[n_grid + c])
        if k:
            l = chain[0] + c
            legs.append(('chain', chain_step, MixEnsemble(k, grid=grid[:1] * 2, chain=(l, l),
                                                          chain_share=1.0, threads=k, fused=fused)))
    for _, _, e in legs[:4]:  # warm-up (module load)
        e.run(1)
    torch.cuda.synchronize()
    t = {'grid': 0.0, 'chain': 0.0}
    a = {'grid': 0, 'chain': 0}
    step = {'grid': grid_step, 'chain': chain_step}
    for kind in ('grid', 'chain'):
        sel = [e for k, _, e in legs if k == kind]
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for e in sel:
            e.run(3)
        e1.record(stream)
        torch.cuda.synchronize()
        t[kind] = e0.elapsed_time(e1) * 1e-3
        a[kind] = sum(e.additions for e in sel)
    total_t = sum(step[k] * t[k] for k in t)
    total_a = sum(step[k] * a[k] for k in a)
    out = {'value': total_a / total_t, 'unit': 'bond additions/s',
           'sample': 'every %dth of %d grid lengths and every %dth of %d chain lengths, each '
                     'with its runs of the batched workload in one launch sequence; '
                     'whole-workload estimate = sum over strata of stride x sample'
                     % (grid_step, n_grid, chain_step, chain[1] - chain[0] + 1),
           'launch_sequences': len(legs),
           'sample_seconds': {k: t[k] for k in t}, 'sample_additions': a,
           'estimated_workload_seconds': total_t}
    del legs
    torch.cuda.empty_cache()
    return out


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=5)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--runs', type=int, default=100000, help='runs per step per GPU')
    ap.add_argument('--L', type=int, default=L_DEFAULT)
    ap.add_argument('--P', type=int, default=P_DEFAULT)
    ap.add_argument('--precision', default='fp32', choices=['fp32', 'tf32x3', 'fp64'],
                    help="canonical convolution: FP32 SIMT (default), 3xTF32 on the tensor cores "
                         "(tcgen05), or FP64")
    ap.add_argument('--no-micro', action='store_true')
    ap.add_argument('--window', type=int, default=0)
    ap.add_argument('--cpu-sample', type=int, default=256, help='runs in the CPU baseline sample')
    ap.add_argument('--e2e-steps', type=int, default=2)
    ap.add_argument('--plain-runs', type=int, default=8192,
                    help='runs timed on the plain path (0: skip)')
    ap.add_argument('--plain-chunk', type=int, default=4096)
    ap.add_argument('--surrogate-weights', default='se', choices=['none', 'se'],
                    help='surrogate study: weight the training loss by the Monte Carlo '
                         'standard errors of the targets')
    ap.add_argument('--surrogate-se-floor', type=float, default=0.01,
                    help='surrogate study: standardised error added to each target\'s '
                         'standard error in its loss weight')
    ap.add_argument('--surrogate-steps', type=int, default=30000,
                    help='Adam steps of --study surrogate')
    ap.add_argument('--no-tune', dest='tune', action='store_false',
                    help='skip the launch-shape autotuner of the main leg (library defaults)')
    ap.add_argument('--no-plain-mix', dest='plain_mix', action='store_false',
                    help='skip the one-lattice-per-launch timing of the uneven workload')
    ap.add_argument('--curve-sample', type=int, default=2048,
                    help='timed runs re-run in FP64 for the per-curve error (0: skip)')
    ap.add_argument('--mix-runs', type=int, default=1000000,
                    help='runs of the batched uneven workload (0: skip)')
    ap.add_argument('--study', default=None, choices=[None, 'precision', 'surrogate', 'mlp'],
                    help='precision: FP32 vs FP64 canonical curves at L=1024; surrogate: train '
                         'and judge the MLP surrogate; mlp: MLP training throughput (separate lines)')
    ap.add_argument('--lattice', default='grid', choices=['grid', 'torus'],
                    help='main leg lattice: spanning_2d_grid or the periodic square lattice '
                         '(wrapping in either direction); for profiling the extensions')
    ap.add_argument('--model', default='bond', choices=['bond', 'site'],
                    help='main leg percolation model (site: one step per site)')
    ap.add_argument('--l2-fetch', type=int, default=32,
                    help='L2 fetch granularity of this process (bytes; 0 = leave as is)')
    return ap.parse_args()


def peaks():
    path = os.path.join(REPO, 'MEASURED_PEAKS.json')
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d['hbm_gbs']), 'measured'
    return 6800.0, 'fallback'


def random_gather_rate(gib=16, k=1 << 28, reps=3):
    """Random-access ceiling of this GPU's HBM: 4-byte gathers at uniformly
    random positions of a `gib` GiB array (far larger than L2), each touching
    its own 32-byte sector; returns sectors (gathers) per second, best of
    `reps` (CUDA events).  The union-find's finds are such accesses."""
    import torch
    n = (gib << 30) // 4
    a = torch.zeros(n, dtype=torch.int32, device='cuda')
    gen = torch.Generator(device='cuda')
    gen.manual_seed(7)
    idx = torch.randint(0, n, (k,), device='cuda', generator=gen)
    out = torch.empty(k, dtype=torch.int32, device='cuda')
    torch.index_select(a, 0, idx, out=out)
    best = None
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.index_select(a, 0, idx, out=out)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) * 1e-3
        best = t if best is None else min(best, t)
    del a, idx, out
    torch.cuda.empty_cache()
    return k / best


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
         'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
         'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.Q,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith('active'):
                    reasons.add(name)
        return {'sm_mhz': float(np.median(sm)) if sm else None,
                'sm_max_mhz': float(max(smax)) if smax else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


def cpu_baseline(L, ps, sample, threads=None):
    """The oracle's threaded CPU pipeline on a bounded sample of runs."""
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    N, M = O.lattice_size(O.GRID_2D, L)
    bands = O.band_table(M, ps)
    t0 = time.perf_counter()
    O.ensemble_canonical(O.GRID_2D, L, KEY, 10 ** 9, sample, ps, n_threads=threads, bands=bands)
    dt = time.perf_counter() - t0
    return {'value': sample * M / dt, 'unit': 'bond additions/s', 'cores': threads,
            'kind': 'port',
            'sample': '%d runs of spanning_2d_grid(%d), %d p, union-find + FP64 banded '
                      'canonical convolution + pairwise merge (oracle/nz_oracle.c)' %
                      (sample, L, len(ps))}


def dist_setup(args):
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return world, rank, local


def run_reference(args):
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return 0
    from oracle import oracle as O
    L = args.L
    ps = np.linspace(0.0, 1.0, args.P)
    N, M = O.lattice_size(O.GRID_2D, L)
    threads = os.cpu_count() or 1
    bands = O.band_table(M, ps)
    sample = max(threads * 4, 16)
    for _ in range(args.warmup):
        O.ensemble_canonical(O.GRID_2D, L, KEY, 0, threads, ps, n_threads=threads, bands=bands)
    t0 = time.perf_counter()
    for k in range(args.steps):
        O.ensemble_canonical(O.GRID_2D, L, KEY, k * sample, sample, ps, n_threads=threads,
                             bands=bands)
    dt = (time.perf_counter() - t0) / args.steps
    value = sample * M / dt
    line = {
        'impl': 'reference', 'metric': 'bond additions/s', 'value': value,
        'unit': 'bond additions/s', 'n_gpus': args.gpus, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': dt * 1e3, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'int64/u128 + f64',
        'data': 'synthetic (Philox permutations)',
        'config': {'workload': 'spanning_2d_grid(%d), %d uniform p, bounded sample of %d runs '
                               'per step on the host cores' % (L, args.P, sample),
                   'L': L, 'P': args.P, 'runs_per_step': sample},
        'cpu_baseline': {'value': value, 'unit': 'bond additions/s', 'cores': threads,
                         'kind': 'port',
                         'sample': '%d runs per step (oracle/nz_oracle.c restatement of '
                                   'percolate/hpc.py, pthreads over all cores)' % sample},
        'e2e': {'value': value, 'unit': 'bond additions/s', 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': 0},
    }
    print(json.dumps(line))
    return 0


STAT_NAMES = ('percolation_probability', 'max_cluster_size', 'm0', 'm1', 'm2', 'm3', 'm4')


def precision_study(args):
    """Canonical curves of spanning_2d_grid(L) from FP32 (FP64 chunk sums)
    against FP64 convolution of the same exact records (same Philox runs):
    max absolute and relative error per curve.  Default: L=1024, 2e4 runs,
    1000 uniform p in [0, 1] + 1000 uniform p in [0.48, 0.52]."""
    import torch
    from pypercolate_gb300 import _native as nat
    from pypercolate_gb300.ensemble import Ensemble
    torch.cuda.set_device(0)
    if args.l2_fetch:
        nat.set_l2_fetch_granularity(args.l2_fetch)
    L = args.L if args.L != L_DEFAULT else 1024
    R = args.runs if args.runs != 100000 else 20000
    ps = np.concatenate([np.linspace(0.0, 1.0, 1000), np.linspace(0.48, 0.52, 1000)])
    N = L * L
    out = {}
    times = {}
    for prec in ('fp64', 'fp32'):
        e = Ensemble('grid', L, ps, precision=prec, micro=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        chunk = min(R, 20000)
        done = 0
        while done < R:
            e.run(min(chunk, R - done), key=KEY, run0=done)
            done += min(chunk, R - done)
        torch.cuda.synchronize()
        times[prec] = time.perf_counter() - t0
        ca = e.canonical_averages()
        out[prec] = np.column_stack([ca['percolation_probability_mean'],
                                     ca['max_cluster_size_mean'], ca['moments_mean']])
        del e
        torch.cuda.empty_cache()
    ref, got = out['fp64'], out['fp32']
    norm = np.array([1.0, N, N, N, N, N, N])  # curves as the finalised output reports them
    err = {}
    for j, name in enumerate(STAT_NAMES):
        a = np.abs(got[:, j] - ref[:, j]) / norm[j]
        rel = np.abs(got[:, j] - ref[:, j]) / np.maximum(np.abs(ref[:, j]), 1e-300)
        err[name] = {'max_abs': float(a.max()), 'max_rel': float(rel[np.abs(ref[:, j]) > 0].max())
                     if np.any(np.abs(ref[:, j]) > 0) else 0.0}
    line = {'study': 'canonical precision', 'L': L, 'runs': R, 'P': len(ps),
            'p_grid': '1000 uniform in [0,1] + 1000 uniform in [0.48,0.52]',
            'compare': 'FP32 products/chunk sums (TwoSum FP32 pairs across 128-row chunks) vs FP64 '
                       'convolution of the same exact per-step records',
            'normalisation': 'spanning as is; max and moments divided by N (finalised curves)',
            'errors': err, 'seconds': times}
    print(json.dumps(line))
    return 0


def surrogate_study(args):
    """Train the MLP surrogate on ensembles at square lattices L in
    {16..512} minus 384 and chains l in {1024..65536}, then judge it at the
    held-out L = 384 against a Monte Carlo ensemble (2 standard errors), and
    measure what its p-grid placement gains over a uniform grid."""
    import torch
    from pypercolate_gb300 import _native as nat
    from pypercolate_gb300 import surrogate as S
    torch.cuda.set_device(0)
    if args.l2_fetch:
        nat.set_l2_fetch_granularity(args.l2_fetch)
    P = 52000
    lattices = [('grid', L) for L in (16, 24, 32, 48, 64, 96, 128, 192, 256, 320, 448, 512)] + \
               [('chain', l) for l in (1024, 2048, 4096, 8192, 16384, 32768, 65536)]
    t0 = time.perf_counter()
    X, Y, SE = [], [], []
    for kind, L in lattices:
        M = 2 * L * (L - 1) if kind == 'grid' else L - 1
        runs = int(min(20000, max(1000, 2e9 / M)))
        grid = S.training_grid(kind, L, P)
        y, s = S.ensemble_targets(kind, L, grid, runs, key=L)
        X.append(S.features(grid, L, kind))
        Y.append(S.train_targets(y))
        SE.append(S.train_se(y, s))
    X, Y, SE = np.concatenate(X), np.concatenate(Y), np.concatenate(SE)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    model = S.MLP(seed=0)
    steps, batch = args.surrogate_steps, 4096
    t0 = time.perf_counter()
    weighted = args.surrogate_weights == 'se'
    trace = model.fit(X, Y, steps=steps, batch=batch, lr=1e-3, log_every=1000, decay=0.05,
                      se=SE if weighted else None, se_floor=args.surrogate_se_floor)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    dense = np.linspace(0.0, 1.0, 2001)
    truth, se = S.ensemble_targets('grid', 384, dense, 8000, key=384384)
    pred = S.curves(model.predict(S.features(dense, 384, 'grid')))
    acc = {}
    cheap, cheap_se = S.ensemble_targets('grid', 384, dense, 400, key=384400)
    for j, name in enumerate(S.OUTPUTS):
        _, ok = S.judged(pred[:, j], truth[:, j], se[:, j])
        _, ok_c = S.judged(pred[:, j], cheap[:, j], cheap_se[:, j])
        rms = float(np.sqrt(np.mean((pred[:, j] - truth[:, j]) ** 2)))
        acc[name] = {'judge_8000_runs': float(ok.mean()), 'judge_400_runs': float(ok_c.mean()),
                     'rms_error_vs_8000_runs': rms,
                     'median_se_8000_runs': float(np.median(se[:, j]))}
    gains = {}
    for k in (16, 32, 64):
        uni = np.linspace(0.0, 1.0, k)
        placed = S.place_p_grid(model, 384, 'grid', k)
        e_uni = float(np.max(np.abs(np.interp(dense, uni, np.interp(uni, dense, truth[:, 0]))
                                    - truth[:, 0])))
        e_pl = float(np.max(np.abs(np.interp(dense, placed, np.interp(placed, dense, truth[:, 0]))
                                   - truth[:, 0])))
        gains[k] = {'uniform_max_err': e_uni, 'surrogate_max_err': e_pl, 'ratio': e_uni / e_pl}
    nxt, scores = S.pick_next_length(model, [352, 384, 416], 'grid', pilot_runs=500)
    line = {'study': 'MLP surrogate', 'widths': list(S.WIDTHS), 'tuples': int(X.shape[0]),
            'lattices': ['%s %d' % t for t in lattices], 'p_per_lattice': P,
            'p_grid': 'half uniform, half in the finite-size transition window',
            'data_seconds': t_data, 'train_seconds': t_train, 'steps': steps, 'batch': batch,
            'loss_weights': ('1 / (se^2 + %g^2), standardised Monte Carlo standard errors'
                             % args.surrogate_se_floor if weighted else 'none'),
            'samples_per_s': steps * batch / t_train, 'loss_trace': trace,
            'held_out': 'square L=384, 8000 runs, 2001 p',
            'accepted_fraction_2se': acc, 'p_grid_gain_spanning': gains,
            'next_length': {'choice': nxt, 'mean_abs_z': scores, 'candidates': [352, 384, 416]}}
    print(json.dumps(line))
    return 0


def mlp_study(args):
    """Training throughput of the MLP surrogate's kernels (tcgen05 BF16
    GEMMs, GELU, loss, Adam): `args.steps` Adam steps of batch 4096 on
    20,000 synthetic rows after `args.warmup` warm-up steps."""
    import torch
    from pypercolate_gb300.surrogate import MLP, WIDTHS
    torch.cuda.set_device(0)
    rng = np.random.default_rng(0)
    X = rng.uniform(0, 1, size=(20000, WIDTHS[0])).astype(np.float32)
    Y = np.column_stack([np.tanh(8 * (X[:, 0] - 0.5)), X[:, 1] ** 2, np.sin(3 * X[:, 2])])
    model = MLP(seed=2)
    model.fit(X, Y, steps=max(1, args.warmup), batch=4096)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    trace = model.fit(X, Y, steps=args.steps, batch=4096, lr=1e-3, log_every=max(1, args.steps // 2))
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    print(json.dumps({'study': 'MLP training throughput', 'widths': list(WIDTHS), 'batch': 4096,
                      'steps': args.steps, 'samples_per_s': args.steps * 4096 / dt,
                      'ms_per_step': dt / args.steps * 1e3, 'final_loss': trace[-1][1],
                      'gemm': 'tcgen05.mma kind::f16 (BF16 operands, FP32 TMEM accumulator)'}))
    return 0


def main():
    args = parse()
    if args.impl == 'reference':
        return run_reference(args)
    if args.study == 'precision':
        return precision_study(args)
    if args.study == 'surrogate':
        return surrogate_study(args)
    if args.study == 'mlp':
        return mlp_study(args)
    import torch
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('nccl')
    from pypercolate_gb300 import _native as nat
    from pypercolate_gb300.ensemble import Ensemble

    L, R = args.L, args.runs
    if args.l2_fetch:
        nat.set_l2_fetch_granularity(args.l2_fetch)
    l2_fetch = nat.get_l2_fetch_granularity()
    ps = np.linspace(0.0, 1.0, args.P)
    # launch shapes from the autotuner, timed on this workload (before the
    # main ensemble holds its workspace)
    ens_tuned = None
    tuning, window = None, args.window
    if args.tune:
        from pypercolate_gb300.autotune import tune_ensemble
        ens_tuned = tune_ensemble(args.lattice, L, ps, R, precision=args.precision,
                                  micro=not args.no_micro, model=args.model, cache_path=None)
        tuning = ens_tuned['best']
        window = window or tuning['window']
    ens = Ensemble(args.lattice, L, ps, precision=args.precision, micro=not args.no_micro,
                   window=window, model=args.model, tuning=tuning)
    N, M = ens.N, ens.M  # M = number of steps (bonds, or sites for the site model)
    default_leg = args.lattice == 'grid' and args.model == 'bond'
    unit = 'bond additions/s' if args.model == 'bond' else 'site additions/s'
    if not default_leg:  # the extensions are measured on their own lattice only
        args.plain_runs = args.mix_runs = 0
    run_base = rank * 10 ** 9  # disjoint run ids per rank (weak scaling)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for w in range(args.warmup):
        ens.run(R, key=KEY, run0=run_base + w * R)
    torch.cuda.synchronize()
    nat.profile_read()
    nat.profile_enable(True)
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.steps):
        ens.run(R, key=KEY, run0=run_base + (args.warmup + k) * R)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    uf_errors = ens.errors()  # runs whose union-find state came out corrupt: 0
    nat.profile_enable(False)
    prof = nat.profile_read()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device='cuda')
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = R * M * world / (ms * 1e-3)
    merged_runs = None
    if world > 1:
        # the one exchange of the multi-GPU path, after timing: every rank's
        # ensemble state gathered and merged on the device (Ensemble.merge)
        from pypercolate_gb300.distributed import merged_ensemble
        merged_runs = int(merged_ensemble(ens).count.cpu().numpy()[0])

    # dominant kernel: union-find windows
    uf_n, uf_ms = prof['union_find']
    adds_per_launch = R * M / max(uf_n / args.steps, 1)
    uf_avg_s = uf_ms / max(uf_n, 1) * 1e-3
    uf_bytes = uf_bytes_per_add(N)
    achieved = uf_bytes * adds_per_launch / uf_avg_s / 1e9
    peak, peak_kind = peaks()
    launches = {k: v[0] for k, v in prof.items()}
    # second ceiling for the union-find: HBM's rate of scattered sector reads
    gather_rate = random_gather_rate()
    uf_adds_per_s = adds_per_launch / uf_avg_s
    # kernels per profiled launch sequence: set-up (band weights, FP32
    # weights, node and state initialisation), union-find, micro reductions,
    # convolution (FP32: max-set, other statistics, compensated m2; tf32x3:
    # tcgen05 kernel, compensated m2; FP64: max-set, other statistics),
    # reduction (micro count, two run-reduction passes, count)
    kernels_per_seq = {'setup': 3 if args.precision == 'fp64' else 4, 'union_find': 1, 'micro': 1,
                       'conv': {'fp32': 3, 'tf32x3': 2, 'fp64': 2}[args.precision], 'reduce': 4}
    gpu_launches = int(sum(launches[k] * kernels_per_seq[k] for k in launches))

    # per-curve error of the timed arithmetic against FP64, on a sample of
    # the timed runs (outside the timed region)
    curve_err = None
    if args.curve_sample > 0 and default_leg:
        curve_err = curve_errors_vs_fp64(L, ps, args.precision, min(args.curve_sample, R),
                                         run_base + args.warmup * R, bench_window(M, R, window))

    # plain GPU path (one lattice per launch): chunks of runs whose records for
    # all M+1 rows are materialised by one union-find launch, then reduced
    # and convolved by separate launches; same kernels and arithmetic as the
    # batched leg, without the window pipeline (nothing overlaps)
    plain = None
    if args.plain_runs > 0:
        chunk = min(args.plain_chunk, args.plain_runs)
        pe = Ensemble('grid', L, ps, precision=args.precision, micro=not args.no_micro, window=M + 1)
        pe.run(chunk, key=KEY, run0=run_base + 2 * 10 ** 8)  # warm-up
        torch.cuda.synchronize()
        nat.profile_read()
        nat.profile_enable(True)
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        done = 0
        while done < args.plain_runs:
            pe.run(chunk, key=KEY, run0=run_base + 3 * 10 ** 8 + done)
            done += chunk
        p1.record(stream)
        torch.cuda.synchronize()
        nat.profile_enable(False)
        pprof = nat.profile_read()
        pms = p0.elapsed_time(p1)
        puf_n, puf_ms = pprof['union_find']
        plain = {'value': done * M / (pms * 1e-3), 'unit': 'bond additions/s', 'runs': done,
                 'chunk': chunk, 'ms': pms, 'precision': args.precision,
                 'union_find_only': done * M / (puf_ms * 1e-3),
                 'kernel_ms': {k: v[1] for k, v in pprof.items()},
                 'path': 'records for all M+1 rows per union-find launch, consumers after it '
                         '(no overlap), same kernels and arithmetic as the batched leg'}
        del pe
        torch.cuda.empty_cache()

    # batched uneven workload: 10^6 runs, 2D L log-uniform in [8, 512] and
    # chains l log-uniform in [1024, 65536], 50/50, one persistent launch per
    # ensemble replayed as a CUDA graph; launch shape from the autotuner
    mix = None
    if args.mix_runs > 0:
        from pypercolate_gb300.autotune import tune_mix
        from pypercolate_gb300.mix import MixEnsemble
        tuned = tune_mix(args.mix_runs, cache_path=None)
        threads, block, smem, fused = tuned['best']
        me = MixEnsemble(args.mix_runs, threads=threads, block=block, smem_words=smem, fused=fused)
        me.capture()
        me.replay(7)
        torch.cuda.synchronize()
        m0e = torch.cuda.Event(enable_timing=True)
        m1e = torch.cuda.Event(enable_timing=True)
        m0e.record(stream)
        for k in range(2):
            me.replay(8 + k)
        m1e.record(stream)
        torch.cuda.synchronize()
        mms = m0e.elapsed_time(m1e) / 2
        adds = me.additions
        counts = me.count.cpu().numpy().astype(np.int64)
        mix = {'value': adds / (mms * 1e-3), 'unit': 'bond additions/s', 'runs': args.mix_runs,
               'additions_per_ensemble': adds, 'ms_per_ensemble': mms,
               'launch': {'threads': threads, 'block': block, 'smem_words': smem,
                          'reduction': 'fused' if fused else 'records'},
               'autotune': [list(t) for t in tuned['table']], 'cuda_graph': True,
               'workload': '2D L log-uniform [8,512] + chains l log-uniform [1024,65536], '
                           '50/50, 256 checkpoints, exact per-lattice reductions; union-find '
                           'and microcanonical checkpoint reductions only (no canonical '
                           'convolution), in both this leg and its plain leg'}
        del me
        torch.cuda.empty_cache()
        if args.plain_mix:
            mix['plain'] = plain_mix_leg(counts, stream, fused=fused)
            mix['batched_vs_plain'] = mix['value'] / mix['plain']['value']

    # end to end through the public API: inputs (p-grid) from pinned host
    # memory, results read back every step -- the finalized canonical
    # averages and, with the fused micro reductions on, the microcanonical
    # averages of every n (means and confidence bounds, 21 values per n)
    h_ps = torch.from_numpy(ps.copy()).pin_memory()
    h2d = h_ps.numel() * 8
    d2h = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.e2e_steps):
        e = Ensemble(args.lattice, L, h_ps.numpy(), precision=args.precision, model=args.model,
                     micro=not args.no_micro, window=window, tuning=tuning)
        e._ws = ens._ws  # reuse the device workspace
        e.d_ps.copy_(h_ps, non_blocking=True)
        e.run(R, key=KEY, run0=run_base + 10 ** 8 + k * R)
        fin = e.finalized(0.05)
        d2h = fin.nbytes + e.canonical_averages().nbytes
        if e.micro is not None:
            mic = e.microcanonical_averages(0.05)
            d2h += sum(v.nbytes for v in mic.values() if isinstance(v, np.ndarray))
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.e2e_steps
    e2e_value = R * M * world / e2e_s

    line = {
        'metric': unit, 'value': value, 'unit': unit,
        'n_gpus': world, 'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': ms,
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
        'dtype': 'int32 union-find, u64/u128 moments, %s convolution' % args.precision,
        'data': 'synthetic (Philox-4x32-10 keyed permutations, seed %d)' % KEY,
        'config': {'workload': '%s batched ensemble: %d runs/step/GPU, '
                               '%d uniform p in [0,1], fused micro reductions=%s'
                               % ('spanning_2d_grid(%d)' % L if default_leg else
                                  '%s %s percolation, L=%d' % (args.lattice, args.model, L),
                                  R, args.P, not args.no_micro),
                   'L': L, 'N': N, 'M': M, 'runs_per_step': R, 'P': args.P,
                   'precision': args.precision, 'l2_fetch_bytes': l2_fetch,
                   'l2': 'inputs larger than L2 (%.1f GB of union-find state per step)'
                         % (R * N * 4 / 1e9)},
        'roofline': {'bound': 'hbm', 'achieved': achieved, 'peak': peak, 'unit': 'GB/s',
                     'frac': achieved / peak, 'traffic': UF_TRAFFIC_PER_ADD * adds_per_launch,
                     'traffic_source': 'ncu dram__bytes_read.sum + dram__bytes_write.sum per '
                                       'addition on a 12,288-run capture, scaled to the '
                                       'launch by its additions',
                     'kernel': 'uf_window_kernel', 'peak_source': peak_kind,
                     'bytes_per_addition': uf_bytes,
                     'avg_launch_ms': uf_avg_s * 1e3,
                     'random_access': {
                         'gather_sectors_per_s': gather_rate,
                         'uf_read_sectors_per_s': uf_adds_per_s * UF_READ_PER_ADD / 32.0,
                         'frac': uf_adds_per_s * UF_READ_PER_ADD / 32.0 / gather_rate,
                         'note': 'ceiling = 4-B torch.index_select gathers at random positions of '
                                 'a 16 GiB array; union-find sector reads from the measured '
                                 '%.1f B read per addition' % UF_READ_PER_ADD}},
        'kernel_ms_per_step': {k: v[1] / args.steps for k, v in prof.items()},
        'plain_gpu': plain,
        'batched_uneven': mix,
        'batched_vs_plain': (value / world / plain['value']) if plain else None,
        'union_find_only': {'batched': uf_adds_per_s,
                            'plain': plain['union_find_only'] if plain else None},
        'curve_err_vs_fp64': curve_err,
        'clocks': clocks,
        'autotune': ({'best': ens_tuned['best'],
                      'table': [[c, ms] for c, ms in ens_tuned['table']],
                      'candidates_ms': 'one ensemble step of the workload per candidate '
                                       '(best of two after a warm-up step)'}
                     if ens_tuned else None),
        'gpu_launches': gpu_launches,
        'merged_runs': merged_runs,
        'union_find_errors': uf_errors,
        'e2e': {'value': e2e_value, 'unit': unit, 'h2d_bytes_per_step': h2d,
                'd2h_bytes_per_step': d2h},
    }
    if not default_leg:
        # the traffic figure and the CPU oracle pipeline are for the bond grid
        line['roofline']['kernel'] = ('torus_window_kernel' if args.lattice == 'torus'
                                      else 'site_window_kernel')
        line['roofline']['traffic'] = None
        line['roofline'].pop('random_access', None)
    if rank == 0:
        if default_leg:
            try:
                line['cpu_baseline'] = cpu_baseline(L, ps, args.cpu_sample)
            except Exception as exc:  # the oracle is a measurement aid only
                line['cpu_baseline'] = {'value': None, 'error': repr(exc)}
        else:
            line['cpu_baseline'] = None
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == '__main__':
    sys.exit(main())
