"""Autotuners for the two ensemble paths.

tune_mix       batched uneven ensembles (``nz_mix``): persistent threads
               (runs in flight), threads per CTA (runs per CTA), the
               shared-memory node slot per thread (placement: small lattices
               in shared memory, the rest in HBM / L2) and the reduction
               (per-run checkpoint records reduced by a second kernel, or
               fused into the union-find as exact integer atomics).
tune_ensemble  one lattice per ensemble (``nz_ensemble_tuned``): runs per
               CTA of the union-find, the probability tiles of the compensated
               m2 convolution and of the other statistics' convolution, the
               record window (rows reduced and convolved
               per pass: the reduction tiling over n) and the slices of runs
               of the canonical run reduction (its tiling over runs).

Each candidate runs the same workload, timed with CUDA events on the
launching stream; the fastest wins.  Results are cached in a JSON file keyed
by the GPU name and the workload, so later processes reuse the choice.
"""
import json
import os

import numpy as np

from . import _native as nat

DEFAULT_CACHE = os.path.join(os.path.expanduser('~'), '.cache', 'pypercolate_gb300',
                             'autotune.json')


def _candidates(nmax, free_bytes):
    """A compact grid: runs in flight x runs per CTA x shared-memory slot
    (64 words hold the grids up to L = 8, 128 words up to L = 10: the
    smallest lattices of the mix run out of shared memory)."""
    out = []
    for threads, block, smem in ((49152, 128, 0), (65536, 128, 0), (98304, 128, 0),
                                 (131072, 128, 0), (65536, 64, 0), (98304, 64, 0),
                                 (65536, 128, 64), (98304, 128, 128)):
        if 4 * nmax * threads <= 0.6 * free_bytes:
            out.append((threads, block, smem))
    return out or [(8192, 128, 0)]


def _key(spec_tuple):
    torch = nat.torch_cuda()
    return '%s|%s' % (torch.cuda.get_device_name(), ','.join(map(str, spec_tuple)))


def tune_mix(n_runs, grid=(8, 512), chain=(1024, 65536), chain_share=0.5, checkpoints=256,
             sample_runs=None, cache_path=DEFAULT_CACHE, candidates=None, key=7):
    """Best (threads, block, smem_words, fused) for this workload and the
    table of all timings: {'best': (...), 'table': [(threads, block, smem,
    fused, G adds/s), ...]}.  The launch shapes are timed with the records
    reduction; the fastest shape is then timed with the fused reduction too."""
    from .mix import MixEnsemble
    torch = nat.torch_cuda()
    spec = ('mix2', n_runs, grid[0], grid[1], chain[0], chain[1], chain_share, checkpoints)
    ck = _key(spec)
    cache = {}
    if cache_path and os.path.exists(cache_path):
        try:
            cache = json.load(open(cache_path))
        except (OSError, ValueError):
            cache = {}
    if ck in cache and candidates is None:
        hit = cache[ck]
        return {'best': tuple(hit['best']), 'table': hit['table'], 'cached': True}
    sample = int(min(n_runs, sample_runs or n_runs))
    nmax = max(grid[1] ** 2, chain[1])
    free, _ = torch.cuda.mem_get_info()
    cands = candidates or _candidates(nmax, free)

    def timed(threads, block, smem, fused):
        ens = MixEnsemble(sample, grid=grid, chain=chain, chain_share=chain_share,
                          checkpoints=checkpoints, threads=min(threads, sample), block=block,
                          smem_words=smem, fused=fused)
        ens.run(key)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        ens.run(key + 1)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        row = (threads, block, smem, fused, ens.additions / ms / 1e6)
        del ens
        torch.cuda.empty_cache()
        return row

    table = [timed(threads, block, smem, False) for threads, block, smem in cands]
    shape = max(table, key=lambda t: t[4])
    table.append(timed(shape[0], shape[1], shape[2], True))
    best = max(table, key=lambda t: t[4])
    result = {'best': tuple(best[:4]), 'table': table, 'cached': False}
    if cache_path:
        os.makedirs(os.path.dirname(cache_path), exist_ok=True)
        cache[ck] = {'best': list(best[:4]), 'table': table}
        with open(cache_path, 'w') as f:
            json.dump(cache, f, indent=1)
    return result


def default_window(M, n_runs):
    """Record-window rows nz_ensemble picks by itself: ~32 GiB of 36-byte
    records per window, 256 .. M + 1 rows."""
    return int(min(M + 1, max(256, 32.0 * (1 << 30) / (n_runs * 36))))


def ensemble_candidates(M, n_runs):
    """The library's defaults, then one launch-shape change at a time."""
    w = default_window(M, n_runs)
    base = {'uf_block': 128, 'm2_tile': 8, 'conv_tile': 8, 'taper': 0,
            'reduce_slices': 64 if n_runs >= 65536 else 16, 'window': w}
    out = [dict(base)]
    for key, vals in (('uf_block', (64, 32)), ('m2_tile', (16,)), ('conv_tile', (16,)), ('taper', (1,)),
                      ('window', (min(M + 1, max(256, w // 2)), min(M + 1, (3 * w) // 2))),
                      ('reduce_slices', (16 if base['reduce_slices'] != 16 else 64, 256))):
        for v in vals:
            c = dict(base)
            c[key] = int(v)
            if c not in out:
                out.append(c)
    return out


def combined_candidate(table):
    """From [(candidate, ms), ...] whose first row is the defaults and whose
    other rows each change the defaults: the defaults with every change that
    was faster than them, the fastest change applied last (so it wins where
    two changes set the same shape)."""
    base, base_ms = table[0]
    combo = dict(base)
    for cand, ms in sorted(table[1:], key=lambda t: -t[1]):  # the best change last
        if ms < base_ms:
            combo.update({k: v for k, v in cand.items() if v != base[k]})
    return combo


def _time_ensemble(kind, length, ps, n_runs, precision, micro, model, cand, key, reps, warm=False):
    """Best of `reps` CUDA-event timings (ms) of one ensemble step with the
    launch shapes `cand` (after an untimed step when `warm`: a process's
    first steps run slower -- module loading, cold TLBs)."""
    from .ensemble import Ensemble
    torch = nat.torch_cuda()
    stream = torch.cuda.current_stream()
    ens = Ensemble(kind, length, ps, precision=precision, micro=micro, window=cand['window'],
                   model=model, tuning=cand)
    ens._ws = nat.device_empty(ens.workspace_bytes(n_runs))  # allocated outside the timing
    if warm:
        ens.run(n_runs, key=key, run0=0)
    best_ms = None
    for rep in range(reps):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ens.run(n_runs, key=key, run0=(rep + 1) * n_runs)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best_ms = ms if best_ms is None else min(best_ms, ms)
    del ens
    torch.cuda.empty_cache()
    return best_ms


def tune_ensemble(kind, length, ps, n_runs, precision='fp32', micro=True, model='bond',
                  cache_path=DEFAULT_CACHE, candidates=None, key=5, reps=2):
    """Best launch shapes {'uf_block', 'm2_tile', 'conv_tile', 'taper',
    'reduce_slices', 'window'} for one ensemble step of n_runs runs of this
    lattice and p grid, and the table of all timings (the best of `reps`
    steps per candidate, after one untimed warm-up step; the last row
    combines every single change that beat the defaults):
    {'best': {...}, 'table': [({...}, ms), ...]}."""
    ps = np.asarray(ps, dtype=np.float64)
    spec = ('ensemble', kind, int(length), model, len(ps), float(ps.min()), float(ps.max()),
            int(n_runs), precision, bool(micro))
    ck = _key(spec)
    cache = {}
    if cache_path and os.path.exists(cache_path):
        try:
            cache = json.load(open(cache_path))
        except (OSError, ValueError):
            cache = {}
    if ck in cache and candidates is None:
        hit = cache[ck]
        return {'best': hit['best'], 'table': hit['table'], 'cached': True}
    table = []
    from .ensemble import lattice_kind
    from .hpc import GraphSpec
    M = GraphSpec(lattice_kind(kind, model), int(length)).M
    cands = candidates or ensemble_candidates(M, n_runs)
    for i, cand in enumerate(cands):
        table.append((dict(cand), _time_ensemble(kind, length, ps, n_runs, precision, micro, model,
                                                 cand, key, reps, warm=(i == 0))))
    if candidates is None and len(table) > 1:
        # the candidates change one shape at a time: also time every change
        # that beat the defaults, together
        combo = combined_candidate(table)
        if combo not in [c for c, _ in table]:
            table.append((combo, _time_ensemble(kind, length, ps, n_runs, precision, micro, model,
                                                combo, key, reps)))
    best = min(table, key=lambda t: t[1])[0]
    result = {'best': best, 'table': table, 'cached': False}
    if cache_path:
        os.makedirs(os.path.dirname(cache_path), exist_ok=True)
        cache[ck] = {'best': best, 'table': table}
        with open(cache_path, 'w') as f:
            json.dump(cache, f, indent=1)
    return result
