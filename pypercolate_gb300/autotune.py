"""Autotuner for the batched uneven ensembles (``nz_mix``).

Candidates are (persistent threads = runs in flight, threads per CTA,
shared-memory node slot per thread = placement).  Each candidate runs the
same workload on a sample of the runs, timed with CUDA events; the fastest
wins.  Results are cached in a JSON file keyed by the GPU name and the
workload, so later processes reuse the choice.
"""
import json
import os

import numpy as np

from . import _native as nat

DEFAULT_CACHE = os.path.join(os.path.expanduser('~'), '.cache', 'pypercolate_gb300',
                             'autotune.json')


def _candidates(nmax, free_bytes):
    """A compact grid: runs in flight x runs per CTA x shared-memory slot."""
    out = []
    for threads, block, smem in ((49152, 128, 0), (65536, 128, 0), (98304, 128, 0),
                                 (65536, 64, 0), (65536, 128, 64)):
        if 4 * nmax * threads <= 0.6 * free_bytes:
            out.append((threads, block, smem))
    return out or [(8192, 128, 0)]


def _key(spec_tuple):
    torch = nat.torch_cuda()
    return '%s|%s' % (torch.cuda.get_device_name(), ','.join(map(str, spec_tuple)))


def tune_mix(n_runs, grid=(8, 512), chain=(1024, 65536), chain_share=0.5, checkpoints=256,
             sample_runs=None, cache_path=DEFAULT_CACHE, candidates=None, key=7):
    """Best (threads, block, smem_words) for this workload and the table of
    all timings: {'best': (...), 'table': [(threads, block, smem, G adds/s), ...]}."""
    from .mix import MixEnsemble
    torch = nat.torch_cuda()
    spec = (n_runs, grid[0], grid[1], chain[0], chain[1], chain_share, checkpoints)
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
    table = []
    for threads, block, smem in cands:
        ens = MixEnsemble(sample, grid=grid, chain=chain, chain_share=chain_share,
                          checkpoints=checkpoints, threads=min(threads, sample), block=block,
                          smem_words=smem)
        ens.run(key)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        ens.run(key + 1)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        table.append((threads, block, smem, ens.additions / ms / 1e6))
        del ens
        torch.cuda.empty_cache()
    best = max(table, key=lambda t: t[3])
    result = {'best': tuple(best[:3]), 'table': table, 'cached': False}
    if cache_path:
        os.makedirs(os.path.dirname(cache_path), exist_ok=True)
        cache[ck] = {'best': list(best[:3]), 'table': table}
        with open(cache_path, 'w') as f:
            json.dump(cache, f, indent=1)
    return result
