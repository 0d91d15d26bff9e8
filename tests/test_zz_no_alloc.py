"""The no-allocation variant of the microcanonical entry point.

Some callers of this library cannot allocate device memory: a host framework
that owns the whole device pool and hands out only its own buffers, or a
foreign-language binding that can pass pointers to buffers it already holds
but has no way to get new ones.  ``nz_microcanonical_noalloc`` serves them by
keeping the union-find scratch in a fixed 64 MiB array inside the library
instead of a caller-provided workspace.

These tests call it through the C ABI and require its records to equal those
of ``nz_microcanonical`` (which takes caller-provided scratch) exactly -- the
records are integers -- on two calls in a row, for the three permutation
sources and for an explicit edge list.  The file sorts last so that a run
stopping at the first failure has already run every other test.
"""
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


def _run(nat, spec, spanning, n_runs, mode, key=0, run0=0, perms=None, seeds=None, noalloc=False):
    """Records of one call of either entry point, as host arrays."""
    import torch
    lib = nat.lib_handle()
    g = spec.struct()
    rec = nat.Records(spec.M + 1, n_runs, with_edge=True)
    keep = []
    d_perm = d_words = d_len = None
    stride = 1
    if perms is not None:
        d_perm = nat.to_device(np.ascontiguousarray(perms, dtype=np.uint32))
    if seeds is not None:
        words = np.asarray(seeds, dtype=np.uint32).reshape(n_runs, 1)
        d_words = nat.to_device(words)
        d_len = nat.to_device(np.zeros(n_runs, dtype=np.int32))
    keep += [d_perm, d_words, d_len]
    rs = rec.struct()
    if noalloc:
        st = lib.nz_microcanonical_noalloc(g, int(spanning), n_runs, mode, key, run0,
                                           nat.ptr(d_perm), nat.ptr(d_words), nat.ptr(d_len),
                                           stride, rs, nat.stream_handle())
    else:
        ws_bytes = lib.nz_microcanonical_workspace_bytes(g, n_runs, mode)
        ws = nat.device_empty(ws_bytes)
        keep.append(ws)
        st = lib.nz_microcanonical(g, int(spanning), n_runs, mode, key, run0, nat.ptr(d_perm),
                                   nat.ptr(d_words), nat.ptr(d_len), stride, nat.ptr(ws),
                                   ws_bytes, rs, nat.stream_handle())
    assert st == nat.NZ_OK, st
    torch.cuda.synchronize()
    return rec.host()


def _assert_same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_noalloc_matches_workspace_entry_point_philox(gpu):
    from pypercolate_gb300 import hpc
    spec = hpc.GraphSpec(gpu.GRAPH_GRID2D, 32)
    for key in (1234, 99):  # two calls in a row on the shared array
        want = _run(gpu, spec, True, 40, gpu.PERM_PHILOX, key=key, run0=7)
        got = _run(gpu, spec, True, 40, gpu.PERM_PHILOX, key=key, run0=7, noalloc=True)
        _assert_same(got, want)


def test_noalloc_matches_workspace_entry_point_mt19937(gpu):
    from pypercolate_gb300 import hpc
    spec = hpc.GraphSpec(gpu.GRAPH_GRID2D, 16)
    for seeds in ([0, 42, 4294967295], [5, 6, 7]):
        want = _run(gpu, spec, True, 3, gpu.PERM_MT19937, seeds=seeds)
        got = _run(gpu, spec, True, 3, gpu.PERM_MT19937, seeds=seeds, noalloc=True)
        _assert_same(got, want)


def test_noalloc_matches_workspace_entry_point_edge_list(gpu):
    from pypercolate_gb300 import hpc
    z = load_golden('kat_3x3.npz')
    spec = hpc.GraphSpec(gpu.GRAPH_EDGES, 0, 9, 12, z['eu'], z['ev'], z['side'])
    perms = np.stack([z['perm'], z['perm'][::-1]])
    for _ in range(2):
        want = _run(gpu, spec, True, 2, gpu.PERM_GIVEN, perms=perms)
        got = _run(gpu, spec, True, 2, gpu.PERM_GIVEN, perms=perms, noalloc=True)
        _assert_same(got, want)
    assert np.array_equal(got['max_span'][:, 0] & 0x7fffffff, z['test_max'])


def test_noalloc_refuses_requests_beyond_its_array(gpu):
    from pypercolate_gb300 import hpc
    lib = gpu.lib_handle()
    limit = lib.nz_static_scratch_bytes()
    assert limit == 64 << 20
    spec = hpc.GraphSpec(gpu.GRAPH_GRID2D, 256)
    g = spec.struct()
    assert lib.nz_microcanonical_workspace_bytes(g, 256, gpu.PERM_PHILOX) > limit
    rec = gpu.Records(1, 1)  # never written: the size check comes first
    st = lib.nz_microcanonical_noalloc(g, 1, 256, gpu.PERM_PHILOX, 0, 0, None, None, None, 1,
                                       rec.struct(), gpu.stream_handle())
    assert st == gpu.NZ_ERR_TOO_LARGE


def test_noalloc_call_allocates_no_device_memory(gpu):
    """Device memory in use, as the driver and torch's allocator see it, is
    the same before and after a call (once the library's kernels are loaded
    by a first call), with the per-kernel timing instrumentation off: that
    instrumentation creates CUDA events and is not for this path."""
    import torch
    from pypercolate_gb300 import hpc
    lib = gpu.lib_handle()
    gpu.profile_enable(False)
    spec = hpc.GraphSpec(gpu.GRAPH_GRID2D, 24)
    n_runs = 33
    g = spec.struct()
    rec = gpu.Records(spec.M + 1, n_runs, with_edge=True)
    rs = rec.struct()

    def call(key):
        st = lib.nz_microcanonical_noalloc(g, 1, n_runs, gpu.PERM_PHILOX, key, 0, None, None, None,
                                           1, rs, gpu.stream_handle())
        assert st == gpu.NZ_OK, st
        torch.cuda.synchronize()

    call(1)  # loads the kernels and takes the array's address in this context
    free0, _ = torch.cuda.mem_get_info()
    used0 = torch.cuda.memory_allocated()
    reserved0 = torch.cuda.memory_reserved()
    call(2)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_allocated() == used0
    assert torch.cuda.memory_reserved() == reserved0
    # and the records are those of the workspace entry point
    got = rec.host()
    want = _run(gpu, spec, True, n_runs, gpu.PERM_PHILOX, key=2)
    _assert_same(got, want)
