"""ctypes bindings of libnzgb300.so (declared in include/nz_gb300.h).

Device memory and streams come from PyTorch (``torch.empty(..., device=
'cuda')`` and ``torch.cuda.current_stream()``); every computation is a call
into the library.  There is no CPU fallback: if the library cannot be loaded,
or no CUDA device is present, the functions raise.
"""
import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, '_lib', 'libnzgb300.so')

NZ_OK = 0
NZ_ERR_INVALID = 1
NZ_ERR_SPANNING_SIDES = 2
NZ_ERR_TOO_LARGE = 3
NZ_ERR_CUDA = 4
NZ_ERR_WORKSPACE = 5

GRAPH_GRID2D = 0
GRAPH_CHAIN1D = 1
GRAPH_EDGES = 2
GRAPH_TORUS2D = 3
KIND_MASK = 0xFF
MODEL_SITE = 0x100
WRAP = {'either': 0x000, 'x': 0x200, 'y': 0x400, 'both': 0x600}

PERM_PHILOX = 0
PERM_GIVEN = 1
PERM_MT19937 = 2

MAX_NODES = 1 << 21

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_vp = ctypes.c_void_p


class NzGraph(ctypes.Structure):
    _fields_ = [('kind', ctypes.c_int32), ('length', ctypes.c_uint32),
                ('num_nodes', ctypes.c_uint32), ('num_edges', ctypes.c_uint32),
                ('edge_u', _vp), ('edge_v', _vp), ('node_side', _vp)]


class NzRecords(ctypes.Structure):
    _fields_ = [('max_span', _vp), ('m0', _vp), ('m2', _vp), ('m3', _vp),
                ('m4_lo', _vp), ('m4_hi', _vp), ('edge', _vp),
                ('run_stride', ctypes.c_int64), ('site', ctypes.c_int32),
                ('narrow', ctypes.c_int32)]


class NzMicroAccum(ctypes.Structure):
    _fields_ = [('count', _vp), ('span_count', _vp), ('sum_lo', _vp),
                ('sum_hi', _vp), ('m2', _vp)]


class NzTuning(ctypes.Structure):
    _fields_ = [('uf_block', ctypes.c_int32), ('m2_tile', ctypes.c_int32),
                ('reduce_slices', ctypes.c_int32), ('conv_tile', ctypes.c_int32),
                ('taper', ctypes.c_int32)]


class NzMixSpec(ctypes.Structure):
    _fields_ = [('grid_min', ctypes.c_uint32), ('grid_max', ctypes.c_uint32),
                ('chain_min', ctypes.c_uint32), ('chain_max', ctypes.c_uint32),
                ('chain_share', ctypes.c_uint32), ('checkpoints', ctypes.c_int32),
                ('reduction', ctypes.c_int32)]


class NzMixAccum(ctypes.Structure):
    _fields_ = [('count', _vp), ('span', _vp), ('sum_lo', _vp), ('sum_hi', _vp), ('m2', _vp),
                ('errors', _vp)]


# (name, restype, argtypes) of every exported entry point
_SIGNATURES = [
    ('nz_version', ctypes.c_char_p, []),
    ('nz_status_string', ctypes.c_char_p, [ctypes.c_int]),
    ('nz_graph_size', ctypes.c_int, [ctypes.POINTER(NzGraph), _u32p, _u32p]),
    ('nz_microcanonical_workspace_bytes', ctypes.c_size_t,
     [ctypes.POINTER(NzGraph), ctypes.c_int32, ctypes.c_int32]),
    ('nz_microcanonical', ctypes.c_int,
     [ctypes.POINTER(NzGraph), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
      ctypes.c_uint64, ctypes.c_uint64, _vp, _vp, _vp, ctypes.c_int32, _vp,
      ctypes.c_size_t, ctypes.POINTER(NzRecords), _vp]),
    ('nz_microcanonical_noalloc', ctypes.c_int,
     [ctypes.POINTER(NzGraph), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
      ctypes.c_uint64, ctypes.c_uint64, _vp, _vp, _vp, ctypes.c_int32,
      ctypes.POINTER(NzRecords), _vp]),
    ('nz_static_scratch_bytes', ctypes.c_size_t, []),
    ('nz_permutations', ctypes.c_int,
     [ctypes.c_uint32, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_uint64,
      _vp, _vp, ctypes.c_int32, _vp, _vp]),
    ('nz_pack_microcanonical_rows', ctypes.c_int,
     [ctypes.POINTER(NzRecords), ctypes.c_int32, ctypes.c_uint32, ctypes.c_uint32,
      ctypes.c_int32, _vp, _vp]),
    ('nz_binomial_band_cap', ctypes.c_int32, [ctypes.c_uint32, ctypes.c_double]),
    ('nz_binomial_weights', ctypes.c_int,
     [ctypes.c_uint32, _vp, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, _vp, _vp,
      _vp, _vp]),
    ('nz_binomial_pmf', ctypes.c_int,
     [ctypes.c_uint32, _vp, ctypes.c_int32, _vp, _vp]),
    ('nz_band_dot', ctypes.c_int,
     [_vp, _vp, _vp, ctypes.c_int32, ctypes.c_int32, _vp, ctypes.c_uint32, ctypes.c_int32, _vp,
      _vp]),
    ('nz_canonical_statistics_rows', ctypes.c_int,
     [_vp, ctypes.c_uint32, ctypes.c_int32, _vp, ctypes.c_int32, _vp, _vp]),
    ('nz_canonical_statistics_records', ctypes.c_int,
     [ctypes.POINTER(NzRecords), ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32,
      ctypes.c_int32, _vp, _vp, _vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp]),
    ('nz_initialize_canonical_averages', ctypes.c_int,
     [_vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp]),
    ('nz_bond_reduce', ctypes.c_int,
     [_vp, _vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp]),
    ('nz_finalize_canonical_averages', ctypes.c_int,
     [_vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, _vp, ctypes.c_double, _vp,
      _vp]),
    ('nz_microcanonical_finalize', ctypes.c_int,
     [ctypes.POINTER(NzMicroAccum), ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32,
      ctypes.c_double, ctypes.c_int32, _vp, _vp]),
    ('nz_microcanonical_reduce', ctypes.c_int,
     [ctypes.POINTER(NzRecords), ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int32,
      ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(NzMicroAccum), _vp]),
    ('nz_canonical_merge', ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.c_int32, _vp]),
    ('nz_ensemble_errors', ctypes.c_int,
     [ctypes.POINTER(NzGraph), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, _vp, ctypes.c_size_t, _vp,
      _vp]),
    ('nz_micro_merge', ctypes.c_int,
     [ctypes.POINTER(NzMicroAccum), ctypes.POINTER(NzMicroAccum), ctypes.c_uint32, _vp]),
    ('nz_mt_stream_permutations', ctypes.c_int,
     [_vp, ctypes.c_uint32, ctypes.c_int32, _vp, _vp, _vp]),
    ('nz_student_t_quantile', ctypes.c_int, [_vp, _vp, ctypes.c_int32, _vp, _vp]),
    ('nz_mix_workspace_bytes', ctypes.c_size_t,
     [ctypes.POINTER(NzMixSpec), ctypes.c_int32, ctypes.c_int32]),
    ('nz_mix', ctypes.c_int,
     [ctypes.POINTER(NzMixSpec), _vp, _vp, _vp, ctypes.c_int32, ctypes.c_int32,
      ctypes.c_int32, ctypes.c_uint32, _vp, ctypes.c_size_t, ctypes.POINTER(NzMixAccum), _vp]),
    ('nz_mlp_param_count', ctypes.c_int64, [_vp, ctypes.c_int32]),
    ('nz_mlp_activation_count', ctypes.c_int64, [_vp, ctypes.c_int32, ctypes.c_int32]),
    ('nz_mlp_params_to_bf16', ctypes.c_int, [_vp, ctypes.c_int64, _vp, _vp]),
    ('nz_mlp_forward', ctypes.c_int,
     [_vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ('nz_mlp_loss', ctypes.c_int,
     [_vp, _vp, _vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp, ctypes.c_int32, _vp]),
    ('nz_mlp_backward', ctypes.c_int,
     [_vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ('nz_mlp_take_errors', ctypes.c_int, [_vp]),
    ('nz_mlp_adam', ctypes.c_int,
     [_vp, _vp, _vp, _vp, _vp, ctypes.c_int64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
      ctypes.c_float, ctypes.c_int32, _vp]),
    ('nz_set_l2_fetch_granularity', ctypes.c_int, [ctypes.c_int32]),
    ('nz_get_l2_fetch_granularity', ctypes.c_int, [_vp]),
    ('nz_profile_enable', None, [ctypes.c_int32]),
    ('nz_profile_read', ctypes.c_int, [ctypes.c_int32, _vp, _vp]),
    ('nz_ensemble_workspace_bytes', ctypes.c_size_t,
     [ctypes.POINTER(NzGraph), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    ('nz_ensemble', ctypes.c_int,
     [ctypes.POINTER(NzGraph), ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64,
      ctypes.c_uint64, _vp, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
      ctypes.c_int32, _vp, ctypes.c_size_t, _vp, _vp, _vp,
      ctypes.POINTER(NzMicroAccum), _vp]),
    ('nz_ensemble_tuned', ctypes.c_int,
     [ctypes.POINTER(NzGraph), ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64,
      ctypes.c_uint64, _vp, ctypes.c_int32, ctypes.c_double, ctypes.c_int32,
      ctypes.c_int32, ctypes.POINTER(NzTuning), _vp, ctypes.c_size_t, _vp, _vp, _vp,
      ctypes.POINTER(NzMicroAccum), _vp]),
]

EXPORTED = [name for name, _, _ in _SIGNATURES]

_lib = None
_lock = threading.Lock()


class NzError(RuntimeError):
    """A library call returned a status other than NZ_OK."""

    def __init__(self, status, where):
        self.status = status
        msg = lib_handle().nz_status_string(status).decode()
        super().__init__('%s: %s (status %d)' % (where, msg, status))


def lib_handle(build_if_missing=True):
    """Load libnzgb300.so (building it with nvcc if it is absent)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                if not build_if_missing:
                    raise ImportError('libnzgb300.so is not built (%s)' % LIB_PATH)
                from . import build as _build
                _build.build()
            lib = ctypes.CDLL(LIB_PATH)
            for name, res, args in _SIGNATURES:
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def set_l2_fetch_granularity(nbytes):
    """Context-wide L2 fetch granularity hint (0, 32, 64, 128 bytes)."""
    torch_cuda()
    check(lib_handle().nz_set_l2_fetch_granularity(int(nbytes)), 'nz_set_l2_fetch_granularity')


def get_l2_fetch_granularity():
    torch_cuda()
    v = ctypes.c_int32()
    check(lib_handle().nz_get_l2_fetch_granularity(ctypes.byref(v)), 'nz_get_l2_fetch_granularity')
    return v.value


PROF_CATEGORIES = ('setup', 'union_find', 'micro', 'conv', 'reduce')


def profile_enable(flag=True):
    lib_handle().nz_profile_enable(1 if flag else 0)


def profile_read():
    """{category: (launch sequences, total ms)} since the last read."""
    n = len(PROF_CATEGORIES)
    launches = np.zeros(n, dtype=np.int64)
    ms = np.zeros(n, dtype=np.float64)
    check(lib_handle().nz_profile_read(n, launches.ctypes.data_as(_vp), ms.ctypes.data_as(_vp)),
          'nz_profile_read')
    return {c: (int(launches[i]), float(ms[i])) for i, c in enumerate(PROF_CATEGORIES)}


def check(status, where):
    if status == NZ_OK:
        return
    if status in (NZ_ERR_INVALID, NZ_ERR_SPANNING_SIDES):
        msg = lib_handle().nz_status_string(status).decode()
        raise ValueError('%s: %s' % (where, msg))
    raise NzError(status, where)


# ---------------------------------------------------------------------------
# device plumbing (PyTorch is used for memory and streams only)
# ---------------------------------------------------------------------------
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError('pypercolate_gb300 needs a CUDA device (GB300, sm_103a); '
                           'there is no CPU fallback')
    return torch


def stream_handle(stream=None):
    torch = torch_cuda()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def device_empty(nbytes, align_elems=1):
    torch = torch_cuda()
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device='cuda')


def to_device(arr):
    """Copy a numpy array (any dtype, incl. structured) to a device byte buffer."""
    torch = torch_cuda()
    a = np.ascontiguousarray(arr)
    raw = a.view(np.uint8).reshape(-1) if a.size else np.zeros(1, np.uint8)
    return torch.from_numpy(raw.copy()).to('cuda')


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def to_host(t, dtype, shape):
    """Device byte buffer -> numpy array of the given dtype/shape."""
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    raw = t[:n].cpu().numpy() if n else np.zeros(0, np.uint8)
    return raw.view(dtype).reshape(shape).copy()


def make_graph(kind, length=0, num_nodes=0, num_edges=0, edge_u=None, edge_v=None,
               node_side=None):
    g = NzGraph()
    g.kind = kind
    g.length = int(length)
    g.num_nodes = int(num_nodes)
    g.num_edges = int(num_edges)
    g.edge_u = ptr(edge_u).value if edge_u is not None else None
    g.edge_v = ptr(edge_v).value if edge_v is not None else None
    g.node_side = ptr(node_side).value if node_side is not None else None
    return g


def graph_size(g):
    n = ctypes.c_uint32()
    m = ctypes.c_uint32()
    check(lib_handle().nz_graph_size(ctypes.byref(g), ctypes.byref(n), ctypes.byref(m)),
          'nz_graph_size')
    return n.value, m.value


class Records:
    """Device record planes for n_runs runs over `rows` rows (n-major)."""

    def __init__(self, rows, n_runs, with_edge=False, site=False):
        torch = torch_cuda()
        cnt = int(rows) * int(n_runs)
        self.site = bool(site)
        self.rows = int(rows)
        self.n_runs = int(n_runs)
        self.max_span = torch.empty(max(cnt, 1), dtype=torch.int32, device='cuda')
        self.m0 = torch.empty(max(cnt, 1), dtype=torch.int32, device='cuda')
        self.m2 = torch.empty(max(cnt, 1), dtype=torch.int64, device='cuda')
        self.m3 = torch.empty(max(cnt, 1), dtype=torch.int64, device='cuda')
        self.m4_lo = torch.empty(max(cnt, 1), dtype=torch.int64, device='cuda')
        self.m4_hi = torch.empty(max(cnt, 1), dtype=torch.int32, device='cuda')
        self.edge = torch.empty(max(cnt, 1), dtype=torch.int32, device='cuda') if with_edge else None

    def struct(self):
        r = NzRecords()
        r.max_span = self.max_span.data_ptr()
        r.m0 = self.m0.data_ptr()
        r.m2 = self.m2.data_ptr()
        r.m3 = self.m3.data_ptr()
        r.m4_lo = self.m4_lo.data_ptr()
        r.m4_hi = self.m4_hi.data_ptr()
        r.edge = self.edge.data_ptr() if self.edge is not None else None
        r.run_stride = self.n_runs
        r.site = int(self.site)
        return r

    def host(self):
        """Planes as numpy arrays shaped (rows, n_runs)."""
        shp = (self.rows, self.n_runs)
        cnt = self.rows * self.n_runs

        def h(t, dt):
            return t[:cnt].cpu().numpy().view(dt).reshape(shp)
        out = {
            'max_span': h(self.max_span, np.uint32),
            'm0': h(self.m0, np.uint32),
            'm2': h(self.m2, np.uint64),
            'm3': h(self.m3, np.uint64),
            'm4_lo': h(self.m4_lo, np.uint64),
            'm4_hi': h(self.m4_hi, np.uint32),
        }
        if self.edge is not None:
            out['edge'] = h(self.edge, np.uint32)
        return out
