"""ctypes binding of libpmx.so (the C ABI declared in include/pmx.h).

The product path always runs the CUDA library: if it is missing or a call
fails, an error is raised -- there is no CPU fallback.
"""

import ctypes
import os
import threading

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, 'libpmx.so')

c_f = ctypes.c_float
c_d = ctypes.c_double
c_i64 = ctypes.c_int64
c_i32 = ctypes.c_int32
c_p = ctypes.c_void_p
c_int = ctypes.c_int


class EnmeshSpec(ctypes.Structure):
    """``pmx_enmesh_spec`` (include/pmx.h)."""
    _fields_ = [('dim', c_i32), ('wrap_shape', c_i32 * 3), ('mesh_shape', c_i64 * 3),
                ('conf_cell_size', c_d), ('offset', c_d * 3), ('cell_size', c_d),
                ('drop', c_i32)]


class PmxSim(ctypes.Structure):
    """``pmx_sim`` (include/pmx.h): one simulation of a batched call."""
    _fields_ = [('pmid', c_p), ('disp', c_p), ('vel', c_p), ('acc', c_p), ('disp_cot', c_p),
                ('vel_cot', c_p), ('acc_cot', c_p), ('n', c_i64), ('ptcl_num', c_i64),
                ('omega_m', c_d), ('factors', c_p), ('dots', c_p)]


# name -> (restype, argtypes); every entry point of include/pmx.h
SIGNATURES = {
    'pmx_version': (c_int, []),
    'pmx_last_error': (ctypes.c_char_p, []),
    'pmx_device_sms': (c_int, [ctypes.POINTER(c_int)]),
    'pmx_stream_create': (c_int, [c_int, ctypes.POINTER(c_p)]),
    'pmx_stream_destroy': (c_int, [c_p]),
    'pmx_enmesh': (c_int, [ctypes.POINTER(EnmeshSpec), c_p, c_p, c_i64, c_p, c_p, c_p, c_p]),
    'pmx_scatter': (c_int, [ctypes.POINTER(EnmeshSpec), c_p, c_p, c_i64, c_p, c_f, c_i64, c_p, c_p]),
    'pmx_scatter_adj': (c_int, [ctypes.POINTER(EnmeshSpec), c_p, c_p, c_i64, c_p, c_f, c_i64, c_p,
                                c_p, c_p, c_p]),
    'pmx_gather': (c_int, [ctypes.POINTER(EnmeshSpec), c_p, c_p, c_i64, c_p, c_i64, c_p, c_f, c_p,
                           c_p]),
    'pmx_gather_adj': (c_int, [ctypes.POINTER(EnmeshSpec), c_p, c_p, c_i64, c_p, c_i64, c_p, c_p,
                               c_p, c_p]),
    'pmx_workspace_bytes': (c_int, [ctypes.POINTER(c_i64), c_i32, ctypes.POINTER(ctypes.c_size_t)]),
    'pmx_workspace_create': (c_int, [ctypes.POINTER(c_i64), c_i32, ctypes.POINTER(c_p)]),
    'pmx_workspace_destroy': (c_int, [c_p]),
    'pmx_workspace_create_batch': (c_int, [ctypes.POINTER(c_i64), c_i32, c_i32,
                                           ctypes.POINTER(c_p)]),
    'pmx_workspace_slots': (c_int, [c_p, ctypes.POINTER(c_i32)]),
    'pmx_workspace_tma_status': (c_int, [c_p, ctypes.POINTER(c_i32)]),
    'pmx_nbody_steps_batch': (c_int, [c_p, ctypes.POINTER(EnmeshSpec), c_i32,
                                      ctypes.POINTER(PmxSim), c_i32, c_i32, c_p]),
    'pmx_nbody_adj_steps_batch': (c_int, [c_p, ctypes.POINTER(EnmeshSpec), c_i32,
                                          ctypes.POINTER(PmxSim), c_i32, c_i32, c_p]),
    'pmx_force': (c_int, [c_p, ctypes.POINTER(EnmeshSpec), c_p, c_p, c_i64, c_i64, c_d, c_p, c_p]),
    'pmx_force_vjp': (c_int, [c_p, ctypes.POINTER(EnmeshSpec), c_p, c_p, c_i64, c_i64, c_d, c_p,
                              c_p, c_p, c_p, c_p]),
    'pmx_kick': (c_int, [c_p, c_p, c_i64, c_f, c_p]),
    'pmx_drift': (c_int, [c_p, c_p, c_i64, c_f, c_p]),
    'pmx_kick_adj': (c_int, [c_p, c_p, c_p, c_p, c_p, c_i64, c_f, c_p, c_p]),
    'pmx_drift_adj': (c_int, [c_p, c_p, c_p, c_p, c_i64, c_f, c_p, c_p]),
    'pmx_dot': (c_int, [c_p, c_p, c_i64, c_p, c_p]),
    'pmx_dot_noalloc': (c_int, [c_p, c_p, c_i64, c_p, c_p]),
    'pmx_nbody_step': (c_int, [c_p, ctypes.POINTER(EnmeshSpec), c_p, c_p, c_p, c_p, c_i64, c_i64,
                               ctypes.POINTER(c_f), c_d, c_p]),
    'pmx_nbody_adj_step': (c_int, [c_p, ctypes.POINTER(EnmeshSpec), c_p, c_p, c_p, c_p, c_p, c_p,
                                   c_p, c_i64, c_i64, ctypes.POINTER(c_f), c_d, c_p, c_p]),
    'pmx_nbody_step_kahan': (c_int, [c_p, ctypes.POINTER(EnmeshSpec), c_p, c_p, c_p, c_p, c_p,
                                     c_p, c_i64, c_i64, ctypes.POINTER(c_f), c_d, c_p]),
    'pmx_nbody_adj_step_kahan': (c_int, [c_p, ctypes.POINTER(EnmeshSpec), c_p, c_p, c_p, c_p, c_p,
                                         c_p, c_p, c_p, c_p, c_i64, c_i64, ctypes.POINTER(c_f),
                                         c_d, c_p, c_p]),
    'pmx_nbody_steps': (c_int, [c_p, ctypes.POINTER(EnmeshSpec), c_p, c_p, c_p, c_p, c_i64, c_i64,
                                c_i32, c_p, c_d, c_p]),
    'pmx_nbody_adj_steps': (c_int, [c_p, ctypes.POINTER(EnmeshSpec), c_p, c_p, c_p, c_p, c_p, c_p,
                                    c_p, c_i64, c_i64, c_i32, c_p, c_d, c_p, c_p]),
    'pmx_powspec_bin': (c_int, [c_p, c_p, c_i64, ctypes.POINTER(c_i64), c_p, c_p, c_p, c_p, c_i32,
                                c_i32, c_i32, c_d, c_p, c_p, c_p, c_p]),
    'pmx_powspec_bin_zmajor': (c_int, [c_p, c_p, c_i64, ctypes.POINTER(c_i64), c_p, c_p, c_p, c_p,
                                       c_i32, c_i32, c_i32, c_d, c_p, c_p, c_p, c_p]),
    'pmx_growth_ode': (c_int, [c_p, c_i64, c_p, c_i64, c_d, c_d, c_p, c_p]),
    'pmx_random_bits': (c_int, [ctypes.c_uint32, ctypes.c_uint32, c_i64, c_int, c_p, c_p]),
    'pmx_normal': (c_int, [ctypes.c_uint32, ctypes.c_uint32, c_i64, c_int, c_p, c_p]),
    'pmx_profile_enable': (c_int, [c_p, c_int]),
    'pmx_profile_read': (c_int, [c_p, ctypes.POINTER(c_d), ctypes.POINTER(c_i64),
                                 ctypes.POINTER(c_i64)]),
    'pmx_profile_stage_name': (ctypes.c_char_p, [c_int]),
}

PROF_STAGES = 15


def profile_read(ws):
    """{stage: (ms, calls)} and the libpmx launch count since the last read."""
    lib = load()
    ms = (c_d * PROF_STAGES)()
    calls = (c_i64 * PROF_STAGES)()
    launches = c_i64()
    check(lib.pmx_profile_read(ws.handle, ms, calls, ctypes.byref(launches)), 'pmx_profile_read')
    out = {}
    for i in range(PROF_STAGES):
        out[lib.pmx_profile_stage_name(i).decode()] = (ms[i], calls[i])
    return out, launches.value

PMX_WS_ADJOINT = 1
PMX_WS_CUFFT3D = 2
PMX_WS_WINDOW = 4
PMX_WS_PLANE = 8
PMX_WS_VEC = 16
PMX_WS_NO_GRAPH = 32
PMX_WS_PLANE16 = 64
PMX_WS_AGG = 128
PMX_WS_TMA = 1 << 16
PMX_WS_CHAINS_SHIFT = 8
PMX_WS_SLAB_SHIFT = 12

_lib = None
_lock = threading.Lock()


class PmxError(RuntimeError):
    pass


def load(path=LIB_PATH):
    """Load libpmx.so (once) and declare every signature."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise PmxError(f'{path} is missing: run `python -c "import __graft_entry__ as g; '
                           f'g.build()"` (or pmwd_gb300/_build.py) first; the CUDA library is '
                           f'required, there is no CPU fallback')
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status, what=''):
    if status != 0:
        msg = load().pmx_last_error().decode(errors='replace')
        raise PmxError(f'{what} failed with status {status}: {msg}')


def call(name, *args):
    """Call an entry point.  Tensor arguments are passed as device pointers
    and stay referenced until the call has enqueued its work, so a temporary
    cannot be freed (and its memory reused by the caching allocator) before
    the kernels that read it are on the stream."""
    keep = [a for a in args if torch.is_tensor(a)]
    conv = [c_p(a.data_ptr()) if torch.is_tensor(a) else a for a in args]
    check(getattr(load(), name)(*conv), name)
    del keep


def ptr(t):
    """Device pointer of a tensor (None -> NULL)."""
    if t is None:
        return None
    return c_p(t.data_ptr())


def stream_ptr(device=None):
    return c_p(torch.cuda.current_stream(device).cuda_stream)


_LIB_STREAMS = {}
_LIB_STREAM_LOCK = threading.Lock()


def lib_stream(device):
    """A non-blocking CUDA stream that the library created on ``device``
    (``pmx_stream_create``; one per device, kept for the life of the
    process), as a ``torch.cuda.ExternalStream``.  ``torch.cuda.Stream()``
    hands out streams from a fixed pool (32 per device), so a pooled stream
    may be the very stream another thread launches its work on, and a graph
    captured on it would record that work too; this stream is never handed
    to anyone else."""
    dev = torch.device(device)
    idx = dev.index if dev.index is not None else torch.cuda.current_device()
    with _LIB_STREAM_LOCK:
        s = _LIB_STREAMS.get(idx)
        if s is None:
            h = c_p()
            check(load().pmx_stream_create(idx, ctypes.byref(h)), 'pmx_stream_create')
            s = torch.cuda.ExternalStream(h.value, device=torch.device('cuda', idx))
            _LIB_STREAMS[idx] = s
    return s


def make_spec(dim, wrap_shape, mesh_shape, conf_cell_size, offset=0, cell_size=None, drop=True):
    """``pmx_enmesh_spec``; ``wrap_shape=None``: no periodic wrapping."""
    s = EnmeshSpec()
    s.dim = dim
    s.drop = int(bool(drop))
    off = offset
    if not hasattr(off, '__len__'):
        off = (float(off),) * dim
    off = [float(x) for x in off]
    for a in range(3):
        s.wrap_shape[a] = (0 if wrap_shape is None else int(wrap_shape[a])) if a < dim else 1
        s.mesh_shape[a] = int(mesh_shape[a]) if a < dim else 1
        s.offset[a] = off[a] if a < dim else 0.0
    s.conf_cell_size = float(conf_cell_size)
    s.cell_size = -1.0 if cell_size is None else float(cell_size)
    return s


class Workspace:
    """Owner of a ``pmx_workspace`` (mesh buffers, spectra, cuFFT plans)."""

    def __init__(self, mesh_shape, adjoint=True, device=None, cufft3d=False, window=False,
                 plane=False, vec=False, graphs=True, plane16=False, chains=0, slab_log2=0,
                 slots=1, agg=False, tma=False):
        """Flags of pmx_workspace_create (include/pmx.h): ``cufft3d`` 3-D
        cuFFT plans instead of the fused x pass, ``window`` warp-window
        deposits, ``plane`` cluster plane kernels (``plane16``: clusters of
        16), ``vec`` vector z-pair reductions, ``agg`` warp-aggregated
        deposits, ``tma`` TMA-staged forward gathers, ``graphs`` slab loops as CUDA
        graphs, ``chains`` concurrent slab chains and ``slab_log2`` planes
        per cuFFT execution (0: defaults).  ``slots`` > 1: a batched
        workspace for that many simulations of this mesh shape
        (pmx_workspace_create_batch)."""
        load()
        self.mesh_shape = tuple(int(s) for s in mesh_shape)
        self.adjoint = adjoint
        flags = ((PMX_WS_ADJOINT if adjoint else 0) | (PMX_WS_CUFFT3D if cufft3d else 0)
                 | (PMX_WS_WINDOW if window else 0) | (PMX_WS_PLANE if plane else 0)
                 | (PMX_WS_VEC if vec else 0) | (0 if graphs else PMX_WS_NO_GRAPH)
                 | (PMX_WS_PLANE16 if plane16 else 0) | (PMX_WS_AGG if agg else 0)
                 | (PMX_WS_TMA if tma else 0)
                 | ((int(chains) & 7) << PMX_WS_CHAINS_SHIFT)
                 | ((int(slab_log2) & 15) << PMX_WS_SLAB_SHIFT))
        self.device = torch.device('cuda', torch.cuda.current_device() if device is None else device)
        shp = (c_i64 * 3)(*self.mesh_shape)
        h = c_p()
        self.slots = int(slots)
        with torch.cuda.device(self.device):
            if self.slots == 1:
                check(_lib.pmx_workspace_create(shp, flags, ctypes.byref(h)),
                      'pmx_workspace_create')
            else:
                check(_lib.pmx_workspace_create_batch(shp, flags, self.slots, ctypes.byref(h)),
                      'pmx_workspace_create_batch')
        self.handle = h

    def __del__(self):
        h = getattr(self, 'handle', None)
        if h is not None and _lib is not None:
            try:
                with torch.cuda.device(self.device):
                    _lib.pmx_workspace_destroy(h)
            except Exception:
                pass
            self.handle = None


_ws_cache = {}


def workspace(mesh_shape, adjoint=True, device=None):
    """Cached workspace per (device, mesh shape).  New workspaces are always
    created with the adjoint buffers, so one allocation serves forward and
    backward calls; ``adjoint=False`` only means the caller needs no more
    than the forward buffers."""
    dev = torch.cuda.current_device() if device is None else device
    key = (dev, tuple(mesh_shape))
    ws = _ws_cache.get(key)
    if ws is None or (adjoint and not ws.adjoint):
        _ws_cache.pop(key, None)
        ws = Workspace(mesh_shape, adjoint=True, device=dev)
        _ws_cache[key] = ws
    return ws


def release_workspaces():
    _ws_cache.clear()
