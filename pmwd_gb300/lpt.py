"""Lagrangian perturbation theory initial conditions (pmwd/lpt.py:1-212),
torch on the GPU (cuFFT through torch.fft; autograd gives its VJP)."""

import math
import threading
from collections import OrderedDict
from itertools import combinations, permutations

import torch

from . import _hostmath, _lib
from .boltzmann import growth
from .cosmology import E2
from .gravity import laplace, neg_grad
from .particles import Particles
from .pm_util import fftfreq, fftfwd, fftinv


def _strain(kvec, i, j, pot, conf):
    """LPT strain component from a scalar potential (lpt.py:13-37); the
    Nyquist planes are zeroed only when i != j."""
    k_i, k_j = kvec[i], kvec[j]
    nyquist = math.pi / conf.ptcl_spacing
    eps = nyquist * torch.finfo(torch.float32).eps
    if i != j:
        k_i = torch.where(torch.abs(torch.abs(k_i) - nyquist) <= eps, torch.zeros_like(k_i), k_i)
        k_j = torch.where(torch.abs(torch.abs(k_j) - nyquist) <= eps, torch.zeros_like(k_j), k_j)
    strain = -k_i * k_j * pot
    return fftinv(strain, shape=conf.ptcl_grid_shape).to(torch.float32)


def _nyq_zeroed(k, conf):
    nyquist = math.pi / conf.ptcl_spacing
    eps = nyquist * torch.finfo(torch.float32).eps
    return torch.where(torch.abs(torch.abs(k) - nyquist) <= eps, torch.zeros_like(k), k)


def _L3(kvec, pot, conf):
    """2nd-order source of one potential in 3-D (lpt.py:40-76 with m = n):
    the six strain fields come from one batched inverse FFT (each diagonal
    strain once), and the products are summed in the reference's order,
    L = phi_00 phi_22 + phi_00 phi_11 + phi_11 phi_22
        - phi_01^2 - phi_02^2 - phi_12^2."""
    kz = [_nyq_zeroed(k, conf) for k in kvec]
    pairs = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))
    spec = torch.stack([-(kvec[i] if i == j else kz[i]) * (kvec[j] if i == j else kz[j]) * pot
                        for i, j in pairs])
    phi = fftinv(spec, shape=conf.ptcl_grid_shape, axes=(-3, -2, -1)).to(torch.float32)
    L = phi[0] * phi[2]
    L = torch.addcmul(L, phi[0], phi[1])
    L = torch.addcmul(L, phi[1], phi[2])
    for c in (3, 4, 5):
        L = torch.addcmul(L, phi[c], phi[c], value=-1)
    return L


def _L(kvec, pot_m, pot_n, conf):
    """2nd-order source (lpt.py:40-76)."""
    m_eq_n = pot_n is None
    if m_eq_n and conf.dim == 3:
        return _L3(kvec, pot_m, conf)
    if m_eq_n:
        pot_n = pot_m
    L = torch.zeros(conf.ptcl_grid_shape, dtype=torch.float32, device=pot_m.device)
    for i in range(conf.dim):
        strain_m = _strain(kvec, i, i, pot_m, conf)
        for j in range(conf.dim - 1, i, -1):
            L = L + strain_m * _strain(kvec, j, j, pot_n, conf)
        if not m_eq_n:
            for j in range(i - 1, -1, -1):
                L = L + strain_m * _strain(kvec, j, j, pot_n, conf)
    if not m_eq_n:
        L = L * 0.5
    for i in range(conf.dim - 1):
        for j in range(i + 1, conf.dim):
            strain_m = _strain(kvec, i, j, pot_m, conf)
            strain_n = strain_m if m_eq_n else _strain(kvec, j, i, pot_n, conf)
            L = L - strain_m * strain_n
    return L


def levi_civita(indices):
    """Levi-Civita symbol (lpt.py:79-100)."""
    indices = list(indices)
    eps = 1
    for lo, hi in combinations(range(len(indices)), 2):
        d = indices[hi] - indices[lo]
        eps *= (d > 0) - (d < 0)
    return eps


def _M(kvec, pot, conf):
    """3rd-order determinant source (lpt.py:103-116)."""
    M = torch.zeros(conf.ptcl_grid_shape, dtype=torch.float32, device=pot.device)
    for i, j, k in permutations(range(conf.dim), r=3):
        M = M + (levi_civita((i, j, k)) * _strain(kvec, 0, i, pot, conf)
                 * _strain(kvec, 1, j, pot, conf) * _strain(kvec, 2, k, pot, conf))
    return M


def _growth_factors(cosmo, conf):
    """(lpt_order, 2) float32 host tensor of (D_m, a^2 H dD_m/dlna) at
    conf.a_start, the factors of lpt.py:197-210 (differentiable in the
    cosmology)."""
    a = conf.a_start
    rows = []
    for order in range(1, 1 + conf.lpt_order):
        D = growth(a, cosmo, conf, order=order)
        dD_dlna = growth(a, cosmo, conf, order=order, deriv=1)
        a2HDp = a ** 2 * torch.sqrt(E2(a, cosmo)) * dD_dlna
        rows.append(torch.stack([D.reshape(()), a2HDp.reshape(())]))
    return torch.stack(rows).to(torch.float32)


def _lpt_device(modes, fac, kvec, disp0, vel0, conf):
    """The device work of lpt (lpt.py:136-212) for lpt_order >= 1: the
    potentials, the 2nd-order source, and every displacement field of every
    order from one batched inverse FFT; fac (lpt_order, 2) float32 on the
    device.  Returns disp, vel as (dim, n) columns: disp_i += D_m g_mi,
    vel_i += a^2 H dD_m/dlna g_mi, order by order as the reference
    accumulates them."""
    modes = modes / conf.ptcl_cell_vol
    pot = [laplace(kvec, modes)]
    if conf.lpt_order > 1:
        src_2 = fftfwd(_L(kvec, pot[0], None, conf))
        pot.append(laplace(kvec, src_2))
    grads = torch.stack([neg_grad(k, pot[o], conf.ptcl_spacing)
                         for o in range(conf.lpt_order) for k in kvec])
    grads = fftinv(grads, shape=conf.ptcl_grid_shape,
                   axes=tuple(range(-conf.dim, 0))).to(torch.float32)
    grads = grads.reshape(conf.lpt_order, conf.dim, -1)
    disp, vel = disp0, vel0
    for o in range(conf.lpt_order):
        disp = disp + fac[o, 0] * grads[o]
        vel = vel + fac[o, 1] * grads[o]
    return disp, vel


# CUDA-graph replay of _lpt_device for calls without gradients on small
# grids, where launching ~10^3 small kernels one by one would cost more than
# the transforms themselves.  One graph per (configuration, device); the
# growth factors are a graph input, so a graph serves every cosmology.
# Builds and replays run on one library-created stream per device under a
# lock, so concurrent callers (the serving threads) never share the static
# buffers in flight and no replay lands in another graph's capture.
GRAPH_MAX_PTCL = 256 ** 3
_GRAPHS = OrderedDict()
_GRAPHS_MAX = 8
_GRAPH_LOCK = threading.Lock()


class _LptGraph:
    def __init__(self, conf, dev, spec_shape):
        self.conf, self.dev = conf, dev
        # warm-up, capture and every replay on the library's own stream (one
        # per device, shared by the graphs; built with the replay lock held,
        # so no replay is enqueued on it during a capture): a pooled torch
        # stream may be the stream another thread launches a request's work
        # on, which a capture would then record as well
        self.stream = _lib.lib_stream(dev)
        self.modes = torch.zeros(spec_shape, dtype=torch.complex64, device=dev)
        self.fac = torch.zeros((conf.lpt_order, 2), dtype=torch.float32, device=dev)
        # pinned staging for the factors: a ring, each slot reused only after
        # its last upload has completed
        self.ring = [torch.zeros((conf.lpt_order, 2), dtype=torch.float32).pin_memory()
                     for _ in range(4)]
        self.ring_ev = [None] * 4
        self.slot = 0
        grid = Particles.gen_grid(conf, vel=True, device=dev)
        self.pmid = grid.pmid
        self.disp0, self.vel0 = grid.disp.t(), grid.vel.t()
        self.kvec = fftfreq(conf.ptcl_grid_shape, conf.ptcl_spacing, dtype=torch.float32,
                            device=dev)
        cur = torch.cuda.current_stream(dev)
        self.stream.wait_stream(cur)
        with torch.no_grad():
            with torch.cuda.stream(self.stream):
                for _ in range(2):   # plans and allocator pools before capture
                    _lpt_device(self.modes, self.fac, self.kvec, self.disp0, self.vel0, conf)
            self.stream.synchronize()
            # captured on this stream with stream-level syncs only (no device
            # synchronize, which fails while another thread captures), in
            # thread-local mode so other threads keep launching meanwhile
            self.graph = torch.cuda.CUDAGraph()
            with torch.cuda.stream(self.stream):
                self.graph.capture_begin(capture_error_mode='thread_local')
                try:
                    self.disp, self.vel = _lpt_device(self.modes, self.fac, self.kvec,
                                                      self.disp0, self.vel0, conf)
                finally:
                    self.graph.capture_end()
            self.stream.synchronize()

    def run(self, modes, fac):
        cur = torch.cuda.current_stream(self.dev)
        with _GRAPH_LOCK, torch.no_grad():
            i = self.slot
            self.slot = (i + 1) % len(self.ring)
            if self.ring_ev[i] is not None:
                self.ring_ev[i].synchronize()
            self.ring[i].copy_(fac)
            self.stream.wait_stream(cur)   # modes are ready
            with torch.cuda.stream(self.stream):
                self.fac.copy_(self.ring[i], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(self.stream)
                self.ring_ev[i] = ev
                self.modes.copy_(modes)
                self.graph.replay()
                out = (self.pmid.clone(), self.disp.t().contiguous(), self.vel.t().contiguous())
        cur.wait_stream(self.stream)
        for t in out:   # allocated on the graph's stream, used on the caller's
            t.record_stream(cur)
        modes.record_stream(self.stream)
        return out


_BUILD_LOCK = threading.Lock()


def _graph_for(conf, modes):
    key = (conf, modes.device.index)
    with _GRAPH_LOCK:
        g = _GRAPHS.get(key)
        if g is not None:
            _GRAPHS.move_to_end(key)
            return g
    with _BUILD_LOCK:   # one capture at a time; a racing caller finds it built
        with _GRAPH_LOCK:   # and no replay on the shared stream meanwhile
            g = _GRAPHS.get(key)
            if g is None:
                g = _LptGraph(conf, modes.device, tuple(modes.shape))
                _GRAPHS[key] = g
                while len(_GRAPHS) > _GRAPHS_MAX:
                    _GRAPHS.popitem(last=False)
    return g


def _wants_graph(modes, cosmo, conf):
    if not modes.is_cuda or conf.lpt_order < 1 or conf.ptcl_num > GRAPH_MAX_PTCL:
        return False
    if modes.dtype != torch.complex64 or tuple(modes.shape) != tuple(
            conf.ptcl_grid_shape[:-1]) + (conf.ptcl_grid_shape[-1] // 2 + 1,):
        return False
    return not _hostmath.needs_grad(modes, cosmo)


def lpt(modes, cosmo, conf):
    """LPT displacements and velocities at conf.a_start (lpt.py:136-212).

    Returns ``(ptcl, None)`` with particles on the Lagrangian grid.  Calls
    that need no gradient, on grids up to 256^3, replay a CUDA graph of the
    device work.
    """
    if conf.dim not in (1, 2, 3):
        raise ValueError(f'dim={conf.dim} not supported')
    if conf.lpt_order not in (0, 1, 2, 3):
        raise ValueError(f'lpt_order={conf.lpt_order} not supported')
    if conf.lpt_order > 2:
        raise NotImplementedError('TODO')
    dev = modes.device
    if conf.lpt_order == 0:
        return Particles.gen_grid(conf, vel=True, device=dev), None
    if _wants_graph(modes, cosmo, conf):
        fac = torch.from_numpy(_hostmath.lpt_factors(cosmo, conf))
        pmid, disp, vel = _graph_for(conf, modes).run(modes, fac)
        return Particles(conf, pmid, disp, vel=vel), None
    fac = _growth_factors(cosmo, conf).to(dev)
    kvec = fftfreq(conf.ptcl_grid_shape, conf.ptcl_spacing, dtype=torch.float32, device=dev)
    ptcl = Particles.gen_grid(conf, vel=True, device=dev)
    disp, vel = _lpt_device(modes, fac, kvec, ptcl.disp.t(), ptcl.vel.t(), conf)
    return ptcl.replace(disp=disp.t().contiguous(), vel=vel.t().contiguous()), None
