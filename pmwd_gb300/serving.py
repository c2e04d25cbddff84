"""Continuous-batching server for many independent simulations on one GPU.

Requests differ in particle grid, mesh factor, step count, cosmology and
white-noise seed; some ask for the gradient of the squared-density
objective (forward run, then pmwd's reversible adjoint, nbody.py:251-276).
The server

* admits requests as they arrive while their device memory fits an HBM
  budget (particle state + cotangents + a mesh workspace; workspaces are
  pooled and reused per mesh shape);
* prepares each admitted request (float64 background tables, white noise,
  2LPT) on a host worker thread, so host work overlaps device work;
* runs every simulation as a job on its own CUDA stream and advances the
  jobs in turn a few leapfrog steps (forward or adjoint; one multi-step call
  of up to STEP_CHUNK steps) at a time, so kernels of different simulations
  overlap on the device and a newly admitted request starts while others
  are mid-run (continuous batching at step granularity);
* retires a job when the event after its last work completes, frees its
  slot and memory, and admits waiting requests;
* records per-request latency (arrival -> result ready): sims/s, p50, p99.

Each job runs exactly the kernels a stand-alone run would (own workspace,
own stream), so a result is the same alone and in the mix up to the order
of float32 atomic adds.
"""

import ctypes
import importlib
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .boltzmann import boltzmann
from .configuration import Configuration
from .cosmology import Cosmology
from .lpt import lpt
from .modes import linear_modes, white_noise
from .particles import Particles
from .scatter import scatter

_nb = importlib.import_module('pmwd_gb300.nbody')

# leapfrog steps a job issues per scheduling turn (one multi-step call, in
# which consecutive steps share particle passes)
STEP_CHUNK = 8


@dataclass
class Request:
    """One simulation request."""
    rid: int
    ptcl_side: int
    mesh_factor: int
    steps: int
    cosmo: dict            # sigma8 or A_s_1e9, n_s, Omega_m, Omega_b, h
    seed: int
    grad: bool = False
    arrival: float = 0.0   # seconds after the start of the stream
    ptcl_spacing: float = 2.0


@dataclass
class Result:
    rid: int
    latency: float
    disp_rms: float                  # rms displacement at a = 1
    obj: float                       # sum of squared density contrast at a = 1
    grad_rms: float = None           # rms of d obj / d (real white-noise modes)
    dobj_dOm: float = None           # d obj / d Omega_m
    state: dict = field(default=None, repr=False)


def request_bytes(side, grad):
    """Device bytes of a request besides its workspace: particle state
    (42 B per particle), cotangents and Kahan-free adjoint state (36 B), and
    the initial-condition transients (~64 B per particle at peak)."""
    n = side ** 3
    return 42 * n + (48 * n if grad else 0) + 64 * n


def workspace_bytes(mesh_side):
    """Meshes and spectra of a workspace plus a cuFFT work-area allowance."""
    m = mesh_side ** 3
    mc = mesh_side * mesh_side * (mesh_side // 2 + 1)
    return 4 * m + 3 * 8 * mc + 6 * 4 * m + 8 * mc


class WorkspacePool:
    """Reusable workspaces per (device, mesh shape); one job at a time uses
    a workspace (its buffers and cuFFT plans are bound to the job's
    stream)."""

    def __init__(self):
        self.free = {}
        self.lock = threading.Lock()

    def acquire(self, mesh, dev):
        key = (dev, tuple(mesh))
        with self.lock:
            lst = self.free.get(key)
            if lst:
                return lst.pop()
        return _lib.Workspace(mesh, adjoint=True, device=dev)

    def release(self, ws):
        key = (ws.device.index, ws.mesh_shape)
        with self.lock:
            self.free.setdefault(key, []).append(ws)

    def drop(self):
        with self.lock:
            self.free.clear()


class _Job:
    """One request as a step-wise state machine on its own CUDA stream:
    setup -> forward steps -> objective -> adjoint steps -> host backprop ->
    done."""

    def __init__(self, req, dev, pool):
        self.req = req
        self.dev = dev
        self.pool = pool
        self.stream = torch.cuda.Stream(device=dev)
        side = req.ptcl_side
        self.conf = Configuration(req.ptcl_spacing, (side,) * 3, req.mesh_factor,
                                  a_nbody_maxstep=(1 - 1 / 64) / req.steps)
        self.phase = 'setup'
        self.i = 0
        self.event = None
        self.setup_future = None

    # ---- host + device preparation (runs on a worker thread) ----
    def setup(self):
        torch.cuda.set_device(self.dev)
        r, conf = self.req, self.conf
        c = dict(r.cosmo)
        if 'sigma8' in c:
            s8 = c.pop('sigma8')
            base = Cosmology.from_sigma8(conf, s8, **c)
            c['A_s_1e9'] = float(base.A_s_1e9)
        cosmo = Cosmology(conf, **c)
        if r.grad:
            self.Om_leaf = cosmo.Omega_m.clone().requires_grad_(True)
            cosmo = cosmo.replace(Omega_m=self.Om_leaf)
        cosmo = boltzmann(cosmo, conf, varlin=False)
        self.cosmo = cosmo
        self.ws = self.pool.acquire(conf.mesh_shape, self.dev.index)
        with torch.cuda.stream(self.stream):
            modes = white_noise(r.seed, conf, real=True, device=self.dev)
            if r.grad:
                modes.requires_grad_(True)
                self.modes = modes
            with torch.set_grad_enabled(r.grad):
                ptcl, _ = lpt(linear_modes(modes, cosmo, conf), cosmo, conf)
            self.ptcl0 = ptcl
            self.pmid = ptcl.pmid.contiguous()
            self.disp = ptcl.disp.detach().contiguous().clone()
            self.vel = ptcl.vel.detach().contiguous().clone()
            self.acc = torch.empty_like(self.disp)
        fwd = _nb.op_factors(_nb.forward_ops(conf), cosmo, conf).detach()
        self.f_fwd = fwd.to(torch.float32).numpy().reshape(-1, 3)
        if r.grad:
            self.adj = _nb.op_factors(_nb.adjoint_ops(conf), cosmo, conf)
            self.f_adj = self.adj.detach().to(torch.float32).numpy().reshape(-1, 3)
        self.spec = _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)
        self.Om = float(torch.as_tensor(cosmo.Omega_m).detach())
        lib = _lib.load()
        P = _lib.ptr
        _lib.check(lib.pmx_force(self.ws.handle, self.spec, P(self.pmid), P(self.disp),
                                 self.pmid.shape[0], conf.ptcl_num, self.Om, P(self.acc),
                                 _lib.c_p(self.stream.cuda_stream)), 'pmx_force')

    def start(self, executor):
        self.setup_future = executor.submit(self.setup)

    # ---- one unit of device work per call ----
    def advance(self):
        """Issues the job's next unit of work; returns False when it has to
        wait (host setup or a device event still running)."""
        if self.phase == 'setup':
            if not self.setup_future.done():
                return False
            self.setup_future.result()      # re-raises setup errors
            self.phase = 'fwd'
            return True
        lib = _lib.load()
        P = _lib.ptr
        st = _lib.c_p(self.stream.cuda_stream)
        n = self.pmid.shape[0]
        conf = self.conf
        if self.phase == 'fwd':
            k = min(STEP_CHUNK, self.f_fwd.shape[0] - self.i)
            fac = np.ascontiguousarray(self.f_fwd[self.i:self.i + k])
            _lib.check(lib.pmx_nbody_steps(self.ws.handle, self.spec, P(self.pmid), P(self.disp),
                                           P(self.vel), P(self.acc), n, conf.ptcl_num, k,
                                           fac.ctypes.data_as(ctypes.c_void_p), self.Om, st),
                       'pmx_nbody_steps')
            self.i += k
            if self.i == self.f_fwd.shape[0]:
                self.phase = 'objective'
            return
        if self.phase == 'objective':
            with torch.cuda.stream(self.stream):
                disp = self.disp.clone().requires_grad_(self.req.grad)
                dens = scatter(Particles(conf, self.pmid, disp), conf)
                obj = (dens - 1).square().sum()
                self.obj_dev = obj.detach()
                self.rms_dev = self.disp.square().mean().sqrt()
                if self.req.grad:
                    (self.disp_cot,) = torch.autograd.grad(obj, disp)
                    self.vel_cot = torch.zeros_like(self.vel)
                    self.alpha = torch.zeros_like(self.disp)
                    nsteps = self.f_adj.shape[0]
                    self.dd = torch.zeros((nsteps + 1, 4), dtype=torch.float64, device=self.dev)
            if not self.req.grad:
                self._finish()
                return
            _lib.check(lib.pmx_force_vjp(self.ws.handle, self.spec, P(self.pmid), P(self.disp), n,
                                         conf.ptcl_num, self.Om, P(self.vel_cot), P(self.acc),
                                         P(self.alpha), P(self.dd[-1, 3:]), st), 'pmx_force_vjp')
            self.phase = 'adj'
            self.i = 0
            return
        if self.phase == 'adj':
            k = min(STEP_CHUNK, self.f_adj.shape[0] - self.i)
            fac = np.ascontiguousarray(self.f_adj[self.i:self.i + k])
            _lib.check(lib.pmx_nbody_adj_steps(self.ws.handle, self.spec, P(self.pmid),
                                               P(self.disp), P(self.vel), P(self.acc),
                                               P(self.disp_cot), P(self.vel_cot), P(self.alpha),
                                               n, conf.ptcl_num, k,
                                               fac.ctypes.data_as(ctypes.c_void_p), self.Om,
                                               P(self.dd[self.i]), st), 'pmx_nbody_adj_steps')
            self.i += k
            if self.i == self.f_adj.shape[0]:
                self.host_dd = torch.empty(self.dd.shape, dtype=torch.float64, pin_memory=True)
                with torch.cuda.stream(self.stream):
                    self.host_dd.copy_(self.dd, non_blocking=True)
                self.event = torch.cuda.Event()
                self.event.record(self.stream)
                self.phase = 'adj_wait'
            return
        if self.phase == 'adj_wait':
            if not self.event.query():
                return False
            self._backprop()
            self._finish()
            return True
        return False  # done_wait

    def _backprop(self):
        """Chain the adjoint's results to the white-noise modes and Omega_m:
        initial-state cotangents through 2LPT/linear_modes (autograd), factor
        sensitivities through the float64 factor functions, plus the direct
        Omega_m term of every force (nbody.py:80-99)."""
        dd = self.host_dd
        nsteps = self.f_adj.shape[0]
        dots = dd[:nsteps, :3].reshape(-1)
        om_force = torch.cat((dd[nsteps:, 3], dd[:nsteps, 3]))
        f64 = torch.tensor(self.f_adj, dtype=torch.float64)
        om_direct = -(om_force[:nsteps] * f64[:, 0]).sum() - (om_force[1:] * f64[:, 2]).sum()
        with torch.cuda.stream(self.stream):
            torch.autograd.backward([self.ptcl0.disp, self.ptcl0.vel, self.adj],
                                    [self.disp_cot, self.vel_cot, -dots])
        self.grad_rms = self.modes.grad.square().mean().sqrt()
        self.dobj_dOm = self.Om_leaf.grad + om_direct

    def _finish(self):
        self.event = torch.cuda.Event()
        self.event.record(self.stream)
        self.phase = 'done_wait'

    def ready(self):
        return self.phase == 'done_wait' and self.event.query()

    def result(self):
        g = self.req.grad
        return Result(self.req.rid, None, float(self.rms_dev), float(self.obj_dev),
                      float(self.grad_rms) if g else None, float(self.dobj_dOm) if g else None)


class Server:
    """Continuous batching with HBM admission (see the module docstring)."""

    def __init__(self, budget_bytes=150e9, max_jobs=64, device=None, host_workers=4):
        self.budget = budget_bytes
        self.max_jobs = max_jobs
        self.dev = torch.device('cuda', torch.cuda.current_device() if device is None else device)
        self.pool = WorkspacePool()
        self.host_workers = host_workers

    def cost(self, req):
        return (request_bytes(req.ptcl_side, req.grad)
                + workspace_bytes(req.ptcl_side * req.mesh_factor))

    def run(self, requests, realtime=True):
        """Serve ``requests`` (arrival offsets in seconds; realtime=False
        makes all available at t = 0).  Returns (results in request order,
        stats)."""
        pending = sorted(requests, key=lambda r: r.arrival)
        qi = 0
        waiting, active = [], []
        used = 0.0
        results = {}
        ex = ThreadPoolExecutor(max_workers=self.host_workers)
        t0 = time.perf_counter()
        try:
            while qi < len(pending) or waiting or active:
                now = time.perf_counter() - t0
                while qi < len(pending) and (not realtime or pending[qi].arrival <= now):
                    waiting.append(pending[qi])
                    qi += 1
                while waiting and len(active) < self.max_jobs:
                    c = self.cost(waiting[0])
                    if used + c > self.budget and active:
                        break
                    req = waiting.pop(0)
                    job = _Job(req, self.dev, self.pool)
                    job.cost = c
                    job.t_arr = req.arrival if realtime else 0.0
                    job.start(ex)
                    used += c
                    active.append(job)
                if not active:
                    if qi < len(pending):
                        time.sleep(max(0.0, min(0.002, pending[qi].arrival - now)))
                    continue
                moved = False
                for job in list(active):
                    if job.advance() is not False:
                        moved = True
                    if job.ready():
                        moved = True
                        res = job.result()
                        res.latency = (time.perf_counter() - t0) - job.t_arr
                        results[job.req.rid] = res
                        self.pool.release(job.ws)
                        used -= job.cost
                        active.remove(job)
                if not moved:
                    # every job waits on host setup or the device: yield the
                    # GIL to the setup threads instead of spinning
                    time.sleep(2e-4)
        finally:
            ex.shutdown(wait=True)
        torch.cuda.synchronize(self.dev)
        wall = time.perf_counter() - t0
        lat = np.array([r.latency for r in results.values()])
        stats = {'sims': len(results), 'wall_s': wall, 'sims_per_s': len(results) / wall,
                 'p50_s': float(np.percentile(lat, 50)) if len(lat) else None,
                 'p99_s': float(np.percentile(lat, 99)) if len(lat) else None}
        return [results[r.rid] for r in requests], stats


def run_sequential(requests, device=None):
    """The plain path: the same requests one at a time, each to completion
    (one job, no overlap) -- the baseline the served form is compared to."""
    return Server(budget_bytes=float('inf'), max_jobs=1, device=device,
                  host_workers=1).run(requests, realtime=False)


def make_stream(n, rate_hz, seed=0, sides=(64, 128, 256), factors=(1, 2), steps=(10, 100),
                grad_frac=0.2):
    """The serving workload: Poisson arrivals at ``rate_hz``, particle grid
    side from ``sides``, mesh factor from ``factors``, step count uniform in
    ``steps``, cosmology uniform in Omega_m [0.2, 0.4], sigma8 [0.7, 0.9],
    n_s [0.92, 1.0], h [0.6, 0.8] (Omega_b = 0.05), own white-noise seed, a
    fraction ``grad_frac`` asking for the gradient."""
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for i in range(n):
        t += rng.exponential(1.0 / rate_hz) if rate_hz > 0 else 0.0
        reqs.append(Request(
            rid=i, ptcl_side=int(rng.choice(sides)), mesh_factor=int(rng.choice(factors)),
            steps=int(rng.integers(steps[0], steps[1] + 1)),
            cosmo=dict(sigma8=float(rng.uniform(0.7, 0.9)), n_s=float(rng.uniform(0.92, 1.0)),
                       Omega_m=float(rng.uniform(0.2, 0.4)), Omega_b=0.05,
                       h=float(rng.uniform(0.6, 0.8))),
            seed=int(rng.integers(1 << 31)), grad=bool(rng.random() < grad_frac), arrival=t))
    return reqs
