"""Continuous-batching server for many independent simulations on one GPU.

Requests differ in particle grid, mesh factor, step count, cosmology and
white-noise seed; some ask for the gradient of the squared-density
objective (forward run, then pmwd's reversible adjoint, nbody.py:251-276).
pmwd itself runs one simulation per host loop (nbody.py:216-223); the
server

* admits requests as they arrive while their device memory fits an HBM
  budget (particle state and cotangents per request, plus the batched
  workspaces of the mesh groups in use); a request larger than the whole
  budget is rejected at once with an error result;
* prepares each admitted request (float64 background tables, white noise,
  2LPT) on a host worker thread, so host work overlaps device work;
* groups the admitted simulations that share a mesh shape and cell size
  and are in the same phase (forward or adjoint steps): each group
  advances a chunk of leapfrog steps in ONE batched call
  (pmx_nbody_steps_batch / pmx_nbody_adj_steps_batch), whose particle
  kernels serve every simulation of the group in one launch and whose plane
  transforms run over all their meshes at once; meshes the fused x pass
  does not cover run one simulation per call;
* lets newly admitted requests join their group at the next chunk while the
  others are mid-run (continuous batching at step granularity);
* isolates failures: a request whose host setup or device call raises, or
  that is cancelled, ends with an error result, its slot and memory are
  freed once nothing of it is in flight, and every other request goes on;
* records per-request latency (arrival -> result ready): sims/s, p50, p99.

The scheduling logic (``Scheduler``) is host code over an engine interface;
``GpuEngine`` issues the device work.  A simulation's arithmetic is the one
of the single-simulation path, so a result is the same alone and in the mix
up to the order of float32 atomic adds.
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

# leapfrog steps a group issues per scheduling turn (one batched call, in
# which consecutive steps share particle passes)
STEP_CHUNK = 8
# most simulations per batched call
MAX_SLOTS = 8


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
    disp_rms: float = None           # rms displacement at a = 1
    obj: float = None                # sum of squared density contrast at a = 1
    grad_rms: float = None           # rms of d obj / d (real white-noise modes)
    dobj_dOm: float = None           # d obj / d Omega_m
    error: str = None                # why the request failed (None: it did not)
    state: dict = field(default=None, repr=False)


def request_bytes(side, grad):
    """Device bytes of a request besides the workspaces: particle state
    (42 B per particle), cotangents and Kahan-free adjoint state (36 B), and
    the initial-condition transients (~64 B per particle at peak)."""
    n = side ** 3
    return 42 * n + (48 * n if grad else 0) + 64 * n


def workspace_bytes(mesh_side, slots=1):
    """Meshes and spectra of a workspace with `slots` simulation slots, a
    cuFFT work-area allowance, and the per-block float64 partial sums of the
    particle kernels (4 x 2^19 in a single-simulation workspace, 4 x 2^16 per
    slot of a batched one)."""
    m = mesh_side ** 3
    mc = mesh_side * mesh_side * (mesh_side // 2 + 1)
    part = 4 * 8 * (2 ** 19 if slots == 1 else slots * 2 ** 16)
    return slots * (4 * m + 3 * 8 * mc + 6 * 4 * m + 8 * mc) + part


def batchable(mesh_side):
    """Meshes of the fused x-pass path, which batched calls need."""
    return mesh_side in (64, 128, 256, 512, 1024)


def group_slots(mesh_side, budget):
    """Simulations per batched workspace: up to MAX_SLOTS, with the
    workspace at most a quarter of the budget; 1 where batching does not
    apply."""
    if not batchable(mesh_side):
        return 1
    per_slot = workspace_bytes(mesh_side, MAX_SLOTS) / MAX_SLOTS
    return int(max(1, min(MAX_SLOTS, (0.25 * budget) // per_slot)))


class Job:
    """Host-side state of one admitted request.  Phases: setup -> fwd ->
    objective -> (adj_init -> adj -> backprop) -> done; or failed."""

    def __init__(self, req, t_arr, cost):
        self.req = req
        self.t_arr = t_arr
        self.cost = cost
        self.key = (req.ptcl_side * req.mesh_factor,
                    req.ptcl_spacing / req.mesh_factor)   # mesh side, cell size
        self.phase = 'setup'
        self.i = 0                  # steps done in the current phase
        self.init = True            # forward: the first call also computes acc
        self.cancel = False
        self.error = None
        self.future = None
        self.dev = None             # engine state


class Scheduler:
    """Admission, grouping, chunked stepping, failure isolation and
    cancellation over an engine (``GpuEngine`` or a test double):

    * engine.slots(key) -> simulations per call for a group key;
    * engine.group_bytes(key) -> device bytes of that group's shared
      workspace; engine.job_bytes(req) -> device bytes of one request;
    * engine.setup(job) (worker thread; may raise);
    * engine.fwd(jobs, init, k) / engine.adj_init(jobs) / engine.adj(jobs, k):
      one call for jobs of one key, in the same phase (may raise);
    * engine.objective(job) / engine.backprop(job) (may raise);
    * engine.idle(job) -> nothing of the job is in flight on the device;
    * engine.result(job) -> Result; engine.release(job);
    * engine.resident() -> keys whose group workspace exists; engine.drop(key)
      frees one.
    """

    def __init__(self, engine, budget_bytes=150e9, max_jobs=64, host_workers=4):
        self.engine = engine
        self.budget = budget_bytes
        self.max_jobs = max_jobs
        self.host_workers = host_workers
        self._cancel = set()
        self._lock = threading.Lock()

    def cost(self, req):
        return self.engine.job_bytes(req)

    def cancel(self, rid):
        """Cancels request ``rid`` (thread-safe): a waiting request is dropped,
        an active one stops at its next step boundary; its result carries
        error 'cancelled'."""
        with self._lock:
            self._cancel.add(rid)

    def run(self, requests, realtime=True, on_turn=None):
        """Serve ``requests`` (arrival offsets in seconds; realtime=False
        makes all available at t = 0).  Returns (results in request order,
        stats).  ``on_turn(scheduler, t)`` is called once per scheduling turn
        (tests use it to cancel)."""
        eng = self.engine
        pending = sorted(requests, key=lambda r: r.arrival)
        qi = 0
        waiting, active = [], []
        # key -> bytes charged for its workspace (groups of earlier runs
        # keep theirs until the budget needs the room)
        groups = {k: eng.group_bytes(k) for k in eng.resident()}
        used = float(sum(groups.values()))
        results = {}
        ex = ThreadPoolExecutor(max_workers=self.host_workers)
        t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        def finish(job, res):
            res.latency = now() - job.t_arr
            results[job.req.rid] = res

        def fail(job, err):
            job.error = err
            job.phase = 'failed'

        try:
            while qi < len(pending) or waiting or active:
                t = now()
                if on_turn is not None:
                    on_turn(self, t)
                while qi < len(pending) and (not realtime or pending[qi].arrival <= t):
                    waiting.append(pending[qi])
                    qi += 1
                with self._lock:
                    cancels = set(self._cancel)
                for r in [r for r in waiting if r.rid in cancels]:
                    waiting.remove(r)
                    results[r.rid] = Result(r.rid, 0.0, error='cancelled')
                for job in active:
                    if job.req.rid in cancels and job.phase not in ('done', 'failed'):
                        job.cancel = True
                # admission by HBM budget (request state + new group workspaces)
                while waiting and len(active) < self.max_jobs:
                    req = waiting[0]
                    key = (req.ptcl_side * req.mesh_factor, req.ptcl_spacing / req.mesh_factor)
                    c = self.cost(req)
                    g = 0.0 if key in groups else eng.group_bytes(key)
                    if c + eng.group_bytes(key) > self.budget:
                        waiting.pop(0)
                        results[req.rid] = Result(req.rid, 0.0, error=(
                            f'over budget: needs {(c + eng.group_bytes(key)) / 1e9:.2f} GB of '
                            f'{self.budget / 1e9:.2f} GB'))
                        continue
                    if used + c + g > self.budget:
                        # free the workspaces of groups nobody uses any more
                        live = {j.key for j in active}
                        for k in [k for k in groups if k not in live]:
                            used -= groups.pop(k)
                            eng.drop(k)
                        g = 0.0 if key in groups else eng.group_bytes(key)
                        if used + c + g > self.budget:
                            break
                    waiting.pop(0)
                    if key not in groups:
                        groups[key] = eng.group_bytes(key)
                        used += groups[key]
                    job = Job(req, req.arrival if realtime else 0.0, c)
                    job.future = ex.submit(eng.setup, job)
                    used += c
                    active.append(job)
                if not active:
                    if qi < len(pending):
                        time.sleep(max(0.0, min(0.002, pending[qi].arrival - now())))
                    continue
                moved = False
                # per-job phases
                for job in active:
                    try:
                        if job.cancel and job.phase not in ('failed', 'done'):
                            fail(job, 'cancelled')
                        if job.phase == 'setup' and job.future.done():
                            job.future.result()          # re-raises the setup error
                            job.phase = 'fwd'
                            moved = True
                        elif job.phase == 'objective':
                            eng.objective(job)
                            job.phase = 'adj_init' if job.req.grad else 'done'
                            moved = True
                        elif job.phase == 'backprop' and eng.idle(job):
                            eng.backprop(job)
                            job.phase = 'done'
                            moved = True
                    except Exception as e:               # isolate this request
                        fail(job, f'{type(e).__name__}: {e}')
                        moved = True
                # grouped device phases: one call per (key, phase) group
                moved |= self._step_groups(active, fail)
                # retire finished and failed jobs once nothing of them is in flight
                for job in list(active):
                    if job.phase not in ('done', 'failed') or not job.future.done():
                        continue                         # running, or its setup still is
                    if eng.idle(job):
                        if job.phase == 'done':
                            try:
                                res = eng.result(job)
                            except Exception as e:
                                res = Result(job.req.rid, 0.0, error=f'{type(e).__name__}: {e}')
                        else:
                            res = Result(job.req.rid, 0.0, error=job.error)
                        finish(job, res)
                        eng.release(job)
                        used -= job.cost
                        active.remove(job)
                        moved = True
                if not moved:
                    # every job waits on host setup or the device: yield the
                    # GIL to the setup threads instead of spinning
                    time.sleep(2e-4)
        finally:
            ex.shutdown(wait=True)
        eng.synchronize()
        wall = now()
        ok = [r for r in results.values() if r.error is None]
        lat = np.array([r.latency for r in ok])
        stats = {'sims': len(ok), 'failed': len(results) - len(ok), 'wall_s': wall,
                 'sims_per_s': len(ok) / wall,
                 'p50_s': float(np.percentile(lat, 50)) if len(lat) else None,
                 'p99_s': float(np.percentile(lat, 99)) if len(lat) else None}
        return [results[r.rid] for r in requests], stats

    def _step_groups(self, active, fail):
        eng = self.engine
        moved = False
        buckets = {}
        for job in active:
            if job.cancel or job.phase not in ('fwd', 'adj_init', 'adj'):
                continue
            ph = 'fwd_init' if (job.phase == 'fwd' and job.init) else job.phase
            buckets.setdefault((job.key, ph), []).append(job)
        for (key, ph), jobs in buckets.items():
            n = eng.slots(key)
            for i in range(0, len(jobs), n):
                part = jobs[i:i + n]
                moved = True
                try:
                    self._issue(ph, part)
                except Exception as e:
                    if len(part) == 1 or not getattr(e, 'before_launch', False):
                        for job in part:
                            fail(job, f'{type(e).__name__}: {e}')
                        continue
                    # a rejected batch launched nothing: find the culprit alone
                    for job in part:
                        try:
                            self._issue(ph, [job])
                        except Exception as e1:
                            fail(job, f'{type(e1).__name__}: {e1}')
        return moved

    def _issue(self, ph, jobs):
        eng = self.engine
        if ph == 'adj_init':
            eng.adj_init(jobs)
            for job in jobs:
                job.phase, job.i = 'adj', 0
            return
        left = min(job.req.steps - job.i for job in jobs)
        k = min(STEP_CHUNK, left)
        if ph in ('fwd', 'fwd_init'):
            eng.fwd(jobs, ph == 'fwd_init', k)
            for job in jobs:
                job.init = False
                job.i += k
                if job.i == job.req.steps:
                    job.phase = 'objective'
        else:
            eng.adj(jobs, k)
            for job in jobs:
                job.i += k
                if job.i == job.req.steps:
                    job.phase = 'backprop'


class BatchRejected(_lib.PmxError):
    """A batched call refused on the host before anything was launched."""
    before_launch = True


class GpuEngine:
    """Device work of the scheduler.  Per request: setup, objective and
    backprop on the request's own CUDA stream.  Groups whose mesh the fused
    x pass covers share one batched workspace (``slots`` simulations) and
    one stream, and advance through the batched entry points; other meshes,
    and every mesh with ``batch=False`` (the plain path), run one
    simulation per call through the single-simulation entry points, on the
    request's stream with a workspace of its own."""

    def __init__(self, device=None, budget_bytes=150e9, batch=True):
        self.dev = torch.device('cuda', torch.cuda.current_device() if device is None else device)
        self.budget = budget_bytes
        self.batch = batch
        self.group_ws = {}           # key -> batched workspace
        self.streams = {}            # key -> group stream
        self.free = {}               # key -> free single workspaces
        self.lock = threading.Lock()

    # ---- groups ----
    def slots(self, key):
        return group_slots(key[0], self.budget) if self.batch else 1

    def group_bytes(self, key):
        s = self.slots(key)
        return workspace_bytes(key[0], s) if s > 1 else 0

    def job_bytes(self, req):
        key = (req.ptcl_side * req.mesh_factor, req.ptcl_spacing / req.mesh_factor)
        own = workspace_bytes(key[0]) if self.slots(key) == 1 else 0
        return request_bytes(req.ptcl_side, req.grad) + own

    def _group(self, key):
        with self.lock:
            ws = self.group_ws.get(key)
            st = self.streams.get(key)
        if ws is None:
            ws = _lib.Workspace((key[0],) * 3, adjoint=True, device=self.dev.index,
                                slots=self.slots(key))
            st = torch.cuda.Stream(device=self.dev)
            with self.lock:
                self.group_ws[key] = ws
                self.streams[key] = st
        return ws, st

    def _single_ws(self, job):
        d = job.dev
        if 'ws' not in d:
            with self.lock:
                lst = self.free.get(job.key)
                ws = lst.pop() if lst else None
            if ws is None:
                ws = _lib.Workspace((job.key[0],) * 3, adjoint=True, device=self.dev.index)
            d['ws'] = ws
        return d['ws']

    def resident(self):
        with self.lock:
            return list(self.group_ws)

    def drop(self, key):
        torch.cuda.synchronize(self.dev)
        with self.lock:
            self.group_ws.pop(key, None)
            self.streams.pop(key, None)
            self.free.pop(key, None)

    def close(self):
        """Frees every workspace the engine holds."""
        torch.cuda.synchronize(self.dev)
        with self.lock:
            self.group_ws.clear()
            self.streams.clear()
            self.free.clear()

    def synchronize(self):
        torch.cuda.synchronize(self.dev)

    # ---- per request ----
    def setup(self, job):
        """Host tables, white noise, 2LPT (on the request's own stream)."""
        torch.cuda.set_device(self.dev)
        r = job.req
        conf = Configuration(r.ptcl_spacing, (r.ptcl_side,) * 3, r.mesh_factor,
                             a_nbody_maxstep=(1 - 1 / 64) / r.steps)
        d = job.dev = {'conf': conf, 'stream': torch.cuda.Stream(device=self.dev), 'event': None}
        c = dict(r.cosmo)
        if 'sigma8' in c:
            s8 = c.pop('sigma8')
            base = Cosmology.from_sigma8(conf, s8, **c)
            c['A_s_1e9'] = float(base.A_s_1e9)
        cosmo = Cosmology(conf, **c)
        if r.grad:
            d['Om_leaf'] = cosmo.Omega_m.clone().requires_grad_(True)
            cosmo = cosmo.replace(Omega_m=d['Om_leaf'])
        cosmo = boltzmann(cosmo, conf, varlin=False)
        with torch.cuda.stream(d['stream']):
            modes = white_noise(r.seed, conf, real=True, device=self.dev)
            if r.grad:
                modes.requires_grad_(True)
                d['modes'] = modes
            with torch.set_grad_enabled(r.grad):
                ptcl, _ = lpt(linear_modes(modes, cosmo, conf), cosmo, conf)
            d['ptcl0'] = ptcl
            d['pmid'] = ptcl.pmid.contiguous()
            d['disp'] = ptcl.disp.detach().contiguous().clone()
            d['vel'] = ptcl.vel.detach().contiguous().clone()
            d['acc'] = torch.empty_like(d['disp'])
        fwd = _nb.op_factors(_nb.forward_ops(conf), cosmo, conf).detach()
        d['f_fwd'] = np.ascontiguousarray(fwd.to(torch.float32).numpy().reshape(-1, 3))
        if r.grad:
            d['adj'] = _nb.op_factors(_nb.adjoint_ops(conf), cosmo, conf)
            d['f_adj'] = np.ascontiguousarray(
                d['adj'].detach().to(torch.float32).numpy().reshape(-1, 3))
        d['spec'] = _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)
        d['Om'] = float(torch.as_tensor(cosmo.Omega_m).detach())
        d['event'] = self._record(d['stream'])

    def _record(self, stream):
        ev = torch.cuda.Event()
        ev.record(stream)
        return ev

    def idle(self, job):
        d = job.dev
        return d is None or d.get('event') is None or d['event'].query()

    def _sim(self, job, factors, dots):
        d = job.dev
        return _lib.PmxSim(d['pmid'].data_ptr(), d['disp'].data_ptr(), d['vel'].data_ptr(),
                           d['acc'].data_ptr(),
                           d['disp_cot'].data_ptr() if 'disp_cot' in d else None,
                           d['vel_cot'].data_ptr() if 'vel_cot' in d else None,
                           d['alpha'].data_ptr() if 'alpha' in d else None,
                           d['pmid'].shape[0], d['conf'].ptcl_num, d['Om'],
                           None if factors is None else factors.ctypes.data,
                           None if dots is None else dots.data_ptr())

    def _call(self, jobs, name, tables, init, k):
        """One batched call of the group's jobs on the group stream, after
        each job's last work; records the jobs' new event."""
        ws, st = self._group(jobs[0].key)
        for job in jobs:
            if job.dev['event'] is not None:
                st.wait_event(job.dev['event'])
        arr = (_lib.PmxSim * len(jobs))(*tables)
        lib = _lib.load()
        status = getattr(lib, name)(ws.handle, jobs[0].dev['spec'], len(jobs), arr, int(init),
                                    int(k), _lib.c_p(st.cuda_stream))
        if status != 0:
            msg = lib.pmx_last_error().decode(errors='replace')
            cls = BatchRejected if status in (-1, -2, -3) else _lib.PmxError
            raise cls(f'{name} failed with status {status}: {msg}')
        ev = self._record(st)
        for job in jobs:
            job.dev['event'] = ev

    def _single(self, job, fn):
        """fn(lib, ws, stream pointer) on the request's own stream and workspace."""
        d = job.dev
        ws = self._single_ws(job)
        st = d['stream']
        if d['event'] is not None:
            st.wait_event(d['event'])
        fn(_lib.load(), ws, _lib.c_p(st.cuda_stream))
        d['event'] = self._record(st)

    def _batched(self, jobs):
        return self.slots(jobs[0].key) > 1

    def fwd(self, jobs, init, k):
        keep = [np.ascontiguousarray(j.dev['f_fwd'][j.i:j.i + k]) for j in jobs]
        if self._batched(jobs):
            self._call(jobs, 'pmx_nbody_steps_batch',
                       [self._sim(j, f, None) for j, f in zip(jobs, keep)], init, k)
            return
        P = _lib.ptr
        for j, f in zip(jobs, keep):
            d = j.dev
            n, N = d['pmid'].shape[0], d['conf'].ptcl_num

            def run(lib, ws, st, d=d, f=f, n=n, N=N):
                if init:
                    _lib.check(lib.pmx_force(ws.handle, d['spec'], P(d['pmid']), P(d['disp']), n,
                                             N, d['Om'], P(d['acc']), st), 'pmx_force')
                _lib.check(lib.pmx_nbody_steps(ws.handle, d['spec'], P(d['pmid']), P(d['disp']),
                                               P(d['vel']), P(d['acc']), n, N, k,
                                               f.ctypes.data_as(ctypes.c_void_p), d['Om'], st),
                           'pmx_nbody_steps')
            self._single(j, run)

    def adj_init(self, jobs):
        if self._batched(jobs):
            self._call(jobs, 'pmx_nbody_adj_steps_batch',
                       [self._sim(j, None, j.dev['dd'][-1]) for j in jobs], 1, 0)
            return
        P = _lib.ptr
        for j in jobs:
            d = j.dev

            def run(lib, ws, st, d=d):
                _lib.check(lib.pmx_force_vjp(ws.handle, d['spec'], P(d['pmid']), P(d['disp']),
                                             d['pmid'].shape[0], d['conf'].ptcl_num, d['Om'],
                                             P(d['vel_cot']), P(d['acc']), P(d['alpha']),
                                             P(d['dd'][-1, 3:]), st), 'pmx_force_vjp')
            self._single(j, run)

    def adj(self, jobs, k):
        keep = [np.ascontiguousarray(j.dev['f_adj'][j.i:j.i + k]) for j in jobs]
        if self._batched(jobs):
            self._call(jobs, 'pmx_nbody_adj_steps_batch',
                       [self._sim(j, f, j.dev['dd'][j.i]) for j, f in zip(jobs, keep)], 0, k)
            return
        P = _lib.ptr
        for j, f in zip(jobs, keep):
            d = j.dev
            i0 = j.i

            def run(lib, ws, st, d=d, f=f, i0=i0):
                _lib.check(lib.pmx_nbody_adj_steps(
                    ws.handle, d['spec'], P(d['pmid']), P(d['disp']), P(d['vel']), P(d['acc']),
                    P(d['disp_cot']), P(d['vel_cot']), P(d['alpha']), d['pmid'].shape[0],
                    d['conf'].ptcl_num, k, f.ctypes.data_as(ctypes.c_void_p), d['Om'],
                    P(d['dd'][i0]), st), 'pmx_nbody_adj_steps')
            self._single(j, run)

    def objective(self, job):
        """Objective sum((rho - 1)^2) at a = 1 and, for gradients, its
        cotangent of disp (the adjoint's initial disp_cot)."""
        d, r = job.dev, job.req
        conf = d['conf']
        st = d['stream']
        st.wait_event(d['event'])
        with torch.cuda.stream(st):
            disp = d['disp'].clone().requires_grad_(r.grad)
            dens = scatter(Particles(conf, d['pmid'], disp), conf)
            obj = (dens - 1).square().sum()
            d['obj'] = obj.detach()
            d['rms'] = d['disp'].square().mean().sqrt()
            if r.grad:
                (d['disp_cot'],) = torch.autograd.grad(obj, disp)
                d['vel_cot'] = torch.zeros_like(d['vel'])
                d['alpha'] = torch.zeros_like(d['disp'])
                d['dd'] = torch.zeros((r.steps + 1, 4), dtype=torch.float64, device=self.dev)
        d['event'] = self._record(st)

    def backprop(self, job):
        """Chain the adjoint's results to the white-noise modes and Omega_m:
        initial-state cotangents through 2LPT/linear_modes (autograd), factor
        sensitivities through the float64 factor functions, plus the direct
        Omega_m term of every force (nbody.py:80-99)."""
        d = job.dev
        dd = d['dd'].cpu()
        nsteps = d['f_adj'].shape[0]
        dots = dd[:nsteps, :3].reshape(-1)
        om_force = torch.cat((dd[nsteps:, 3], dd[:nsteps, 3]))
        f64 = torch.tensor(d['f_adj'], dtype=torch.float64)
        om_direct = -(om_force[:nsteps] * f64[:, 0]).sum() - (om_force[1:] * f64[:, 2]).sum()
        st = d['stream']
        st.wait_event(d['event'])
        with torch.cuda.stream(st):
            torch.autograd.backward([d['ptcl0'].disp, d['ptcl0'].vel, d['adj']],
                                    [d['disp_cot'], d['vel_cot'], -dots])
        d['grad_rms'] = d['modes'].grad.square().mean().sqrt()
        d['dobj_dOm'] = d['Om_leaf'].grad + om_direct
        d['event'] = self._record(st)

    def result(self, job):
        d, g = job.dev, job.req.grad
        return Result(job.req.rid, None, float(d['rms']), float(d['obj']),
                      float(d['grad_rms']) if g else None, float(d['dobj_dOm']) if g else None)

    def release(self, job):
        d = job.dev
        if d is not None and 'ws' in d:
            with self.lock:
                self.free.setdefault(job.key, []).append(d['ws'])
        job.dev = None


class Server:
    """Continuous batching with HBM admission (see the module docstring)."""

    def __init__(self, budget_bytes=150e9, max_jobs=64, device=None, host_workers=4, batch=True):
        self.engine = GpuEngine(device, budget_bytes, batch)
        self.sched = Scheduler(self.engine, budget_bytes, max_jobs, host_workers)

    def cost(self, req):
        return self.sched.cost(req)

    def cancel(self, rid):
        self.sched.cancel(rid)

    def run(self, requests, realtime=True, on_turn=None):
        return self.sched.run(requests, realtime, on_turn)

    def close(self):
        self.engine.close()


def sequential_server(device=None):
    """The plain path: requests one at a time, each to completion (one
    simulation per call, no overlap) -- the baseline the served form is
    compared to."""
    return Server(budget_bytes=float('inf'), max_jobs=1, device=device, host_workers=1,
                  batch=False)


def run_sequential(requests, device=None):
    srv = sequential_server(device)
    try:
        return srv.run(requests, realtime=False)
    finally:
        srv.close()


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
