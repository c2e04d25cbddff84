#!/usr/bin/env python
"""Throughput of pmwd's particle-mesh hot path on GB300.

The timed region is a segment of the 512^3-particle / 1024^3-mesh run (box
1024 Mpc/h, 2LPT initial conditions at a = 1/64, 100 steps to a = 1): its
first K forward leapfrog steps (K/2 D F K/2, nbody.py:121-140) through one
multi-step call, then the K reversible-adjoint steps of those (kick_adj,
drift_adj, force_adj, kick_adj, nbody.py:143-162) through another.  One
bench step is one forward + adjoint step pair; the metric is particle-steps
per second of forward + adjoint (N particles per step pair).  The e2e figure
runs single step pairs through the C ABI with every input copied in from
pinned host memory and every output copied back.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl pmx|reference]

N > 1 (torchrun): independent replicas, one per GPU (the path does not
shard); value = total particle-steps of all ranks / max-over-ranks time.
``--impl reference`` times the CPU restatement of the reference algorithm
(the NumPy/SciPy oracle) on the host cores, on a bounded sample.
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = 'ptcl-steps/s fwd+adjoint at 512^3'
UNIT = 'ptcl-steps/s'

# Cosmology of the reference's configurations (A_s = 2.1e-9, n_s = 0.965,
# Omega_m = 0.3, Omega_b = 0.05, h = 0.7).
COSMO = dict(A_s_1e9=2.1, n_s=0.965, Omega_m=0.3, Omega_b=0.05, h=0.7)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='pmx', choices=['pmx', 'reference'])
    ap.add_argument('--ptcl', type=int, default=512, help='particle grid side')
    ap.add_argument('--mesh', type=float, default=2, help='mesh / particle grid ratio')
    ap.add_argument('--spacing', type=float, default=2.0, help='particle spacing [Mpc/h]')
    ap.add_argument('--nbody-steps', type=int, default=100)
    ap.add_argument('--cpu-sample', type=int, default=48,
                    help='particle grid side of the bounded CPU sample')
    ap.add_argument('--deposit', default='atomic', choices=['atomic', 'agg', 'window'],
                    help='CIC deposits: one float32 reduction per contribution, warp-aggregated '
                         'for particles sharing a cell, or per-warp shared-memory windows')
    ap.add_argument('--tma', action='store_true',
                    help='TMA-staged forward gathers (PMX_WS_TMA)')
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--no-full-run', action='store_true',
                    help='skip the whole-run measurement (all forward steps, then all adjoint '
                         'steps)')
    ap.add_argument('--dry-run', action='store_true',
                    help='no GPU work: each rank reports a fixed synthetic time, to check the '
                         'replica launch and the reduction over ranks on CPU (gloo)')
    ap.add_argument('--serve', type=int, default=0,
                    help='serving mode: number of requests of the serving stream')
    ap.add_argument('--serve-requests', type=int, default=32,
                    help='requests of the serving measurement in the default line (0: none)')
    ap.add_argument('--serve-sides', default='64,128,256')
    ap.add_argument('--contention', action='store_true',
                    help='scatter/gather contention stress: 256^3 particles, 256^3 mesh, 64 Mpc/h '
                         'box evolved to a=1 vs the same particles on the lattice')
    ap.add_argument('--serve-steps', default='10,100')
    ap.add_argument('--gradient', action='store_true',
                    help="the reference quickstart's gradient: 256^3 / 512^3 mesh, 63 steps, "
                         "d var(dens - target) / d(modes, cosmology)")
    ap.add_argument('--powspec', type=int, default=0,
                    help='power-spectrum binning of an N^3 field (rfftn + pmx_powspec_bin)')
    ap.add_argument('--published', action='store_true',
                    help="pmwd's own timing table (perf.py): growth, 2LPT and N-body per step "
                         "for ptcl grids 32^3..512^3 at mesh x1 and x2")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------

def algorithmic_bytes(N, M, Mc):
    """Compulsory HBM bytes of every stage, each operand counted once
    (float32 particle arrays 12 B per particle and array, int16 pmid 6 B,
    float32 mesh 4 B per cell, complex64 8 B per complex cell)."""
    return {
        'fill': None,                       # per launch size differs (M or 3M)
        'deposit_fwd': 6 * N + 36 * N + 24 * N + 4 * M,
        'r2c': 4 * M + 8 * Mc,
        'poisson_fwd': 8 * Mc + 24 * Mc,
        'c2r_x3': 3 * (8 * Mc + 4 * M),
        'gather3_kick': 6 * N + 12 * N + 12 * M + 12 * N + 24 * N,
        'kick_drift_adj_deposit': 6 * N + 72 * N + 48 * N + 4 * M,
        'gather3_adj': 6 * N + 24 * N + 24 * N + 12 * M + 12 * M,
        'r2c_x3': 3 * (4 * M + 8 * Mc),
        'poisson_adj': 24 * Mc + 8 * Mc,
        'c2r': 8 * Mc + 4 * M,
        'scatter_adj_kick': 6 * N + 12 * N + 4 * M + 24 * N + 24 * N + 12 * N + 24 * N,
        'finish': None,
        # consecutive steps joined: gather + kick, kick + drift + deposit
        'gather3_kick_kick_drift_deposit': 6 * N + 48 * N + 12 * M + 4 * M,
        # scatter VJP + kick_adj, kick_adj + drift_adj + deposit
        'scatter_adj_kick_kick_drift_adj_deposit': 6 * N + 120 * N + 4 * M + 4 * M,
    }


OWN_KERNELS = ('deposit_fwd', 'poisson_fwd', 'gather3_kick', 'kick_drift_adj_deposit',
               'gather3_adj', 'poisson_adj', 'scatter_adj_kick', 'gather3_kick_kick_drift_deposit',
               'scatter_adj_kick_kick_drift_adj_deposit')


class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed
    region."""

    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', f'--query-gpu={self.FIELDS}', '--format=csv,noheader,nounits',
                 '-lms', '200'], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
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
        rows = []
        for ln in self.lines:
            p = [x.strip() for x in ln.split(',')]
            if len(p) < 9:
                continue
            rows.append(p)
        idx = {r[0] for r in rows}
        if len(idx) > 1:
            rows = [r for r in rows if r[0] == str(self.gpu)]
        if not rows:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['no samples']}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        pw = [num(r[3]) for r in rows if num(r[3]) is not None]
        thr = (max(pw) * 0.5) if pw else 0
        loaded = [num(r[1]) for r in rows if num(r[3]) is not None and num(r[3]) >= thr]
        names = ('hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap')
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == 'active'})
        return {'sm_mhz': statistics.median(loaded or sm), 'sm_max_mhz': num(rows[0][2]),
                'reasons': reasons, 'samples': len(rows), 'power_w_max': max(pw) if pw else None}


def measured_peak():
    p = os.path.join(ROOT, 'MEASURED_PEAKS.json')
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    except Exception:
        return 6800.0, 'fallback'


def ncu_traffic():
    """Per-launch DRAM bytes of each stage from the committed ncu summary
    (profiles/dram_traffic.txt: '<stage> <bytes per launch>' lines)."""
    p = os.path.join(ROOT, 'profiles', 'dram_traffic.txt')
    out = {}
    try:
        with open(p) as f:
            for ln in f:
                ln = ln.strip()
                if not ln or ln.startswith('#'):
                    continue
                k, v = ln.split()[:2]
                out[k] = float(v)
    except OSError:
        pass
    return out


def replica_throughput(ms_local, units_local, world, device):
    """Whole-job throughput of independent replicas: the slowest rank's time
    (max over ranks) and the units (particle-steps) all ranks processed.
    No data-path collective: this reduction happens once, after timing."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms_local, float(units_local)], dtype=torch.float64, device=device)
    if world > 1:
        mx = t[:1].clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        tot = t[1:].clone()
        dist.all_reduce(tot, op=dist.ReduceOp.SUM)
        t = torch.cat((mx, tot))
    ms = float(t[0])
    return ms, float(t[1]) / (ms / 1e3)


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (CPU restatement of the reference algorithm)
# ---------------------------------------------------------------------------

def cpu_step_pair_rate(side, mesh, spacing, nbody_steps, reps=1):
    """Particle-steps/s of the oracle for one forward + one adjoint step at a
    side^3 particle grid (same mesh ratio and spacing)."""
    import numpy as np
    from oracle import cosmo as oc, ics, nbody as onb
    conf = oc.OConf(spacing, (side,) * 3, mesh, float_dtype=np.float32,
                    a_nbody_maxstep=(1 - 1 / 64) / nbody_steps)
    cos = oc.with_tables(oc.simple_lcdm(A_s_1e9=COSMO['A_s_1e9'], n_s=COSMO['n_s']), conf)
    pmid, disp = ics.gen_grid(conf)
    rng = np.random.default_rng(0)
    disp = (disp + rng.normal(0, 0.1 * spacing, disp.shape)).astype(np.float32)
    vel = rng.normal(0, 0.01, disp.shape).astype(np.float32)
    st = onb.force(conf.a_nbody[0], onb.State(pmid, disp, vel), cos, conf)
    cot = onb.Cot(rng.normal(size=disp.shape).astype(np.float32),
                  rng.normal(size=disp.shape).astype(np.float32))
    a0, a1 = conf.a_nbody[0], conf.a_nbody[1]
    times = []
    for _ in range(reps):
        t = time.perf_counter()
        st1 = onb.integrate(a0, a1, st, cos, conf)
        sens = {'factors': [], 'Omega_m': 0.0}
        st1, cot1, _ = onb.force_adj(a1, st1, cot, cos, conf)
        onb.integrate_adj(a1, a0, st1, cot1, cos, 0.0, conf, sens)
        times.append(time.perf_counter() - t)
    n = conf.ptcl_num
    return n, times


DATA = 'synthetic: seeded white noise -> E&H linear power -> 2LPT at a=1/64'


def workload_config(args, world):
    """The workload both arms report (the GPU arm runs it whole, the CPU
    reference arm samples it)."""
    side = args.ptcl
    mside = int(round(side * args.mesh))
    return {'workload': f'{side}^3 ptcl / {mside}^3 mesh, box {side * args.spacing:g} Mpc/h, '
                        f'K forward leapfrog steps then their K reversible-adjoint steps of a '
                        f'{args.nbody_steps}-step run (rates per fwd+adj step pair)',
            'ptcl': side ** 3, 'mesh_cells': mside ** 3, 'parallelism': f'replicas x{world}',
            'deposit': args.deposit, 'tma_gathers': bool(args.tma),
            'l2': 'inputs larger than L2 (mesh 4.3 GB per array)'}


def run_reference(args, rank):
    if rank != 0:
        return
    side = args.cpu_sample
    cores = os.cpu_count()
    n, times = cpu_step_pair_rate(side, args.mesh, args.spacing, args.nbody_steps,
                                  reps=args.warmup + args.steps)
    timed = times[args.warmup:]
    value = n * len(timed) / sum(timed)
    sample = (f'NumPy/SciPy oracle (CPU restatement of pmwd; JAX is not installed), one forward '
              f'+ one adjoint leapfrog step per bench step at {side}^3 particles on a '
              f'{int(round(side * args.mesh))}^3 mesh (same mesh ratio and spacing as the '
              f'{args.ptcl}^3 workload); FFTs on {cores} threads, particle work single-threaded')
    line = {'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': UNIT,
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup,
            'ms_per_step': 1e3 * sum(timed) / len(timed), 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32', 'data': DATA,
            'config': workload_config(args, args.gpus),
            'cpu_baseline': {'value': value, 'unit': UNIT, 'cores': cores, 'kind': 'port',
                             'sample': sample},
            'e2e': {'value': value, 'unit': UNIT, 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def run_pmx(args, rank, world, local_rank):
    import numpy as np
    import torch
    import torch.distributed as dist

    import pmwd_gb300 as pg
    from pmwd_gb300 import _lib
    import importlib
    gnb = importlib.import_module("pmwd_gb300.nbody")

    torch.cuda.set_device(local_rank)
    dev = torch.device('cuda', local_rank)
    lib = _lib.load()

    side = args.ptcl
    conf = pg.Configuration(args.spacing, (side,) * 3, args.mesh,
                            a_nbody_maxstep=(1 - 1 / 64) / args.nbody_steps)
    cosmo = pg.boltzmann(pg.Cosmology(conf, **COSMO), conf)
    N, M = conf.ptcl_num, conf.mesh_size
    Mc = conf.mesh_shape[0] * conf.mesh_shape[1] * (conf.mesh_shape[2] // 2 + 1)

    # 2LPT initial conditions from seeded white noise (one realisation per rank)
    with torch.no_grad():
        modes = pg.white_noise(rank, conf, device=dev)
        modes = pg.linear_modes(modes, cosmo, conf)
        ptcl, _ = pg.lpt(modes, cosmo, conf)
        del modes
    pmid = ptcl.pmid.contiguous()
    disp = ptcl.disp.contiguous()
    vel = ptcl.vel.contiguous()
    disp0, vel0 = disp.clone(), vel.clone()   # the initial state of the whole-run measurement
    acc = torch.empty_like(disp)
    g = torch.Generator(device=dev)
    g.manual_seed(1234 + rank)
    disp_cot = torch.randn(disp.shape, generator=g, device=dev)
    vel_cot = torch.randn(disp.shape, generator=g, device=dev)
    alpha = torch.zeros_like(disp)
    torch.cuda.empty_cache()

    # factors of the run (float64 -> float32): the timed segment is its first
    # K forward steps, then the adjoint of those K steps (the last K rows of
    # the reverse-time adjoint table), as a run executes them
    fwd = gnb.op_factors(gnb.forward_ops(conf), cosmo, conf).detach()
    adj = gnb.op_factors(gnb.adjoint_ops(conf), cosmo, conf).detach()
    fwd32 = np.ascontiguousarray(fwd.to(torch.float32).numpy().reshape(-1, 3))
    adj32 = np.ascontiguousarray(adj.to(torch.float32).numpy().reshape(-1, 3))
    f_fwd = (_lib.c_f * 3)(*fwd32[0])
    f_adj = (_lib.c_f * 3)(*adj32[-1])
    Om = float(cosmo.Omega_m)

    ws = _lib.Workspace(conf.mesh_shape, adjoint=True, agg=args.deposit == 'agg',
                        window=args.deposit == 'window', tma=args.tma)
    spec = _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)
    dots = torch.zeros(4, dtype=torch.float64, device=dev)
    P = _lib.ptr
    if max(args.steps, args.warmup) > fwd32.shape[0]:
        raise SystemExit(f'--steps/--warmup exceed the {fwd32.shape[0]}-step run')
    seg_dots = torch.zeros((fwd32.shape[0], 4), dtype=torch.float64, device=dev)

    def segment(stream, k, mid_event=None):
        """The run's first k forward steps, then their k adjoint steps
        (multi-step calls: consecutive steps share particle passes)."""
        sf = np.ascontiguousarray(fwd32[:k])
        sa = np.ascontiguousarray(adj32[-k:])
        _lib.check(lib.pmx_nbody_steps(ws.handle, spec, P(pmid), P(disp), P(vel), P(acc), N, N,
                                       k, sf.ctypes.data_as(ctypes.c_void_p), Om, stream),
                   'pmx_nbody_steps')
        if mid_event is not None:
            mid_event.record(torch.cuda.current_stream(dev))
        _lib.check(lib.pmx_nbody_adj_steps(ws.handle, spec, P(pmid), P(disp), P(vel), P(acc),
                                           P(disp_cot), P(vel_cot), P(alpha), N, N, k,
                                           sa.ctypes.data_as(ctypes.c_void_p), Om,
                                           P(seg_dots), stream), 'pmx_nbody_adj_steps')

    def step_fwd(stream):
        _lib.check(lib.pmx_nbody_step(ws.handle, spec, P(pmid), P(disp), P(vel), P(acc), N, N,
                                      f_fwd, Om, stream), 'pmx_nbody_step')

    def step_adj(stream):
        _lib.check(lib.pmx_nbody_adj_step(ws.handle, spec, P(pmid), P(disp), P(vel), P(acc),
                                          P(disp_cot), P(vel_cot), P(alpha), N, N, f_adj, Om,
                                          P(dots), stream), 'pmx_nbody_adj_step')

    def step(stream):
        step_fwd(stream)
        step_adj(stream)

    stream = torch.cuda.current_stream(dev)
    sp = _lib.c_p(stream.cuda_stream)
    _lib.check(lib.pmx_force(ws.handle, spec, P(pmid), P(disp), N, N, Om, P(acc), sp), 'force')
    segment(sp, args.warmup)
    step(sp)                       # the single-step entry points used by e2e
    torch.cuda.synchronize()
    _lib.profile_read(ws)  # clear counters

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local_rank)
    clocks.start()
    lib.pmx_profile_enable(ws.handle, 1)
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    em = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    torch.cuda.nvtx.range_push('timed')   # lets ncu --nvtx-include timed/ select these launches
    segment(sp, args.steps, em)
    torch.cuda.nvtx.range_pop()
    e1.record(stream)
    barrier()
    lib.pmx_profile_enable(ws.handle, 0)
    clk = clocks.stop()
    ms_total = e0.elapsed_time(e1)
    ms_fwd = e0.elapsed_time(em) / args.steps   # the forward half of the segment
    stages, launches = _lib.profile_read(ws)
    ms_total, value = replica_throughput(ms_total, N * args.steps, world, dev)
    ms_step = ms_total / args.steps

    # ---- e2e: the same step pair through the C ABI with host buffers ----
    e2e = None
    dev_bufs = host = None
    if not args.no_e2e:
        dev_bufs = dict(pmid=pmid, disp=disp, vel=vel, acc=acc, disp_cot=disp_cot,
                        vel_cot=vel_cot, alpha=alpha)
        host = {}
        for k, v in dev_bufs.items():
            host[k] = torch.empty(v.shape, dtype=v.dtype, pin_memory=True)
            host[k].copy_(v)
        h2d = sum(v.numel() * v.element_size() for v in host.values())
        outs = ('disp', 'vel', 'acc', 'disp_cot', 'vel_cot', 'alpha')
        d2h = sum(host[k].numel() * host[k].element_size() for k in outs)
        ke = max(2, min(args.steps, 5))
        # Each step's inputs are the previous step's results read back to
        # the host.  One stream uploads and one downloads, each in order
        # (a GB300's link to its Grace host carries both directions at once:
        # 211 GB/s up and 194 GB/s down, 343 GB/s together, measured; many
        # copy streams of mixed directions got 203 GB/s in all).  A
        # buffer goes up once the previous step no longer reads its device
        # copy and its download has landed; the forward step starts once
        # its own inputs are up, while the adjoint's inputs still upload.
        # Copies go in chunks of 256 MB, so an upload trails the download of
        # the same buffer by one chunk instead of one buffer.
        fwd_in = ('pmid', 'disp', 'vel', 'acc')
        adj_in = ('disp_cot', 'vel_cot', 'alpha')
        chunk = 256 << 20

        def pieces(k):
            d, h = dev_bufs[k].view(-1), host[k].view(-1)
            step_n = max(1, chunk // d.element_size())
            return [(d[a:a + step_n], h[a:a + step_n]) for a in range(0, d.numel(), step_n)]

        parts = {k: pieces(k) for k in host}
        up, down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

        def link_rate():
            """This machine's host link for one 1.6 GB buffer: up, down, both at
            once (GB/s), for reading the e2e figure."""
            d, h = dev_bufs['disp'], host['disp']
            d2, h2 = dev_bufs['vel'], host['vel']
            nb = d.numel() * d.element_size()
            out = {}
            for name, jobs in (('h2d', [(up, d, h)]), ('d2h', [(down, h, d)]),
                               ('both', [(up, d, h), (down, h2, d2)])):
                best = 0.0
                for _ in range(3):           # the first copies warm the engines
                    torch.cuda.synchronize()
                    a = torch.cuda.Event(enable_timing=True)
                    b = torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    for st_, dst, src in jobs:
                        st_.wait_stream(stream)
                        with torch.cuda.stream(st_):
                            dst.copy_(src, non_blocking=True)
                        stream.wait_stream(st_)
                    b.record(stream)
                    torch.cuda.synchronize()
                    best = max(best, len(jobs) * nb / (a.elapsed_time(b) / 1e3) / 1e9)
                out[name] = best
            for k in ('disp', 'vel'):       # the buffers hold the step state again
                host[k].copy_(dev_bufs[k])
            return out

        link = link_rate()
        barrier()
        e0.record(stream)
        up.wait_stream(stream)
        done, landed = None, {}
        for _ in range(ke):
            if done is not None:
                up.wait_event(done)           # the previous step no longer reads them
            marks = {}
            for k in fwd_in + adj_in:
                for c, (d, h) in enumerate(parts[k]):
                    if (k, c) in landed:
                        up.wait_event(landed[k, c])   # the previous result is on the host
                    with torch.cuda.stream(up):
                        d.copy_(h, non_blocking=True)
                if k in ('acc', 'alpha'):
                    marks[k] = torch.cuda.Event()
                    marks[k].record(up)
            stream.wait_event(marks['acc'])
            step_fwd(sp)
            stream.wait_event(marks['alpha'])
            step_adj(sp)
            done = torch.cuda.Event()
            done.record(stream)
            down.wait_event(done)
            for k in outs:
                for c, (d, h) in enumerate(parts[k]):
                    with torch.cuda.stream(down):
                        h.copy_(d, non_blocking=True)
                    landed[k, c] = torch.cuda.Event()
                    landed[k, c].record(down)
        stream.wait_stream(down)
        stream.wait_stream(up)
        e1.record(stream)
        barrier()
        t = torch.tensor([e0.elapsed_time(e1)], dtype=torch.float64, device=dev)
        if world > 1:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e = {'value': world * N * ke / (float(t) / 1e3), 'unit': UNIT,
               'h2d_bytes_per_step': h2d, 'd2h_bytes_per_step': d2h,
               'steps': ke, 'link_gbs': link, 'path': 'pmx_nbody_step + pmx_nbody_adj_step (C ABI), pinned host '
                                    'buffers copied in and out every step, each step\'s inputs '
                                    'the previous step\'s results read back (one upload and one '
                                    'download stream, 256 MB chunks; the adjoint inputs upload '
                                    'during the forward step)'}

    # ---- the whole run: every forward step, then every adjoint step ----
    full = None
    if not args.no_full_run:
        full = full_run(lib, ws, spec, pmid, disp0, vel0, disp_cot, vel_cot, alpha, acc, N,
                        fwd32, adj32, Om, stream, dev, world, local_rank, barrier)

    if rank != 0:
        return

    # ---- roofline of the dominant own kernel and of the whole step ----
    peak, peak_kind = measured_peak()
    ab = algorithmic_bytes(N, M, Mc)
    traffic = ncu_traffic()
    stage_rows = {}
    for name, (ms, calls) in stages.items():
        if calls == 0:
            continue
        per = ms / calls
        b = ab.get(name)
        stage_rows[name] = {'ms_per_step': ms / args.steps, 'ms_per_launch': per,
                            'gbs': (b / (per / 1e3) / 1e9) if b else None}
    own = {k: v for k, v in stage_rows.items() if k in OWN_KERNELS}
    dom = max(own, key=lambda k: own[k]['ms_per_step'])
    ach = stage_rows[dom]['gbs']
    tr = traffic.get(dom)
    # the summary is of the 512^3 / 1024^3 step; every operand scales with
    # N (M = 8 N at mesh factor 2), other mesh factors have no capture
    tr = tr * N / 512 ** 3 if tr is not None and args.mesh == 2 else None
    roofline = {'bound': 'hbm', 'kernel': dom, 'achieved': ach, 'peak': peak, 'unit': 'GB/s',
                'frac': ach / peak, 'traffic': tr,
                'algorithmic_bytes': ab[dom], 'peak_kind': f'{peak_kind} (MEASURED_PEAKS.json hbm_gbs)'
                if peak_kind == 'measured' else 'fallback 6.8 TB/s'}
    # whole-step compulsory bytes, a fixed convention (each stage's
    # compulsory operands once): forward step 156 N + 64 M, adjoint step
    # 336 N + 140 M
    step_bytes = 492 * N + 204 * M
    step_gbs = step_bytes / (ms_step / 1e3) / 1e9

    cpu = None
    if not args.no_cpu:
        cs = args.cpu_sample
        n_cpu, times = cpu_step_pair_rate(cs, args.mesh, args.spacing, args.nbody_steps, reps=1)
        cpu = {'value': n_cpu / times[0], 'unit': UNIT, 'cores': os.cpu_count(), 'kind': 'port',
               'sample': f'one fwd+adj step pair of the NumPy/SciPy oracle at {cs}^3 particles / '
                         f'{int(round(cs * args.mesh))}^3 mesh ({times[0]:.1f} s); FFTs on all '
                         f'cores, particle work single-threaded'}

    # the serving stream (the metric's second half), after the large run's
    # buffers are released
    serve = None
    if args.serve_requests > 0 and world == 1:
        del pmid, disp, vel, acc, disp_cot, vel_cot, alpha, disp0, vel0, ws, seg_dots, dots
        del dev_bufs, host
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        sides = tuple(int(s) for s in args.serve_sides.split(','))
        steps_rng = tuple(int(s) for s in args.serve_steps.split(','))
        serve = serving_measure(args.serve_requests, sides, steps_rng)

    line = {
        'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': ms_step, 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
        'data': DATA,
        'config': workload_config(args, world),
        'roofline': roofline,
        'step_roofline': {'bytes_per_step': step_bytes, 'achieved': step_gbs, 'peak': peak,
                          'frac': step_gbs / peak, 'unit': 'GB/s',
                          'convention': '492 N + 204 M bytes per fwd+adj step pair '
                                        '(forward 156 N + 64 M, adjoint 336 N + 140 M)'},
        'stages': stage_rows,
        'cpu_baseline': cpu,
        'e2e': e2e,
        'gpu_launches': launches,
        'forward_only': {'ms_per_step': ms_fwd, 'value': N / (ms_fwd / 1e3), 'unit': UNIT,
                         'note': 'forward half of the timed segment (the metric of the '
                                 'reference\'s published per-step N-body timings)'},
        'full_run': None if full is None else dict(
            full, step_roofline_frac=step_bytes / (full['ms_per_step'] / 1e3) / 1e9 / peak),
        'clocks': clk,
        'serving': serve,
    }
    print(json.dumps(line), flush=True)


def full_run(lib, ws, spec, pmid, disp0, vel0, disp_cot, vel_cot, alpha, acc, N, fwd32, adj32,
             Om, stream, dev, world, local_rank, barrier):
    """All steps of the run from the 2LPT state, as nbody() and its backward
    execute them: force at a_start, every forward step in one multi-step
    call, the force VJP at a_stop, every adjoint step in one multi-step call
    (late, clustered steps included, where the timed segment has the first
    steps only).  Rates per fwd+adj step pair."""
    import torch
    from pmwd_gb300 import _lib
    P = _lib.ptr
    nsteps = fwd32.shape[0]
    disp, vel = disp0.clone(), vel0.clone()
    dd = torch.zeros((nsteps + 1, 4), dtype=torch.float64, device=dev)
    sp = _lib.c_p(stream.cuda_stream)
    e0, em, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    clocks = ClockSampler(local_rank)
    clocks.start()
    lib.pmx_profile_enable(ws.handle, 1)
    barrier()
    e0.record(stream)
    _lib.check(lib.pmx_force(ws.handle, spec, P(pmid), P(disp), N, N, Om, P(acc), sp), 'force')
    _lib.check(lib.pmx_nbody_steps(ws.handle, spec, P(pmid), P(disp), P(vel), P(acc), N, N, nsteps,
                                   fwd32.ctypes.data_as(ctypes.c_void_p), Om, sp),
               'pmx_nbody_steps')
    em.record(stream)
    _lib.check(lib.pmx_force_vjp(ws.handle, spec, P(pmid), P(disp), N, N, Om, P(vel_cot), P(acc),
                                 P(alpha), P(dd[nsteps, 3:]), sp), 'pmx_force_vjp')
    _lib.check(lib.pmx_nbody_adj_steps(ws.handle, spec, P(pmid), P(disp), P(vel), P(acc),
                                       P(disp_cot), P(vel_cot), P(alpha), N, N, nsteps,
                                       adj32.ctypes.data_as(ctypes.c_void_p), Om, P(dd), sp),
               'pmx_nbody_adj_steps')
    e1.record(stream)
    barrier()
    lib.pmx_profile_enable(ws.handle, 0)
    clk = clocks.stop()
    stages, launches = _lib.profile_read(ws)
    ms, value = replica_throughput(e0.elapsed_time(e1), N * nsteps, world, dev)
    back = float((disp - disp0).norm() / disp0.norm())
    return {'steps': nsteps, 'ms_total': ms, 'ms_per_step': ms / nsteps, 'value': value,
            'unit': UNIT, 'forward_ms_per_step': e0.elapsed_time(em) / nsteps,
            'adjoint_ms_per_step': em.elapsed_time(e1) / nsteps,
            'stages_ms_per_step': {k: v[0] / nsteps for k, v in stages.items() if v[1]},
            'gpu_launches': launches, 'reversibility_rel_disp': back, 'clocks': clk}


def run_dry(args, rank, world):
    """The replica launch without GPU work: each rank reports (100 + 10 rank)
    ms for N K particle-steps; rank 0 prints the reduced line."""
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group('gloo')
    n = args.ptcl ** 3
    ms, value = replica_throughput(100.0 + 10.0 * rank, n * args.steps, world, 'cpu')
    if rank == 0:
        print(json.dumps({'metric': METRIC, 'value': value, 'unit': UNIT, 'n_gpus': world,
                          'steps': args.steps, 'ms_per_step': ms / args.steps, 'dry_run': True,
                          'config': workload_config(args, world)}), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def launch_replicas(args):
    """``--gpus N`` outside torchrun: start N ranks (one replica simulation
    per GPU) with torch.distributed.run on this node and pass their output
    through; the exit status is the launcher's."""
    import socket
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    cmd = [sys.executable, '-m', 'torch.distributed.run', '--nnodes=1',
           f'--nproc-per-node={args.gpus}', '--master-addr', '127.0.0.1', '--master-port',
           str(port), os.path.abspath(__file__), *sys.argv[1:]]
    return subprocess.call(cmd)


def serving_measure(n, sides, steps, realtime=True):
    """The serving stream (C5 distribution: particle grid from `sides`, mesh
    factor 1 or 2, steps uniform in `steps`, random cosmologies, 20%
    gradients) served with continuous batching and one at a time, the same
    requests; each server is warmed first with one short request per mesh
    group, so both are timed with their workspaces and plans in place.
    Then the served form under Poisson arrivals at 80% of its throughput,
    for p50/p99 latency."""
    from pmwd_gb300 import serving
    reqs = serving.make_stream(n, rate_hz=0.0, seed=0, sides=sides, steps=steps)
    warm = [serving.Request(1000 + i, s, f, 2, dict(sigma8=0.8, n_s=0.96, Omega_m=0.3,
                                                     Omega_b=0.05, h=0.7), i, grad=True)
            for i, (s, f) in enumerate((s, f) for s in sides for f in (1, 2))]
    seq_srv = serving.sequential_server()
    seq_srv.run(warm, realtime=False)
    _, seq = seq_srv.run(reqs, realtime=False)
    seq_srv.close()
    srv = serving.Server(budget_bytes=150e9)
    srv.run(warm, realtime=False)
    _, st = srv.run(reqs, realtime=False)
    out = {'served_sims_per_s': st['sims_per_s'], 'sequential_sims_per_s': seq['sims_per_s'],
           'speedup_vs_sequential': st['sims_per_s'] / seq['sims_per_s'],
           'failed': st['failed'] + seq['failed'], 'requests': n,
           'workload': f'{n} requests, ptcl grid {sides}^3, mesh factor {{1,2}}, steps U{steps}, '
                       f'20% gradients, HBM budget 150 GB, spacing 2 Mpc/h'}
    if realtime:
        rate = 0.8 * st['sims_per_s']
        timed = serving.make_stream(n, rate_hz=rate, seed=0, sides=sides, steps=steps)
        _, rt = srv.run(timed, realtime=True)
        out.update({'poisson_rate_hz': rate, 'p50_s': rt['p50_s'], 'p99_s': rt['p99_s'],
                    'realtime_sims_per_s': rt['sims_per_s']})
    srv.close()
    return out


def run_serve(args):
    """Serving mode of bench.py: serving_measure on --serve requests."""
    import torch
    torch.cuda.set_device(0)
    sides = tuple(int(s) for s in args.serve_sides.split(','))
    steps = tuple(int(s) for s in args.serve_steps.split(','))
    m = serving_measure(args.serve, sides, steps)
    line = {'metric': 'served sims/s', 'value': m['served_sims_per_s'], 'unit': 'sims/s',
            'higher_is_better': True, 'n_gpus': 1, **m, 'config': {'workload': m['workload']}}
    print(json.dumps(line), flush=True)


def run_contention(args):
    """Scatter/gather contention stress (256^3 particles on a 256^3 mesh in a
    64 Mpc/h box): one density scatter, one force and one 3-channel gather,
    timed on the particles evolved to a = 1 (63 steps, halos with hundreds
    of particles per cell) and on the same particles on the lattice."""
    import numpy as np
    import torch
    import importlib
    import pmwd_gb300 as pg
    from pmwd_gb300 import _lib
    gnb = importlib.import_module('pmwd_gb300.nbody')
    torch.cuda.set_device(0)
    dev = torch.device('cuda', 0)
    lib = _lib.load()
    side = 256
    conf = pg.Configuration(0.25, (side,) * 3, 1)
    cosmo = pg.boltzmann(pg.Cosmology(conf, **COSMO), conf)
    N, M = conf.ptcl_num, conf.mesh_size
    with torch.no_grad():
        ptcl, _ = pg.lpt(pg.linear_modes(pg.white_noise(0, conf, device=dev), cosmo, conf),
                         cosmo, conf)
    pmid = ptcl.pmid.contiguous()
    disp = ptcl.disp.detach().contiguous().clone()
    vel = ptcl.vel.detach().contiguous().clone()
    acc = torch.empty_like(disp)
    ws = _lib.workspace(conf.mesh_shape, adjoint=True)
    spec = _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)
    P = _lib.ptr
    stream = _lib.c_p(torch.cuda.current_stream(dev).cuda_stream)
    Om = float(cosmo.Omega_m)
    fwd = gnb.op_factors(gnb.forward_ops(conf), cosmo, conf).detach()
    f_fwd = fwd.to(torch.float32).numpy().reshape(-1, 3)
    _lib.check(lib.pmx_force(ws.handle, spec, P(pmid), P(disp), N, N, Om, P(acc), stream),
               'pmx_force')
    for i in range(f_fwd.shape[0]):
        fac = (_lib.c_f * 3)(*f_fwd[i])
        _lib.check(lib.pmx_nbody_step(ws.handle, spec, P(pmid), P(disp), P(vel), P(acc), N, N, fac,
                                      Om, stream), 'pmx_nbody_step')
    torch.cuda.synchronize()
    mesh = torch.zeros(conf.mesh_shape, dtype=torch.float32, device=dev)
    mesh3 = torch.randn(conf.mesh_shape + (3,), dtype=torch.float32, device=dev)
    out3 = torch.empty((N, 3), dtype=torch.float32, device=dev)
    val = float(M / N)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, reps):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    # the force VJP (density deposit, gather VJP with its 24 reductions per
    # particle, scatter VJP), through plain atomics and warp windows
    ws_win = _lib.Workspace(conf.mesh_shape, adjoint=True, window=True)
    ws_agg = _lib.Workspace(conf.mesh_shape, adjoint=True, agg=True)
    cot = torch.randn((N, 3), dtype=torch.float32, device=dev,
                      generator=torch.Generator(device=dev).manual_seed(5))
    dcot = torch.empty_like(cot)
    om_cot = torch.zeros((), dtype=torch.float64, device=dev)

    def vjp_stages(w, d, reps=5):
        def fv():
            _lib.check(lib.pmx_force_vjp(w.handle, spec, P(pmid), P(d), N, N, Om, P(cot), P(acc),
                                         P(dcot), P(om_cot), stream), 'pmx_force_vjp')
        for _ in range(2):
            fv()
        torch.cuda.synchronize()
        _lib.profile_read(w)
        lib.pmx_profile_enable(w.handle, 1)
        t = timed(fv, reps)
        lib.pmx_profile_enable(w.handle, 0)
        st, _ = _lib.profile_read(w)
        return {'force_vjp_ms': t,
                'deposit_ms': st['deposit_fwd'][0] / max(st['deposit_fwd'][1], 1),
                'gather3_adj_ms': st['gather3_adj'][0] / max(st['gather3_adj'][1], 1)}

    res = {}
    for name, d in (('clustered', disp), ('lattice', torch.zeros_like(disp))):
        res[name] = {'vjp_atomics': vjp_stages(ws, d), 'vjp_windows': vjp_stages(ws_win, d),
                     'vjp_aggregated': vjp_stages(ws_agg, d)}
        def sc():
            mesh.zero_()
            _lib.check(lib.pmx_scatter(spec, P(pmid), P(d), N, None, val, 1, P(mesh), stream),
                       'pmx_scatter')
        def fo():
            _lib.check(lib.pmx_force(ws.handle, spec, P(pmid), P(d), N, N, Om, P(acc), stream),
                       'pmx_force')
        def ga():
            _lib.check(lib.pmx_gather(spec, P(pmid), P(d), N, P(mesh3), 3, None, 0.0, P(out3),
                                      stream), 'pmx_gather')
        t_zero = timed(lambda: mesh.zero_(), 10)
        sc()
        torch.cuda.synchronize()
        peak = float(mesh.max()) / val  # particles (CIC weight) in the fullest cell
        res[name].update({'scatter_ms': timed(sc, 10) - t_zero, 'force_ms': timed(fo, 5),
                          'gather3_ms': timed(ga, 10), 'max_ptcl_per_cell': peak})
        for k in ('scatter', 'gather3'):
            res[name][k + '_ptcl_per_s'] = N / (res[name][k + '_ms'] / 1e3)
    line = {'metric': 'scatter/gather contention (C3)', 'unit': 'ms',
            'config': {'workload': f'{side}^3 ptcl / {side}^3 mesh, box 64 Mpc/h, evolved to a=1 '
                                   f'in {f_fwd.shape[0]} steps vs the lattice',
                       'ptcl': N, 'mesh_cells': M},
            'clustered': res['clustered'], 'lattice': res['lattice'],
            'clustered_over_lattice': {k: res['clustered'][k] / res['lattice'][k]
                                       for k in ('scatter_ms', 'force_ms', 'gather3_ms')}}
    print(json.dumps(line), flush=True)


# pmwd's own timing table on an H100 PCIe (docs/papers/adjoint/perf.txt,
# made by docs/papers/adjoint/perf.py): rows growth tables, 2LPT, N-body per
# step at mesh factor 1 and 2; columns particle grids 32^3 .. 512^3; seconds.
PUBLISHED_PERF = {
    'growth': (9.656670968979597e-03, 9.563866071403027e-03, 9.559712023474276e-03,
               9.568694978952408e-03, 9.575393050909042e-03),
    'lpt': (7.556179771199822e-04, 7.496170001104474e-04, 1.957484055310488e-03,
            1.269906898960472e-02, 9.726452908944339e-02),
    'nbody_mesh1': (7.354481240327004e-04, 7.306391089514364e-04, 1.220740359713091e-03,
                    7.984881642187247e-03, 9.461856014058867e-02),
    'nbody_mesh2': (7.260151724040043e-04, 7.381303748843493e-04, 2.829991937687736e-03,
                    2.185595865739742e-02, 2.074725039365148e-01),
}


def run_published(args):
    """pmwd's own performance table (perf.py) through this package's API:
    for particle grids 32^3 .. 512^3 (spacing 1 Mpc/h, 63 steps from
    a = 1/64) and mesh factors 1 and 2, the minimum wall time of the growth
    tables (boltzmann), of 2LPT from the linear modes, and of a whole
    forward N-body run divided by its 64 force evaluations, each beside the
    H100 figure.  Timing as perf.py: wall clock around a call that waits
    for the device, minimum over repeats."""
    import torch
    import pmwd_gb300 as pg
    torch.cuda.set_device(0)
    dev = torch.device('cuda', 0)
    sides = (32, 64, 128, 256, 512)
    out = {}

    def best(fn, reps):
        ts = []
        for _ in range(reps + 1):   # the first call warms up (plans, workspaces)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return min(ts[1:])

    for mf in (1, 2):
        for c, side in enumerate(sides):
            conf = pg.Configuration(1.0, (side,) * 3, mesh_shape=mf)
            reps = 3 if side >= 512 else 5
            with torch.no_grad():
                cosmo0 = pg.SimpleLCDM(conf)
                t_growth = best(lambda: pg.boltzmann(cosmo0, conf, varlin=False), reps)
                cosmo = pg.boltzmann(cosmo0, conf)
                modes = pg.white_noise(0, conf, device=dev)
                t_lpt = best(lambda: pg.lpt(pg.linear_modes(modes, cosmo, conf), cosmo, conf), reps)
                ptcl, obs = pg.lpt(pg.linear_modes(modes, cosmo, conf), cosmo, conf)
                nforce = 1 + conf.a_nbody_num
                t_nb = best(lambda: pg.nbody(ptcl, obs, cosmo, conf), reps) / nforce
            key = f'{side}^3 mesh x{mf}'
            row = {'nbody_ms_per_step': 1e3 * t_nb,
                   'nbody_published_ms': 1e3 * PUBLISHED_PERF[f'nbody_mesh{mf}'][c],
                   'nbody_speedup': PUBLISHED_PERF[f'nbody_mesh{mf}'][c] / t_nb,
                   'ptcl_steps_per_s': side ** 3 / t_nb}
            if mf == 2:   # perf.py's growth and 2LPT rows come from its mesh x2 pass
                row.update({'lpt_ms': 1e3 * t_lpt, 'lpt_published_ms': 1e3 * PUBLISHED_PERF['lpt'][c],
                            'growth_ms': 1e3 * t_growth,
                            'growth_published_ms': 1e3 * PUBLISHED_PERF['growth'][c]})
            out[key] = row
            print(json.dumps({key: row}), file=sys.stderr, flush=True)
            del ptcl, obs, modes
            torch.cuda.empty_cache()
    line = {'metric': "pmwd's published timing table (perf.py) on GB300", 'unit': 'ms',
            'config': {'workload': 'ptcl grids 32^3..512^3, spacing 1 Mpc/h, mesh x1 and x2, '
                                   '63 steps from a=1/64, 2LPT, growth tables',
                       'published_hardware': 'H100 PCIe (docs/papers/adjoint/perf.txt)',
                       'timing': 'wall clock, min over repeats, device synchronised'},
            'rows': out}
    print(json.dumps(line), flush=True)


def run_gradient(args):
    """The reference quickstart's gradient workload (docs/examples/
    quickstart.ipynb): 256^3 particles, 512^3 mesh, spacing 1 Mpc/h, 63
    steps; objective var(scatter(nbody(lpt(linear_modes(modes))))) - target)
    with the target from another white-noise seed, differentiated with
    respect to the real white-noise modes and the five SimpleLCDM parameters
    (boltzmann included in the differentiated function).  Wall time of a
    warm call, device synchronised; pmwd publishes 5.27 s on an H100 PCIe
    (and 1.43 s for the forward model)."""
    import torch
    import pmwd_gb300 as pg
    torch.cuda.set_device(0)
    dev = torch.device('cuda', 0)
    conf = pg.Configuration(1.0, (256,) * 3, mesh_shape=2)
    names = ('A_s_1e9', 'n_s', 'Omega_m', 'Omega_b', 'h')
    base = pg.SimpleLCDM(conf)

    def model(modes, cosmo):
        cosmo = pg.boltzmann(cosmo, conf)
        modes = pg.linear_modes(modes, cosmo, conf)
        ptcl, obs = pg.lpt(modes, cosmo, conf)
        return pg.nbody(ptcl, obs, cosmo, conf)

    with torch.no_grad():
        ptcl, _ = model(pg.white_noise(0, conf, device=dev), base)
        tgt = pg.scatter(ptcl, conf)
    modes = pg.white_noise(1, conf, real=True, device=dev)

    def obj_grad():
        m = modes.clone().requires_grad_(True)
        prm = {k: torch.tensor(float(getattr(base, k)), dtype=torch.float64, requires_grad=True)
               for k in names}
        ptcl, _ = model(m, base.replace(**prm))
        loss = (pg.scatter(ptcl, conf) - tgt).var(correction=0)
        loss.backward()
        return float(loss.detach()), m.grad, {k: float(v.grad) for k, v in prm.items()}

    def timed(fn, reps=3):
        ts, out = [], None
        for _ in range(reps + 1):   # the first call warms plans and workspaces
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return min(ts[1:]), out

    with torch.no_grad():
        t_fwd, _ = timed(lambda: model(modes, base))
    t_grad, (loss, mgrad, cgrad) = timed(obj_grad)
    line = {'metric': "quickstart gradient (pmwd's docs/examples/quickstart.ipynb)", 'unit': 's',
            'config': {'workload': '256^3 ptcl, 512^3 mesh, spacing 1 Mpc/h, 63 steps; objective '
                                   'var(scatter(nbody(lpt(linear_modes(modes)))) - target); '
                                   'gradient w.r.t. white-noise modes and 5 cosmological parameters',
                       'published_hardware': 'H100 PCIe (quickstart.ipynb)',
                       'timing': 'wall clock of a warm call, min over 3, device synchronised'},
            'gradient_s': t_grad, 'gradient_published_s': 5.27,
            'gradient_speedup': 5.27 / t_grad,
            'forward_model_s': t_fwd, 'forward_model_published_s': 1.43,
            'loss': loss, 'modes_grad_std': float(mgrad.std()),
            'cosmo_grad': cgrad}
    print(json.dumps(line), flush=True)


def run_powspec(args):
    """Power spectrum of an n^3 Gaussian field (spec_util.py:50-147): torch's
    rfftn (cuFFT), then the binning pass (pmx_powspec_bin*) for pmwd's
    default log bins (1j/3) and for unit linear bins, each after a call
    that caches the grid's k and N sums; CUDA events, mean of 5 calls."""
    import torch
    from pmwd_gb300 import spec_util
    torch.cuda.set_device(0)
    dev = torch.device('cuda', 0)
    n = args.powspec
    grid = (n, n, n)
    f = torch.randn(grid, device=dev, generator=torch.Generator(device=dev).manual_seed(0))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    F = spec_util.fftfwd(f, axes=(-3, -2, -1))
    out = {'rfftn_ms': timed(lambda: spec_util.fftfwd(f, axes=(-3, -2, -1)))}
    for name, bins in (('log_1j/3', 1j / 3), ('linear_unit', 1.0)):
        bnum, _, edges, right = spec_util._getbins(grid, bins, True)
        out[name] = {'bins': bnum, 'binning_ms': timed(
            lambda: spec_util._bin_cuda(F, None, grid, edges, right, bnum, None)),
            'spectrum_gb': F.numel() * 8 / 1e9}
        out[name]['gbs'] = out[name]['spectrum_gb'] / out[name]['binning_ms'] * 1e3
    print(json.dumps({'metric': 'power spectrum binning', 'unit': 'ms',
                      'config': {'workload': f'{n}^3 Gaussian field, complex64 half spectrum'},
                      **out}), flush=True)


def main():
    args = parse()
    if args.gpus > 1 and 'WORLD_SIZE' not in os.environ and args.impl == 'pmx':
        sys.exit(launch_replicas(args))
    rank = int(os.environ.get('RANK', 0))
    world = int(os.environ.get('WORLD_SIZE', 1))
    local_rank = int(os.environ.get('LOCAL_RANK', 0))
    if args.impl == 'reference':
        run_reference(args, rank)
        return
    if args.dry_run:
        run_dry(args, rank, world)
        return
    if args.serve:
        if rank == 0:
            run_serve(args)
        return
    if args.contention:
        if rank == 0:
            run_contention(args)
        return
    if args.published:
        if rank == 0:
            run_published(args)
        return
    if args.gradient:
        if rank == 0:
            run_gradient(args)
        return
    if args.powspec:
        if rank == 0:
            run_powspec(args)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group('nccl')
    run_pmx(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == '__main__':
    main()
