"""Serving: request stream, admission logic (CPU) and, on the GPU, that every
result is the same alone and in the continuously batched mix."""

import numpy as np
import pytest

from pmwd_gb300 import serving


def test_make_stream_distribution():
    reqs = serving.make_stream(400, rate_hz=50.0, seed=3)
    sides = {r.ptcl_side for r in reqs}
    assert sides <= {64, 128, 256} and len(sides) == 3
    assert {r.mesh_factor for r in reqs} == {1, 2}
    assert all(10 <= r.steps <= 100 for r in reqs)
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) >= 0)
    assert abs(np.mean(np.diff(arr)) * 50.0 - 1) < 0.2        # Poisson, rate 50 Hz
    frac = np.mean([r.grad for r in reqs])
    assert 0.12 < frac < 0.28
    om = np.array([r.cosmo['Omega_m'] for r in reqs])
    assert om.min() >= 0.2 and om.max() <= 0.4


def test_admission_cost_monotone():
    small = serving.Request(0, 64, 1, 10, {}, 0)
    big = serving.Request(1, 256, 2, 10, {}, 0)
    grad = serving.Request(2, 256, 2, 10, {}, 0, grad=True)
    for batch in (True, False):
        eng = serving.GpuEngine.__new__(serving.GpuEngine)
        eng.budget, eng.batch = 150e9, batch
        c = eng.job_bytes
        assert c(small) < c(big) < c(grad)
        # a 256^3 / 512^3 gradient request with its group's workspace stays
        # well inside a 150 GB budget
        key = (512, 1.0)
        assert c(grad) + eng.group_bytes(key) < 150e9 / 2
    # batched groups: up to 8 simulations, the workspace at most a quarter
    # of the budget; meshes outside the fused x pass are not batched
    assert serving.group_slots(128, 150e9) == 8
    assert 1 <= serving.group_slots(512, 150e9) < 8
    assert serving.group_slots(32, 150e9) == serving.group_slots(96, 150e9) == 1


class FakeEngine:
    """Host-only stand-in for GpuEngine: a simulation's 'position' counts
    the steps it went forward (and back for gradients); failures are
    injected by request id."""

    def __init__(self, slots=4, fail_setup=(), reject=(), crash=(), group_bytes=1e9):
        self._slots, self.gb = slots, group_bytes
        self.fail_setup, self.reject, self.crash = set(fail_setup), set(reject), set(crash)
        self.calls, self.dropped, self.released = [], [], []

    def slots(self, key):
        return self._slots

    def group_bytes(self, key):
        return self.gb

    def job_bytes(self, req):
        return serving.request_bytes(req.ptcl_side, req.grad)

    def setup(self, job):
        if job.req.rid in self.fail_setup:
            raise RuntimeError('setup failed on the host')
        job.dev = {'pos': 0, 'back': None}

    def _check(self, jobs):
        rids = {j.req.rid for j in jobs}
        if rids & self.reject:
            raise serving.BatchRejected('rejected before launch')
        if rids & self.crash:
            raise RuntimeError('device error')

    def fwd(self, jobs, init, k):
        self._check(jobs)
        self.calls.append(('fwd', tuple(j.req.rid for j in jobs), init, k))
        for j in jobs:
            j.dev['pos'] += k

    def adj_init(self, jobs):
        self._check(jobs)
        self.calls.append(('adj_init', tuple(j.req.rid for j in jobs), 1, 0))

    def adj(self, jobs, k):
        self._check(jobs)
        self.calls.append(('adj', tuple(j.req.rid for j in jobs), 0, k))
        for j in jobs:
            j.dev['pos'] -= k

    def objective(self, job):
        job.dev['obj'] = job.dev['pos']

    def backprop(self, job):
        job.dev['back'] = job.dev['pos']

    def idle(self, job):
        return True

    def result(self, job):
        d = job.dev
        return serving.Result(job.req.rid, None, disp_rms=float(d['pos']), obj=float(d['obj']),
                              grad_rms=None if d['back'] is None else float(d['back']))

    def release(self, job):
        self.released.append(job.req.rid)
        job.dev = None

    def resident(self):
        return []

    def drop(self, key):
        self.dropped.append(key)

    def synchronize(self):
        pass


def _reqs(n, side=16, factor=2, steps=(5, 12), grad_every=3):
    return [serving.Request(i, side, factor, steps[0] + (i * 5) % (steps[1] - steps[0] + 1), {},
                            i, grad=(i % grad_every == 0)) for i in range(n)]


def test_scheduler_groups_equal_meshes_in_batched_calls():
    """Requests of one mesh group advance together: each call carries up to
    `slots` simulations, a chunk is at most STEP_CHUNK steps and never more
    than any member has left; every simulation ends with all its steps done
    (and undone, for gradients)."""
    reqs = _reqs(6) + [serving.Request(6, 32, 1, 7, {}, 6)]   # another mesh
    eng = FakeEngine(slots=4)
    res, st = serving.Scheduler(eng, budget_bytes=100e9).run(reqs, realtime=False)
    assert st['sims'] == 7 and st['failed'] == 0
    for r, q in zip(res, reqs):
        assert r.error is None and r.obj == q.steps
        if q.grad:
            assert r.grad_rms == 0.0
    key_of = {q.rid: (q.ptcl_side * q.mesh_factor) for q in reqs}
    for kind, rids, init, k in eng.calls:
        assert 1 <= len(rids) <= 4 and len({key_of[r] for r in rids}) == 1
        assert k <= serving.STEP_CHUNK
    # the first forward call of the 16^3 group carries four simulations
    first = [c for c in eng.calls if c[0] == 'fwd' and 0 in c[1]][0]
    assert len(first[1]) == 4 and first[2]
    assert sorted(eng.released) == list(range(7))


def test_scheduler_isolates_setup_failure_and_oversize():
    reqs = _reqs(5)
    reqs.append(serving.Request(5, 512, 2, 10, {}, 5))          # larger than the budget
    eng = FakeEngine(slots=2, fail_setup={1})
    res, st = serving.Scheduler(eng, budget_bytes=3e9).run(reqs, realtime=False)
    assert 'setup failed' in res[1].error
    assert res[5].error.startswith('over budget')
    for i in (0, 2, 3, 4):
        assert res[i].error is None and res[i].obj == reqs[i].steps
    assert st['sims'] == 4 and st['failed'] == 2
    assert 1 in eng.released                    # the failed request's memory is freed


def test_scheduler_rejected_batch_is_retried_one_by_one():
    """A batched call refused on the host (nothing launched) is reissued per
    simulation: only the culprit fails; a device error fails its call."""
    reqs = _reqs(4, grad_every=100)
    eng = FakeEngine(slots=4, reject={2})
    res, st = serving.Scheduler(eng, budget_bytes=100e9).run(reqs, realtime=False)
    assert 'rejected' in res[2].error
    assert all(res[i].error is None and res[i].obj == reqs[i].steps for i in (0, 1, 3))
    # a device error fails the simulations of its call (those whose setup
    # had finished by then); the others, and other groups, go on
    reqs = _reqs(4, grad_every=100) + [serving.Request(4, 32, 1, 6, {}, 4)]
    eng = FakeEngine(slots=4, crash={0})
    res, st = serving.Scheduler(eng, budget_bytes=100e9).run(reqs, realtime=False)
    assert 'device error' in res[0].error
    for i in (1, 2, 3):
        assert (res[i].error is not None and 'device error' in res[i].error) or (
            res[i].error is None and res[i].obj == reqs[i].steps)
    assert res[4].error is None and res[4].obj == 6


def test_scheduler_cancel_frees_the_slot():
    """A budget that holds two requests: cancelling an active one between
    steps ends it with 'cancelled' and lets the waiting ones in; cancelling a
    waiting one drops it."""
    reqs = _reqs(4, steps=(40, 40), grad_every=100)
    one = serving.request_bytes(16, False)
    eng = FakeEngine(slots=1, group_bytes=0)
    turns = []

    def on_turn(sched, t):
        turns.append(t)
        if len(turns) == 3:
            sched.cancel(0)
            sched.cancel(3)

    res, st = serving.Scheduler(eng, budget_bytes=2.5 * one).run(reqs, realtime=False,
                                                                 on_turn=on_turn)
    assert res[0].error == 'cancelled' and res[3].error == 'cancelled'
    assert res[1].error is None and res[2].error is None
    assert res[1].obj == 40 and res[2].obj == 40
    assert 3 not in eng.released               # never admitted


@pytest.mark.gpu
def test_results_same_alone_and_in_mix(cuda):
    """Meshes of 16^3..64^3: the 64^3 requests of equal cell size form
    batched groups, the smaller meshes run one simulation per call."""
    reqs = serving.make_stream(6, rate_hz=0.0, seed=11, sides=(16, 32), factors=(1, 2),
                               steps=(4, 8), grad_frac=0.5)
    reqs[0].grad = True
    alone, st_seq = serving.run_sequential(reqs)
    srv = serving.Server(budget_bytes=8e9, max_jobs=8)
    mixed, st_mix = srv.run(reqs, realtime=False)
    srv.close()
    assert st_mix['sims'] == len(reqs) == st_seq['sims']
    # gradients: the bound of the batched-group test below, for the same
    # reason (atomic order, CIC cell boundaries)
    for a, m in zip(alone, mixed):
        assert a.rid == m.rid
        assert abs(m.obj / a.obj - 1) < 1e-4, (a, m)
        assert abs(m.disp_rms / a.disp_rms - 1) < 1e-5
        if a.grad_rms is not None:
            assert abs(m.grad_rms / a.grad_rms - 1) < 5e-3
            assert abs(m.dobj_dOm / a.dobj_dOm - 1) < 5e-3


@pytest.mark.gpu
def test_results_same_alone_and_in_one_batched_group(cuda):
    """Five requests of one 64^3-mesh group (32^3 particles at mesh factor 2,
    cell 1 Mpc/h) with different cosmologies, seeds and step counts, two of
    them gradients: served as one batched group they give the results they
    give one at a time through the single-simulation path."""
    reqs = serving.make_stream(5, rate_hz=0.0, seed=4, sides=(32,), factors=(2,), steps=(5, 9),
                               grad_frac=0.0)
    reqs[1].grad = reqs[3].grad = True
    alone, _ = serving.run_sequential(reqs)
    srv = serving.Server(budget_bytes=8e9, max_jobs=8)
    assert srv.engine.slots((64, 1.0)) > 1
    mixed, st = srv.run(reqs, realtime=False)
    srv.close()
    assert st['sims'] == 5 and st['failed'] == 0
    # the gradients sum cotangents over every step: the order of the float32
    # atomic adds moves a reconstructed particle across a CIC cell boundary
    # now and then, where the weight gradient jumps, and with 32^3 particles
    # one such particle moves the modes gradient's rms by a few 1e-3
    # (measured between the batched and the single-simulation run: 1.9e-3
    # for d obj / d Omega_m, 2.5e-3 for the rms)
    for a, m in zip(alone, mixed):
        assert abs(m.obj / a.obj - 1) < 1e-4, (a, m)
        assert abs(m.disp_rms / a.disp_rms - 1) < 1e-5
        if a.grad_rms is not None:
            assert abs(m.grad_rms / a.grad_rms - 1) < 5e-3
            assert abs(m.dobj_dOm / a.dobj_dOm - 1) < 5e-3


def test_workspace_bytes_counts_the_partials():
    """A workspace's estimate counts its meshes per slot plus the particle
    kernels' per-block float64 partial sums: 4 x 2^19 in a single-simulation
    workspace (one per block at one particle per thread), 4 x 2^16 per slot
    of a batched one."""
    one, two, eight = (serving.workspace_bytes(256, s) for s in (1, 2, 8))
    mesh = (two - 2 * 4 * 8 * 2 ** 16) / 2
    assert one == mesh + 4 * 8 * 2 ** 19
    assert eight == 8 * mesh + 8 * 4 * 8 * 2 ** 16
    assert mesh > 30 * 256 ** 3            # meshes, spectra and work areas
