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
    srv = serving.Server.__new__(serving.Server)
    small = serving.Request(0, 64, 1, 10, {}, 0)
    big = serving.Request(1, 256, 2, 10, {}, 0)
    grad = serving.Request(2, 256, 2, 10, {}, 0, grad=True)
    c = serving.Server.cost
    assert c(srv, small) < c(srv, big) < c(srv, grad)
    # a 256^3 / 512^3 gradient request stays well inside a 150 GB budget
    assert c(srv, grad) < 150e9 / 10


@pytest.mark.gpu
def test_results_same_alone_and_in_mix(cuda):
    reqs = serving.make_stream(6, rate_hz=0.0, seed=11, sides=(16, 32), factors=(1, 2),
                               steps=(4, 8), grad_frac=0.5)
    reqs[0].grad = True
    alone, st_seq = serving.run_sequential(reqs)
    mixed, st_mix = serving.Server(budget_bytes=8e9, max_jobs=8).run(reqs, realtime=False)
    assert st_mix['sims'] == len(reqs) == st_seq['sims']
    for a, m in zip(alone, mixed):
        assert a.rid == m.rid
        assert abs(m.obj / a.obj - 1) < 1e-4, (a, m)
        assert abs(m.disp_rms / a.disp_rms - 1) < 1e-5
        if a.grad_rms is not None:
            assert abs(m.grad_rms / a.grad_rms - 1) < 1e-3
            assert abs(m.dobj_dOm / a.dobj_dOm - 1) < 1e-3
