"""Batched simulations (pmx_nbody_steps_batch / pmx_nbody_adj_steps_batch):
several runs of one mesh shape and cell size advance in one call, one slot
each.  Every simulation must end where the single-simulation entry points
take it (pmx_force + pmx_nbody_steps, pmx_force_vjp + pmx_nbody_adj_steps),
up to the order of float32 atomic adds: the same tolerance as the
multi-step-vs-single-step equality of the unbatched path."""

import ctypes

import numpy as np
import pytest
import torch

import pmwd_gb300 as pg
from pmwd_gb300 import _lib

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel(a, b):
    return float((a.double() - b.double()).norm() / b.double().norm().clamp_min(1e-300))


def close_cot(a, b):
    """A cotangent array after reverse steps: the CIC weight gradient is
    piecewise constant, so the order of float32 atomic adds can move a
    reconstructed particle across a cell boundary and change its cotangent
    by O(1).  At most 0.2% of the particles are set aside; the rest agree to
    1e-4 and the whole array to 3e-2."""
    e = (a.double() - b.double()).norm(dim=1)
    keep = torch.argsort(e)[:len(e) - len(e) // 500]
    return rel(a[keep], b[keep]) < 1e-4 and rel(a, b) < 3e-2


def make_sim(cuda, ptcl, mesh_factor, spacing, seed, Om, nsteps):
    conf = pg.Configuration(spacing, ptcl, mesh_factor)
    grid = pg.Particles.gen_grid(conf, device=cuda)
    g = torch.Generator(device=cuda).manual_seed(seed)
    disp = (grid.disp + 0.8 * conf.cell_size *
            torch.randn(grid.disp.shape, generator=g, device=cuda)).contiguous()
    vel = (0.3 * torch.randn(disp.shape, generator=g, device=cuda)).contiguous()
    rng = np.random.default_rng(seed)
    fac = np.ascontiguousarray(rng.uniform(0.02, 0.2, (nsteps, 3)).astype(np.float32))
    return dict(conf=conf, pmid=grid.pmid, disp=disp, vel=vel, Om=Om, fac=fac,
                vcot=(torch.randn(disp.shape, generator=g, device=cuda)).contiguous(),
                dcot=(torch.randn(disp.shape, generator=g, device=cuda)).contiguous())


def single_run(sim, k, cuda):
    conf = sim['conf']
    ws = _lib.Workspace(conf.mesh_shape, adjoint=True)
    spec = _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)
    st = _lib.stream_ptr(cuda)
    n = len(sim['pmid'])
    disp, vel = sim['disp'].clone(), sim['vel'].clone()
    acc = torch.empty_like(disp)
    _lib.call('pmx_force', ws.handle, spec, sim['pmid'], disp, n, conf.ptcl_num, sim['Om'], acc, st)
    _lib.call('pmx_nbody_steps', ws.handle, spec, sim['pmid'], disp, vel, acc, n, conf.ptcl_num,
              k, sim['fac'].ctypes.data_as(ctypes.c_void_p), sim['Om'], st)
    fwd = (disp.clone(), vel.clone(), acc.clone())
    dcot, vcot = sim['dcot'].clone(), sim['vcot'].clone()
    alpha = torch.zeros_like(disp)
    dots = torch.zeros((k + 1, 4), dtype=torch.float64, device=cuda)
    _lib.call('pmx_force_vjp', ws.handle, spec, sim['pmid'], disp, n, conf.ptcl_num, sim['Om'],
              vcot, acc, alpha, dots[k, 3:], st)
    fa = np.ascontiguousarray(sim['fac'][::-1])
    _lib.call('pmx_nbody_adj_steps', ws.handle, spec, sim['pmid'], disp, vel, acc, dcot, vcot,
              alpha, n, conf.ptcl_num, k, fa.ctypes.data_as(ctypes.c_void_p), sim['Om'], dots, st)
    torch.cuda.synchronize()
    return fwd, (disp, vel, acc, dcot, vcot, alpha, dots)


def batch_run(sims, k, cuda, chunks=None, agg=False):
    """The same runs through the batched entry points; ``chunks``: split the
    steps over several calls (as the server issues them)."""
    conf = sims[0]['conf']
    ws = _lib.Workspace(conf.mesh_shape, adjoint=True, slots=len(sims), agg=agg)
    spec = _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)
    st = _lib.stream_ptr(cuda)
    state = []
    for s in sims:
        d = dict(disp=s['disp'].clone(), vel=s['vel'].clone(), acc=torch.empty_like(s['disp']),
                 dcot=s['dcot'].clone(), vcot=s['vcot'].clone(), alpha=torch.zeros_like(s['disp']),
                 dots=torch.zeros((k + 1, 4), dtype=torch.float64, device=cuda),
                 fa=np.ascontiguousarray(s['fac'][::-1]))
        state.append(d)
    chunks = chunks or [k]

    def table(i0, adjoint):
        arr = (_lib.PmxSim * len(sims))()
        keep = []
        for j, (s, d) in enumerate(zip(sims, state)):
            fac = np.ascontiguousarray((d['fa'] if adjoint else s['fac'])[i0:])
            keep.append(fac)
            arr[j] = _lib.PmxSim(s['pmid'].data_ptr(), d['disp'].data_ptr(), d['vel'].data_ptr(),
                                 d['acc'].data_ptr(), d['dcot'].data_ptr(), d['vcot'].data_ptr(),
                                 d['alpha'].data_ptr(), len(s['pmid']), s['conf'].ptcl_num,
                                 s['Om'], fac.ctypes.data, d['dots'][i0].data_ptr())
        return arr, keep

    i0 = 0
    for j, c in enumerate(chunks):
        arr, keep = table(i0, False)
        _lib.call('pmx_nbody_steps_batch', ws.handle, spec, len(sims), arr, int(j == 0), c, st)
        i0 += c
    torch.cuda.synchronize()
    fwd = [(d['disp'].clone(), d['vel'].clone(), d['acc'].clone()) for d in state]
    # the final-time force VJP (its Omega_m term into row k), then the steps
    arr, keep = table(k, True)
    _lib.call('pmx_nbody_adj_steps_batch', ws.handle, spec, len(sims), arr, 1, 0, st)
    i0 = 0
    for c in chunks:
        arr, keep = table(i0, True)
        _lib.call('pmx_nbody_adj_steps_batch', ws.handle, spec, len(sims), arr, 0, c, st)
        i0 += c
    torch.cuda.synchronize()
    adj = [(d['disp'], d['vel'], d['acc'], d['dcot'], d['vcot'], d['alpha'], d['dots'])
           for d in state]
    return fwd, adj


@pytest.mark.parametrize('mesh_side, chunks, agg', [(64, None, False), (64, [2, 3], False),
                                                     (128, [5], False), (64, [4, 1], True)])
def test_batch_equals_single(cuda, mesh_side, chunks, agg):
    """Three simulations of a mesh_side^3 mesh with cell size 1: two particle
    grids (mesh_side/2 at mesh factor 2, mesh_side at factor 1), different
    Omega_m, states and factors; 5 forward then 5 adjoint steps (with agg:
    the batched kernels' warp-aggregated deposits)."""
    k = 5
    h = mesh_side // 2
    sims = [make_sim(cuda, (h,) * 3, 2, 2.0, 1, 0.3, k),
            make_sim(cuda, (mesh_side,) * 3, 1, 1.0, 2, 0.25, k),
            make_sim(cuda, (h,) * 3, 2, 2.0, 3, 0.35, k)]
    bf, ba = batch_run(sims, k, cuda, chunks, agg)
    for s, bfi, bai in zip(sims, bf, ba):
        sf, sa = single_run(s, k, cuda)
        for a, b in zip(bfi, sf):
            assert rel(a, b) < TOL
        for a, b in zip(bai[:3], sa[:3]):     # disp, vel, acc after the reverse steps
            assert rel(a, b) < 1e-4
        for a, b in zip(bai[3:6], sa[3:6]):   # disp_cot, vel_cot, alpha
            assert close_cot(a, b)
        np.testing.assert_allclose(bai[6].cpu().numpy(), sa[6].cpu().numpy(), rtol=3e-3,
                                   atol=1e-5 * float(sa[6].abs().max()))


def test_batch_rejects_bad_calls(cuda):
    conf = pg.Configuration(2.0, (16,) * 3, 2)
    ws = _lib.Workspace(conf.mesh_shape, adjoint=True, slots=2)
    spec = _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)
    arr = (_lib.PmxSim * 3)()
    with pytest.raises(_lib.PmxError, match='slots'):
        _lib.call('pmx_nbody_steps_batch', ws.handle, spec, 3, arr, 1, 1, _lib.stream_ptr(cuda))
    one = _lib.Workspace((48, 32, 32), adjoint=True, slots=2)   # n0 = 48: no fused x pass
    spec48 = _lib.make_spec(3, (48, 32, 32), (48, 32, 32), 1.0)
    with pytest.raises(_lib.PmxError, match='fused'):
        _lib.call('pmx_nbody_steps_batch', one.handle, spec48, 1, arr, 1, 1, _lib.stream_ptr(cuda))
