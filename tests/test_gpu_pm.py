"""GPU parity of the mesh operators (libpmx through the C ABI) against the
CPU oracle: bit-exact enmesh indices and fractions, scatter/gather and their
VJPs within float32 tolerances."""

import ctypes

import numpy as np
import pytest
import torch

from oracle import cosmo as oc, ics, pm
import pmwd_gb300 as pg
from pmwd_gb300 import _lib

pytestmark = pytest.mark.gpu

RTOL_MESH = 1e-5      # density-mesh relative L2 of a single scatter (the stated bar)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def T(x, dev, dt=None):
    t = torch.from_numpy(np.ascontiguousarray(x))
    if dt is not None:
        t = t.to(dt)
    return t.to(dev)


def ptcl_case(conf, std, seed=0, edge=False):
    pmid, disp = ics.gen_grid(conf)
    rng = np.random.default_rng(seed)
    disp = (disp + rng.normal(0, std, disp.shape)).astype(np.float32)
    if edge:
        # exact cell boundaries, exact zeros and large displacements
        k = len(disp) // 4
        disp[:k] = np.round(disp[:k] / conf.cell_size) * conf.cell_size
        disp[k:2 * k] = 0.0
        disp[2 * k:2 * k + 8] = np.float32(conf.cell_size) * np.float32(3 * max(conf.mesh_shape))
        disp[2 * k + 8:2 * k + 16] = -np.float32(conf.cell_size) * np.float32(2.5)
    return pmid, disp


def enmesh_gpu(dev, dim, wrap, shape, cell, pmid, disp, offset=0, cell_size=None, drop=True):
    n = len(pmid)
    spec = _lib.make_spec(dim, wrap, shape, cell, offset, cell_size, drop=drop)
    nk = 2 ** dim
    ind = torch.empty((n, nk, dim), dtype=torch.int32, device=dev)
    frac = torch.empty((n, nk), dtype=torch.float32, device=dev)
    fg = torch.empty((n, nk, dim), dtype=torch.float32, device=dev)
    _lib.call('pmx_enmesh', spec, T(pmid, dev), T(disp, dev), n,
              _lib.ptr(ind), _lib.ptr(frac), _lib.ptr(fg), _lib.stream_ptr(dev))
    torch.cuda.synchronize()
    return ind.cpu().numpy(), frac.cpu().numpy(), fg.cpu().numpy()


@pytest.mark.parametrize('ptcl, mesh, spacing', [((8, 8, 8), 2, 1.0), ((6, 10, 4), 1, 2.5),
                                                  ((9, 9, 9), 1.5, 3.0), ((16, 16, 16), 2, 0.25)])
@pytest.mark.parametrize('offset, cell_size', [(0, None), (0.3, None), ((0.1, -2.7, 5.0), None),
                                               (0, 'half'), (0.6, 'ratio')])
def test_enmesh_bit_exact(cuda, ptcl, mesh, spacing, offset, cell_size):
    conf = oc.OConf(spacing, ptcl, mesh, float_dtype=np.float32)
    if cell_size == 'half':
        cell_size = conf.cell_size / 2
    elif cell_size == 'ratio':
        cell_size = conf.cell_size * 0.7
    pmid, disp = ptcl_case(conf, 2.0 * conf.cell_size, edge=True)
    shape = conf.mesh_shape if cell_size is None else tuple(2 * s for s in conf.mesh_shape)
    i_o, f_o, g_o = pm.enmesh(pmid, disp, conf.cell_size, conf.mesh_shape, offset, cell_size,
                              shape, True)
    i_g, f_g, g_g = enmesh_gpu(cuda, 3, conf.mesh_shape, shape, conf.cell_size, pmid, disp,
                               offset, cell_size)
    np.testing.assert_array_equal(i_g, i_o.astype(np.int32))
    np.testing.assert_array_equal(f_g, f_o)
    np.testing.assert_array_equal(g_g, g_o)


@pytest.mark.parametrize('dim', [1, 2])
def test_enmesh_low_dim_bit_exact(cuda, dim):
    conf = oc.OConf(2.0, (12,) * dim, (24,) * dim, float_dtype=np.float32)
    pmid, disp = ptcl_case(conf, 3.0, seed=dim)
    for offset, cs in ((0, None), (0.25, None), (0, 0.5)):
        shape = conf.mesh_shape
        i_o, f_o, g_o = pm.enmesh(pmid, disp, conf.cell_size, conf.mesh_shape, offset, cs, shape,
                                  True)
        i_g, f_g, g_g = enmesh_gpu(cuda, dim, conf.mesh_shape, shape, conf.cell_size, pmid, disp,
                                   offset, cs)
        np.testing.assert_array_equal(i_g, i_o.astype(np.int32))
        np.testing.assert_array_equal(f_g, f_o)
        np.testing.assert_array_equal(g_g, g_o)


@pytest.mark.parametrize('offset, cell_size', [(0, None), (0.3, None), ((0.1, -2.7, 5.0), None),
                                               (0, 'half'), (0.6, 'ratio')])
@pytest.mark.parametrize('drop', [True, False])
def test_enmesh_without_wrapping_bit_exact(cuda, offset, cell_size, drop):
    """particles.py:212-254 with wrap=False (s1 = None, pm_util.py:139-140):
    no periodic wrapping; particles displaced past both edges give negative
    indices (replaced by s2 when drop) and indices >= s2."""
    conf = oc.OConf(2.0, (8, 6, 10), 2, float_dtype=np.float32)
    if cell_size == 'half':
        cell_size = conf.cell_size / 2
    elif cell_size == 'ratio':
        cell_size = conf.cell_size * 0.7
    pmid, disp = ptcl_case(conf, 3.0 * conf.cell_size, edge=True)
    shape = conf.mesh_shape if cell_size is None else tuple(2 * s for s in conf.mesh_shape)
    i_o, f_o, g_o = pm.enmesh(pmid, disp, conf.cell_size, None, offset, cell_size,
                              shape if drop else None, True)
    assert (i_o < 0).any() != drop and (i_o >= np.array(shape)).any()
    i_g, f_g, g_g = enmesh_gpu(cuda, 3, None, shape, conf.cell_size, pmid, disp, offset,
                               cell_size, drop=drop)
    np.testing.assert_array_equal(i_g, i_o.astype(np.int32))
    np.testing.assert_array_equal(f_g, f_o)
    np.testing.assert_array_equal(g_g, g_o)


def test_ptcl_enmesh_wrap_false(cuda):
    """The public ptcl_enmesh with wrap=False (and drop) against the oracle."""
    conf = oc.OConf(1.0, (8, 8, 8), 1, float_dtype=np.float32)
    gconf = pg.Configuration(1.0, (8, 8, 8), 1)
    pmid, disp = ptcl_case(conf, 2.0, edge=True)
    ptcl = pg.Particles(gconf, T(pmid, cuda), T(disp, cuda))
    for drop in (True, False):
        ind, frac, fg = pg.ptcl_enmesh(ptcl, gconf, wrap=False, drop=drop, grad=True)
        i_o, f_o, g_o = pm.enmesh(pmid, disp, conf.cell_size, None, 0, None,
                                  conf.mesh_shape if drop else None, True)
        np.testing.assert_array_equal(ind.cpu().numpy(), i_o)
        np.testing.assert_array_equal(frac.cpu().numpy(), f_o)
        np.testing.assert_array_equal(fg.cpu().numpy(), g_o)


def _spec_for(conf, mesh, dim, offset, cell_size):
    return _lib.make_spec(dim, conf.mesh_shape, mesh.shape[:dim], conf.cell_size, offset, cell_size)


@pytest.mark.parametrize('case', ['default', 'chan', 'offset', 'cell', 'small_mesh', 'big'])
def test_scatter_gather_and_vjps(cuda, case):
    dim = 3
    ptcl, mesh_r, std = (16, 16, 16), 2, 1.5
    if case == 'big':
        ptcl, mesh_r, std = (64, 64, 64), 2, 4.0
    conf = oc.OConf(1.0, ptcl, mesh_r, float_dtype=np.float32)
    pmid, disp = ptcl_case(conf, std * conf.cell_size, seed=3)
    n = len(pmid)
    rng = np.random.default_rng(4)
    offset, cell_size, chan = 0, None, ()
    mesh_shape = conf.mesh_shape
    if case == 'chan':
        chan = (2, 3)
    if case == 'offset':
        offset = (0.5, -0.25, 1.75)
    if case == 'cell':
        cell_size = conf.cell_size / 2
        mesh_shape = tuple(2 * s for s in conf.mesh_shape)
    if case == 'small_mesh':
        mesh_shape = tuple(s - 5 for s in conf.mesh_shape)
    C = int(np.prod(chan)) if chan else 1
    val = rng.normal(1.0, 0.3, (n,) + chan).astype(np.float32) if chan else None
    vs = np.float32(conf.mesh_size / conf.ptcl_num)
    mesh0 = rng.normal(size=mesh_shape + chan).astype(np.float32)

    # scatter
    ref = pm.scatter(pmid, disp, conf, mesh=mesh0, val=val if chan else None, offset=offset,
                     cell_size=cell_size)
    out = T(mesh0, cuda)
    spec = _spec_for(conf, mesh0, dim, offset, cell_size)
    dP, dD = T(pmid, cuda), T(disp, cuda)
    dV = T(val, cuda) if chan else None
    _lib.call('pmx_scatter', spec, _lib.ptr(dP), _lib.ptr(dD), n, _lib.ptr(dV), float(vs), C,
              _lib.ptr(out), _lib.stream_ptr(cuda))
    assert rel_l2(out.cpu().numpy() - mesh0, ref - mesh0) < RTOL_MESH

    # scatter VJP
    mcot = rng.normal(size=mesh_shape + chan).astype(np.float32)
    dc_o, _, vc_o = pm.scatter_vjp(pmid, disp, conf, mcot, val=val if chan else None,
                                   offset=offset, cell_size=cell_size)
    dc = torch.empty((n, dim), dtype=torch.float32, device=cuda)
    vc = torch.empty((n, C), dtype=torch.float32, device=cuda)
    _lib.call('pmx_scatter_adj', spec, _lib.ptr(dP), _lib.ptr(dD), n, _lib.ptr(dV), float(vs), C,
              T(mcot, cuda), _lib.ptr(dc), _lib.ptr(vc), _lib.stream_ptr(cuda))
    assert rel_l2(dc.cpu().numpy(), dc_o) < 1e-5
    assert rel_l2(vc.cpu().numpy().reshape(vc_o.shape), vc_o) < 1e-5

    # gather
    gval = rng.normal(size=(n,) + chan).astype(np.float32) if chan else np.float32(0.5)
    g_o = pm.gather(pmid, disp, conf, mesh0, val=gval, offset=offset, cell_size=cell_size)
    out = torch.empty((n, C), dtype=torch.float32, device=cuda)
    gv = T(gval, cuda) if chan else None
    _lib.call('pmx_gather', spec, _lib.ptr(dP), _lib.ptr(dD), n, T(mesh0, cuda), C,
              _lib.ptr(gv), float(gval) if not chan else 0.0, _lib.ptr(out),
              _lib.stream_ptr(cuda))
    assert rel_l2(out.cpu().numpy().reshape(g_o.shape), g_o) < 1e-6

    # gather VJP
    vcot = rng.normal(size=(n,) + chan).astype(np.float32)
    dc_o, mc_o, _ = pm.gather_vjp(pmid, disp, conf, mesh0, vcot, offset=offset,
                                  cell_size=cell_size)
    dc = torch.empty((n, dim), dtype=torch.float32, device=cuda)
    mc = torch.zeros(mesh_shape + chan, dtype=torch.float32, device=cuda)
    _lib.call('pmx_gather_adj', spec, _lib.ptr(dP), _lib.ptr(dD), n, T(mesh0, cuda), C,
              T(vcot, cuda), _lib.ptr(dc), _lib.ptr(mc), _lib.stream_ptr(cuda))
    assert rel_l2(dc.cpu().numpy(), dc_o) < 1e-5
    assert rel_l2(mc.cpu().numpy(), mc_o) < RTOL_MESH


def test_clustered_scatter_gather_force(cuda):
    """Contention case (the C3 stress in miniature): 32^3 particles pulled into
    8 halos of ~0.3-cell radius, up to ~10^3 particles per cell, so the
    deposits' atomics collide.  Scatter, gather VJP (mesh atomics) and the
    fused force path against the oracle."""
    conf = oc.OConf(1.0, (32, 32, 32), 1, float_dtype=np.float32)
    pmid, disp0 = ics.gen_grid(conf)
    rng = np.random.default_rng(7)
    centres = rng.uniform(0, 32, (8, 3))
    which = rng.integers(0, 8, len(pmid))
    target = centres[which] + rng.normal(0, 0.3, (len(pmid), 3))
    disp = (target - pmid.astype(np.float64) * conf.cell_size).astype(np.float32)
    n = len(pmid)
    spec = _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)
    dP, dD = T(pmid, cuda), T(disp, cuda)
    vs = np.float32(conf.mesh_size / conf.ptcl_num)
    ref = pm.scatter(pmid, disp, conf)
    out = torch.zeros(conf.mesh_shape, dtype=torch.float32, device=cuda)
    _lib.call('pmx_scatter', spec, dP, dD, n, None, float(vs), 1, out, _lib.stream_ptr(cuda))
    assert float(ref.max()) / vs > 500       # the contention is real
    assert rel_l2(out.cpu().numpy(), ref) < RTOL_MESH
    mesh0 = rng.normal(size=conf.mesh_shape).astype(np.float32)
    vcot = rng.normal(size=(n,)).astype(np.float32)
    dc_o, mc_o, _ = pm.gather_vjp(pmid, disp, conf, mesh0, vcot)
    dc = torch.empty((n, 3), dtype=torch.float32, device=cuda)
    mc = torch.zeros(conf.mesh_shape, dtype=torch.float32, device=cuda)
    _lib.call('pmx_gather_adj', spec, dP, dD, n, T(mesh0, cuda), 1, T(vcot, cuda), dc, mc,
              _lib.stream_ptr(cuda))
    assert rel_l2(dc.cpu().numpy(), dc_o) < 1e-5
    assert rel_l2(mc.cpu().numpy(), mc_o) < RTOL_MESH
    gconf = pg.Configuration(1.0, (32, 32, 32), 1)
    acc_o = pm.gravity(pmid, disp, 0.3, conf)
    for kw in ({}, {'cufft3d': True}):
        ws = _lib.Workspace(gconf.mesh_shape, adjoint=True, **kw)
        acc = torch.empty((n, 3), dtype=torch.float32, device=cuda)
        _lib.call('pmx_force', ws.handle, spec, dP, dD, n, gconf.ptcl_num, 0.3, acc,
                  _lib.stream_ptr(cuda))
        assert rel_l2(acc.cpu().numpy(), acc_o) < 1e-5


def test_scatter_centered_known_answer(cuda):
    """tests/pm_test.py:43-71 on the GPU: exact 7/8 in every cell."""
    conf = oc.OConf(2.0, (2, 2, 2), (2, 2, 2), float_dtype=np.float32)
    for pos in [(-3., 5., 7.), (3., -5., 7.), (3., 5., -7.)]:
        pmid = np.zeros((7, 3), np.int16)
        disp = np.tile(np.array(pos, np.float32), (7, 1))
        mesh = torch.zeros((2, 2, 2), dtype=torch.float32, device=cuda)
        spec = _lib.make_spec(3, (2, 2, 2), (2, 2, 2), 2.0)
        _lib.call('pmx_scatter', spec, T(pmid, cuda), T(disp, cuda), 7, None,
                  1.0, 1, _lib.ptr(mesh), _lib.stream_ptr(cuda))
        np.testing.assert_array_equal(mesh.cpu().numpy(), np.full((2, 2, 2), 0.875, np.float32))


def test_empty_and_single_particle(cuda):
    spec = _lib.make_spec(3, (4, 4, 4), (4, 4, 4), 1.0)
    mesh = torch.zeros((4, 4, 4), dtype=torch.float32, device=cuda)
    _lib.call('pmx_scatter', spec, None, None, 0, None, 1.0, 1, _lib.ptr(mesh),
              _lib.stream_ptr(cuda))
    assert float(mesh.abs().sum()) == 0.0
    pmid = torch.zeros((1, 3), dtype=torch.int16, device=cuda)
    disp = torch.full((1, 3), 0.25, dtype=torch.float32, device=cuda)
    _lib.call('pmx_scatter', spec, _lib.ptr(pmid), _lib.ptr(disp), 1, None, 1.0, 1,
              _lib.ptr(mesh), _lib.stream_ptr(cuda))
    np.testing.assert_allclose(float(mesh.sum()), 1.0, rtol=1e-6)
    assert abs(float(mesh[0, 0, 0]) - 0.75 ** 3) < 1e-7
