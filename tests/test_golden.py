"""The oracle reproduces the committed golden fixtures (tests/golden/*.npz,
written by tests/golden/make_golden.py); the GPU path matches them."""

import os

import numpy as np
import pytest
import torch

from oracle import cosmo as oc, nbody as onb, pm

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')


def load(name):
    return dict(np.load(os.path.join(HERE, name + '.npz')))


@pytest.mark.parametrize('name', ['enmesh_default', 'enmesh_offset', 'enmesh_cell'])
def test_oracle_enmesh_golden(name):
    g = load(name)
    cs = float(g['cell_size'])
    off = g['offset']
    ind, frac, fg = pm.enmesh(g['pmid'], g['disp'], float(g['conf'][1]), tuple(g['wrap']),
                              off, None if cs < 0 else cs, tuple(g['shape']), True)
    np.testing.assert_array_equal(ind, g['ind'])
    np.testing.assert_array_equal(frac, g['frac'])
    np.testing.assert_array_equal(fg, g['frac_grad'])


def test_oracle_pm_golden():
    g = load('pm_12')
    conf = oc.OConf(float(g['conf'][0]), (12, 12, 12), 2, float_dtype=np.float32)
    np.testing.assert_array_equal(pm.scatter(g['pmid'], g['disp'], conf), g['dens'])
    np.testing.assert_array_equal(pm.gather(g['pmid'], g['disp'], conf, g['mesh']), g['gathered'])
    acc, dcot, omc = pm.gravity_vjp(g['pmid'], g['disp'], 0.3, conf, g['cot'])
    np.testing.assert_allclose(acc, g['acc'], rtol=1e-6, atol=1e-7 * np.abs(g['acc']).max())
    np.testing.assert_allclose(dcot, g['acc_vjp_disp'], rtol=1e-5,
                               atol=1e-6 * np.abs(g['acc_vjp_disp']).max())
    np.testing.assert_allclose(omc, g['acc_vjp_Om'], rtol=1e-6)


def test_oracle_nbody_golden():
    g = load('nbody_8')
    conf = oc.OConf(4.0, (8, 8, 8), 2, float_dtype=np.float32, a_nbody_maxstep=1 / 4)
    cos = oc.with_tables(oc.simple_lcdm(), conf)
    np.testing.assert_allclose(cos.growth, g['growth'], rtol=1e-9)
    log = []
    st = onb.nbody(onb.State(g['pmid'], g['disp0'], g['vel0']), cos, conf, log=log)
    np.testing.assert_allclose([f for *_, f in log], g['factors'], rtol=1e-9)
    np.testing.assert_allclose(st.disp, g['disp'], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(st.vel, g['vel'], rtol=1e-5, atol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize('name', ['enmesh_default', 'enmesh_offset', 'enmesh_cell'])
def test_gpu_enmesh_golden(cuda, name):
    from pmwd_gb300 import _lib
    g = load(name)
    n = len(g['pmid'])
    cs = float(g['cell_size'])
    spec = _lib.make_spec(3, tuple(g['wrap']), tuple(g['shape']), float(g['conf'][1]),
                          tuple(g['offset']), None if cs < 0 else cs)
    ind = torch.empty((n, 8, 3), dtype=torch.int32, device=cuda)
    frac = torch.empty((n, 8), dtype=torch.float32, device=cuda)
    fg = torch.empty((n, 8, 3), dtype=torch.float32, device=cuda)
    _lib.call('pmx_enmesh', spec, torch.from_numpy(g['pmid']).to(cuda),
              torch.from_numpy(g['disp']).to(cuda), n, _lib.ptr(ind), _lib.ptr(frac),
              _lib.ptr(fg), _lib.stream_ptr(cuda))
    np.testing.assert_array_equal(ind.cpu().numpy(), g['ind'].astype(np.int32))
    np.testing.assert_array_equal(frac.cpu().numpy(), g['frac'])
    np.testing.assert_array_equal(fg.cpu().numpy(), g['frac_grad'])


@pytest.mark.gpu
def test_gpu_nbody_golden(cuda):
    import pmwd_gb300 as pg
    g = load('nbody_8')
    conf = pg.Configuration(4.0, (8, 8, 8), 2, a_nbody_maxstep=1 / 4)
    cos = pg.boltzmann(pg.SimpleLCDM(conf), conf)
    ptcl = pg.Particles(conf, torch.from_numpy(g['pmid']).to(cuda),
                        torch.from_numpy(g['disp0']).to(cuda), vel=torch.from_numpy(g['vel0']).to(cuda))
    out, _ = pg.nbody(ptcl, None, cos, conf)
    d = out.disp.cpu().numpy()
    assert np.linalg.norm(d - g['disp']) / np.linalg.norm(g['disp']) < 1e-5
    v = out.vel.cpu().numpy()
    assert np.linalg.norm(v - g['vel']) / np.linalg.norm(g['vel']) < 1e-5
