"""Pins of the CPU oracle: the known answers of the reference's own test file
(tests/pm_test.py), its custom VJPs against float64 autograd (the role of
pmwd/test_util.py:88-149 ``check_custom_vjp``), reversibility, and
background-cosmology limits."""

import numpy as np
import pytest
import torch

from oracle import ad, cosmo as oc, ics, nbody as onb, pm


def _conf(dt=np.float32, ptcl=(4, 6, 8), mesh=2, spacing=4.0, **kw):
    return oc.OConf(spacing, ptcl, mesh, float_dtype=dt, **kw)


@pytest.mark.parametrize('ptcl_num, pos, chan', [
    (3, (-1.,), (2, 1)),
    (5, (1., -3.), (1, 2, 3)),
    (7, (-3., 5., 7.), None),
    (7, (3., -5., 7.), ()),
    (7, (3., 5., -7.), (1,)),
])
@pytest.mark.parametrize('dt', [np.float32, np.float64])
@pytest.mark.parametrize('cell_size', [None, 2.0])
def test_scatter_centered_ptcl(ptcl_num, pos, chan, dt, cell_size):
    """tests/pm_test.py:43-71: particles centred between mesh points spread
    their value uniformly over the 2^dim cells of a periodic 2^dim mesh."""
    dim = len(pos)
    conf = oc.OConf(2.0, (2,) * dim, (2,) * dim, float_dtype=dt)
    pmid = np.zeros((ptcl_num, dim), np.int16)
    disp = np.tile(np.array(pos, dt), (ptcl_num, 1))
    chan = () if chan is None else chan
    val = 1.0 if chan == () else np.ones((ptcl_num,) + chan, dt)
    mesh = np.zeros((2,) * dim + chan, dt)
    out = pm.scatter(pmid, disp, conf, mesh=mesh, val=val, cell_size=cell_size)
    np.testing.assert_array_equal(out, np.full(out.shape, ptcl_num * 2.0 ** -dim, dt))


@pytest.mark.parametrize('ptcl_num, dim, chan', [(3, 1, (2, 1)), (5, 2, (1, 2, 3)), (7, 3, ())])
def test_scatter_sum_gather_uniform(ptcl_num, dim, chan):
    """tests/pm_test.py:86-118: periodic scatter conserves the total; gather
    from a uniform mesh returns the uniform value."""
    rng = np.random.default_rng(0)
    conf = oc.OConf(2.0, (3,) * dim, (3,) * dim, float_dtype=np.float64)
    pmid = np.zeros((ptcl_num, dim), np.int16)
    disp = rng.normal(0, 7.0, (ptcl_num, dim))
    val = np.ones((ptcl_num,) + chan) if chan else 1.0
    out = pm.scatter(pmid, disp, conf, mesh=np.zeros((3,) * dim + chan), val=val)
    np.testing.assert_allclose(out.sum(), ptcl_num * np.prod(chan), rtol=1e-12)
    conf5 = oc.OConf(2.0, (5,) * dim, (5,) * dim, float_dtype=np.float64)
    g = pm.gather(pmid, disp, conf5, np.ones((5,) * dim + chan),
                  val=np.zeros((ptcl_num,) + chan) if chan else 0.0)
    np.testing.assert_allclose(g, 1.0, rtol=1e-14)


def _ptcl(conf, std=3.0, seed=0):
    pmid, disp = ics.gen_grid(conf)
    rng = np.random.default_rng(seed)
    disp = (disp + rng.normal(0, std, disp.shape)).astype(conf.float_dtype)
    return pmid, disp


def test_scatter_gather_vjp_vs_autograd():
    """Custom VJPs (scatter.py:86-148, gather.py:80-142) against autograd."""
    conf = _conf(np.float64)
    pmid, disp = _ptcl(conf)
    rng = np.random.default_rng(1)
    mcot = rng.normal(size=conf.mesh_shape)
    val = conf.mesh_size / conf.ptcl_num
    dcot, _, _ = pm.scatter_vjp(pmid, disp, conf, mcot)
    D = torch.tensor(disp, requires_grad=True)
    m = ad.scatter(torch.tensor(pmid), D, conf.mesh_shape, conf.cell_size, val)
    np.testing.assert_allclose(m.detach().numpy(), pm.scatter(pmid, disp, conf), rtol=1e-12,
                               atol=1e-12)
    (m * torch.tensor(mcot)).sum().backward()
    np.testing.assert_allclose(dcot, D.grad.numpy(), rtol=1e-10, atol=1e-12)

    mesh = rng.normal(size=conf.mesh_shape)
    vcot = rng.normal(size=conf.ptcl_num)
    dcot, mc, _ = pm.gather_vjp(pmid, disp, conf, mesh, vcot)
    D = torch.tensor(disp, requires_grad=True)
    Mt = torch.tensor(mesh, requires_grad=True)
    v = ad.gather(torch.tensor(pmid), D, conf.mesh_shape, conf.cell_size, Mt)
    np.testing.assert_allclose(v.detach().numpy(), pm.gather(pmid, disp, conf, mesh), rtol=1e-12)
    (v * torch.tensor(vcot)).sum().backward()
    np.testing.assert_allclose(dcot, D.grad.numpy(), rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(mc, Mt.grad.numpy(), rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize('ptcl, mesh', [((4, 6, 8), 2), ((7, 8, 5), 1), ((6, 6, 6), 1.5)])
def test_gravity_vjp_vs_autograd(ptcl, mesh):
    """Explicit gravity VJP (the AD of gravity.py:47-72) against autograd,
    even and odd meshes (tests/pm_test.py:154-171 parametrises the same)."""
    conf = _conf(np.float64, ptcl=ptcl, mesh=mesh)
    pmid, disp = _ptcl(conf)
    cot = np.random.default_rng(2).normal(size=disp.shape)
    acc, dcot, Omc = pm.gravity_vjp(pmid, disp, 0.3, conf, cot)
    D = torch.tensor(disp, requires_grad=True)
    Om = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    a = ad.gravity(torch.tensor(pmid), D, Om, conf.mesh_shape, conf.cell_size, conf.ptcl_num)
    np.testing.assert_allclose(acc, a.detach().numpy(), rtol=1e-10, atol=1e-12)
    (a * torch.tensor(cot)).sum().backward()
    np.testing.assert_allclose(dcot, D.grad.numpy(), rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(Omc, Om.grad.item(), rtol=1e-9)


@pytest.fixture(scope='module')
def lcdm_small():
    conf = _conf(np.float64, ptcl=(6, 6, 6), mesh=2, spacing=8.0, a_nbody_maxstep=1 / 4)
    cosmo = oc.with_tables(oc.simple_lcdm(), conf)
    return conf, cosmo


def test_growth_limits(lcdm_small):
    conf, cosmo = lcdm_small
    D1 = float(oc.growth(1.0, cosmo, conf))
    Om, OL = 0.3, 0.7
    cpt = 2.5 * Om / (Om ** (4 / 7) - OL + (1 + Om / 2) * (1 + OL / 70))
    assert abs(D1 / cpt - 1) < 5e-3          # Carroll, Press & Turner (1992) fit
    D2 = float(oc.growth(1.0, cosmo, conf, order=2))
    assert abs(D2 / (3 / 7 * D1 ** 2 * Om ** (-1 / 143)) - 1) < 2e-3  # Bouchet et al. (1995)
    a = 1e-3                                   # matter era: D1 -> a
    assert abs(float(oc.growth(a, cosmo, conf)) / a - 1) < 2e-3


def test_nbody_reversible_f64(lcdm_small):
    """Forward then reverse integration returns to the initial state
    (tests/pm_test.py:177-192; docs/examples/adjoint.ipynb)."""
    conf, cosmo = lcdm_small
    pmid, disp = _ptcl(conf, std=1.0)
    vel = np.random.default_rng(3).normal(0, 0.5, disp.shape)
    st0 = onb.State(pmid, disp, vel)
    st1 = onb.nbody(st0, cosmo, conf)
    st2 = onb.nbody(st1, cosmo, conf, reverse=True)
    np.testing.assert_allclose(st2.disp, disp, rtol=0, atol=1e-10 * np.abs(disp).max())
    np.testing.assert_allclose(st2.vel, vel, rtol=0, atol=1e-10 * np.abs(vel).max())


def _ad_leapfrog(pmid, disp, vel, Om, conf, cosmo, fac_override=None):
    """float64 autograd of nbody's forward (nbody.py:111-140, 193-223)."""
    log = []
    a = conf.a_nbody
    P = torch.tensor(pmid)
    acc = ad.gravity(P, disp, Om, conf.mesh_shape, conf.cell_size, conf.ptcl_num)
    for a_prev, a_next in zip(a[:-1], a[1:]):
        a_mid = a_prev * 0.5 + a_next * 0.5
        K1 = oc.kick_factor(a_prev, a_prev, a_mid, cosmo, conf)
        D = oc.drift_factor(a_mid, a_prev, a_next, cosmo, conf)
        K2 = oc.kick_factor(a_next, a_mid, a_next, cosmo, conf)
        vel = vel + acc * float(K1)
        disp = disp + vel * float(D)
        acc = ad.gravity(P, disp, Om, conf.mesh_shape, conf.cell_size, conf.ptcl_num)
        vel = vel + acc * float(K2)
    return disp, vel


def test_nbody_adjoint_vs_autograd(lcdm_small):
    """nbody_adj (the reversible adjoint, nbody.py:143-162, 226-276) against
    autograd through the stored forward trajectory (grads.py's AD run)."""
    conf, cosmo = lcdm_small
    pmid, disp = _ptcl(conf, std=1.0)
    vel = np.random.default_rng(4).normal(0, 0.3, disp.shape)
    rng = np.random.default_rng(5)
    dcot = rng.normal(size=disp.shape)
    vcot = rng.normal(size=disp.shape)

    st1 = onb.nbody(onb.State(pmid, disp, vel), cosmo, conf)
    st0, cot, sens = onb.nbody_adj(st1, onb.Cot(dcot, vcot), cosmo, conf)

    D = torch.tensor(disp, requires_grad=True)
    V = torch.tensor(vel, requires_grad=True)
    Om = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    d1, v1 = _ad_leapfrog(pmid, D, V, Om, conf, cosmo)
    np.testing.assert_allclose(d1.detach().numpy(), st1.disp, rtol=1e-10, atol=1e-12)
    ((d1 * torch.tensor(dcot)).sum() + (v1 * torch.tensor(vcot)).sum()).backward()
    np.testing.assert_allclose(st0.disp, disp, atol=1e-9)
    np.testing.assert_allclose(cot.disp, D.grad.numpy(), rtol=1e-7, atol=1e-9)
    np.testing.assert_allclose(cot.vel, V.grad.numpy(), rtol=1e-7, atol=1e-9)
    # the direct Omega_m dependence of the forces (factors held fixed)
    np.testing.assert_allclose(sens['Omega_m'], Om.grad.item(), rtol=1e-7)


def test_factor_sensitivities_fd(lcdm_small):
    """dL/d(factor) of the adjoint equals the finite-difference derivative of
    the objective with respect to that factor (one kick and one drift)."""
    conf, cosmo = lcdm_small
    pmid, disp = _ptcl(conf, std=1.0)
    vel = np.random.default_rng(6).normal(0, 0.3, disp.shape)
    rng = np.random.default_rng(7)
    dcot = rng.normal(size=disp.shape)
    vcot = rng.normal(size=disp.shape)
    st1 = onb.nbody(onb.State(pmid, disp, vel), cosmo, conf)
    _, _, sens = onb.nbody_adj(st1, onb.Cot(dcot, vcot), cosmo, conf)
    # adjoint factors are the exact negatives of the forward ones, so
    # dL/dK_fwd = +dot; perturb the first forward drift factor (step 0)
    log = []
    onb.nbody(onb.State(pmid, disp, vel), cosmo, conf, log=log)
    n_adj = len(sens['factors'])
    fwd_drift0 = [i for i, e in enumerate(log) if e[0] == 'drift'][0]
    # adjoint order per step is (kick, drift, kick) over reversed steps; the
    # forward drift of step 0 is the drift of the last adjoint step
    adj_drift_last = [i for i, e in enumerate(sens['factors']) if e[0] == 'drift'][-1]
    assert np.isclose(sens['factors'][adj_drift_last][2], -log[fwd_drift0][2], rtol=1e-15)
    s_adj = sens['factors'][adj_drift_last][3]            # dL/d(adjoint factor)

    def obj(h):
        orig = oc.drift_factor
        calls = {'n': 0}

        def patched(*args):
            v = orig(*args)
            if calls['n'] == 0:
                v = v + h
            calls['n'] += 1
            return v
        onb.oc.drift_factor = patched
        try:
            st = onb.nbody(onb.State(pmid, disp, vel), cosmo, conf)
        finally:
            onb.oc.drift_factor = orig
        return float((st.disp * dcot).sum() + (st.vel * vcot).sum())

    h = 1e-6
    fd = (obj(h) - obj(-h)) / (2 * h)
    # dL/dD_fwd = -dL/dD_adj
    np.testing.assert_allclose(fd, -s_adj, rtol=1e-5)
    assert n_adj == 3 * conf.a_nbody_num
