"""Host-side float64 logic of pmwd_gb300 against the oracle: configuration
derived fields, background functions, growth tables and their parameter
Jacobian, transfer function, time-step factors and the op schedules."""

import importlib

import numpy as np
import pytest
import torch

from oracle import cosmo as oc, nbody as onb
import pmwd_gb300 as pg

gnb = importlib.import_module('pmwd_gb300.nbody')


@pytest.fixture(scope='module')
def both():
    oconf = oc.OConf(2.0, (16, 16, 16), 2, a_nbody_maxstep=1 / 16)
    gconf = pg.Configuration(2.0, (16, 16, 16), 2, a_nbody_maxstep=1 / 16)
    ocos = oc.with_tables(oc.simple_lcdm(), oconf)
    gcos = pg.boltzmann(pg.SimpleLCDM(gconf), gconf)
    return oconf, gconf, ocos, gcos


def test_configuration_fields(both):
    oconf, gconf, _, _ = both
    assert gconf.mesh_shape == (32, 32, 32)
    assert gconf.cell_size == oconf.cell_size == 1.0
    np.testing.assert_array_equal(gconf.a_nbody.numpy(), oconf.a_nbody)
    np.testing.assert_array_equal(gconf.growth_a.numpy(), oconf.growth_a)
    np.testing.assert_array_equal(gconf.transfer_k.numpy(), oconf.transfer_k)
    assert gconf.a_nbody_num == 16
    assert pg.Configuration(1.0, (8, 8, 8)).a_nbody_num == 63   # the reference's default
    with pytest.raises(ValueError):
        pg.Configuration(1.0, (8, 8, 8), (8, 8, 4))
    with pytest.raises(ValueError):
        pg.Configuration(1.0, (8, 8, 8), 0.5)
    with pytest.raises(ValueError):
        pg.Configuration(1.0, (8, 8, 8), symp_splits=((0, 0.5), (1, 0.4)))


def test_background_and_tables(both):
    oconf, gconf, ocos, gcos = both
    a = torch.linspace(0.01, 1.0, 50, dtype=torch.float64)
    np.testing.assert_allclose(pg.E2(a, gcos).numpy(), oc.E2(a.numpy(), ocos), rtol=1e-14)
    np.testing.assert_allclose(pg.H_deriv(a, gcos).numpy(), oc.H_deriv(a.numpy(), ocos),
                               rtol=1e-12)
    np.testing.assert_allclose(gcos.growth.numpy(), ocos.growth, rtol=2e-8, atol=1e-12)
    np.testing.assert_allclose(gcos.transfer.numpy(), ocos.transfer, rtol=1e-12)
    k = torch.logspace(-3, 1, 40, dtype=torch.float64)
    np.testing.assert_allclose(pg.linear_power(k, 0.5, gcos, gconf).numpy(),
                               oc.linear_power(k.numpy(), 0.5, ocos, oconf), rtol=1e-7)
    np.testing.assert_allclose(float(gcos.sigma8), np.sqrt(oc.sigma2_tophat(8.0, ocos, oconf, 1.0)),
                               rtol=2e-4)


@pytest.mark.parametrize('pars', [dict(Omega_m=0.25, Omega_k=0.05, w_0=-0.9, w_a=0.1),
                                  dict(Omega_m=0.35, Omega_k=-0.03, w_0=-1.1, w_a=-0.2)])
def test_growth_tables_other_backgrounds(pars):
    """The host Dormand-Prince integrator (pmx_growth_ode) against the
    oracle's Radau solution with curvature and evolving dark energy."""
    oconf = oc.OConf(2.0, (16, 16, 16), 2, a_nbody_maxstep=1 / 16)
    gconf = pg.Configuration(2.0, (16, 16, 16), 2, a_nbody_maxstep=1 / 16)
    ocos = oc.simple_lcdm(**pars)
    gcos = pg.SimpleLCDM(gconf).replace(**{(k if k == 'Omega_m' else k + '_'):
                                           torch.tensor(v, dtype=torch.float64)
                                           for k, v in pars.items()})
    gcos = pg.boltzmann(gcos, gconf, transfer=False, varlin=False)
    np.testing.assert_allclose(gcos.growth.numpy(), oc.growth_table(ocos, oconf), rtol=2e-8,
                               atol=1e-12)


def test_growth_ode_rejects_bad_arguments():
    from pmwd_gb300 import _lib
    lib = _lib.load()
    prm = np.array([0.3, 0.0, -1.0, 0.0])
    y = np.empty(8)
    f = lambda x: x.ctypes.data_as(__import__('ctypes').c_void_p)
    down = np.array([0.0, -1.0])
    assert lib.pmx_growth_ode(f(prm), 1, f(down), 2, 1e-10, 1e-12, f(y), f(y)) != 0
    assert lib.pmx_growth_ode(f(prm), 1, f(np.array([-1.0, 0.0])), 2, 0.0, 1e-12, f(y), f(y)) != 0


def test_growth_jacobian_matches_finite_differences(both):
    _, gconf, _, _ = both
    Om = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    cos = pg.SimpleLCDM(gconf).replace(Omega_m=Om)
    cos = pg.boltzmann(cos, gconf, transfer=False, varlin=False)
    w = torch.randn(cos.growth.shape, dtype=torch.float64, generator=torch.Generator().manual_seed(0))
    (cos.growth * w).sum().backward()
    h = 1e-5
    vals = []
    for s in (1, -1):
        c = oc.OConf(2.0, (16, 16, 16), 2, a_nbody_maxstep=1 / 16)
        vals.append((oc.growth_table(oc.simple_lcdm(Omega_m=0.3 + s * h), c) * w.numpy()).sum())
    np.testing.assert_allclose(float(Om.grad), (vals[0] - vals[1]) / (2 * h), rtol=1e-5)


@pytest.mark.parametrize('reverse', [False, True])
def test_factors_and_schedules(both, reverse):
    oconf, gconf, ocos, gcos = both
    log = []
    # the oracle's own op order for the forward run
    st = onb.State(np.zeros((1, 3), np.int16), np.zeros((1, 3), np.float32),
                   np.zeros((1, 3), np.float32), np.zeros((1, 3), np.float32))
    a = oconf.a_nbody[::-1] if reverse else oconf.a_nbody
    for a_prev, a_next in zip(a[:-1], a[1:]):
        onb.kick(a_prev, a_prev, a_prev * 0.5 + a_next * 0.5, st, ocos, oconf, log)
        onb.drift(a_prev * 0.5 + a_next * 0.5, a_prev, a_next, st, ocos, oconf, log)
        onb.kick(a_next, a_prev * 0.5 + a_next * 0.5, a_next, st, ocos, oconf, log)
    ops = gnb.forward_ops(gconf, reverse)
    f = gnb.op_factors(ops, gcos, gconf).detach().numpy()
    np.testing.assert_allclose(f, [x[2] for x in log], rtol=1e-8)
    assert [o[0] for o in ops if o[0] != 'force'] == [x[0] for x in log]


def test_factor_gradient_wrt_cosmology(both):
    """d(kick factor)/d(Omega_m) by autograd through the growth Jacobian vs
    central differences of the oracle's factor."""
    oconf, gconf, _, _ = both
    Om = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    cos = pg.boltzmann(pg.SimpleLCDM(gconf).replace(Omega_m=Om), gconf, transfer=False,
                       varlin=False)
    args = (0.25, 0.25, 0.3)
    K = gnb.kick_factor(*args, cos, gconf)
    K.backward()
    h = 1e-5
    fd = []
    for s in (1, -1):
        c = oc.with_tables(oc.simple_lcdm(Omega_m=0.3 + s * h), oconf)
        fd.append(oc.kick_factor(*args, c, oconf))
    np.testing.assert_allclose(float(Om.grad), (fd[0] - fd[1]) / (2 * h), rtol=1e-5)


@pytest.mark.parametrize('pars', [dict(), dict(Omega_m=0.25, Omega_k_=0.05, w_0_=-0.9, w_a_=0.1)])
def test_host_math_matches_torch_path(pars):
    """The NumPy evaluation used by calls without gradients (amplitude table
    of linear_modes, 2LPT growth factors) against the torch code it mirrors:
    the same float32 factors, and amplitudes within one float32 ulp."""
    import math
    hm = importlib.import_module('pmwd_gb300._hostmath')
    glpt = importlib.import_module('pmwd_gb300.lpt')
    conf = pg.Configuration(2.0, (16, 32, 8), 2)
    cos = pg.SimpleLCDM(conf).replace(**{k: torch.tensor(v, dtype=torch.float64)
                                         for k, v in pars.items()})
    cos = pg.boltzmann(cos, conf)
    np.testing.assert_array_equal(hm.lpt_factors(cos, conf), glpt._growth_factors(cos, conf).numpy())
    m = np.arange(0, 3 * 32 * 32 // 4 + 1)
    k = (2 * math.pi / conf.ptcl_spacing) * np.sqrt(m / 32 ** 2)
    amp_np = hm.mode_amplitude(k, 0.5, cos, conf)
    P = pg.linear_power(torch.from_numpy(k), 0.5, cos, conf).to(torch.float32)
    amp_t = torch.sqrt(P * conf.box_vol).numpy()
    np.testing.assert_allclose(amp_np, amp_t, rtol=2.5e-7, atol=0)
    assert not hm.needs_grad(torch.zeros(2), cos)
    assert hm.needs_grad(torch.zeros(2, requires_grad=True))
    with torch.no_grad():
        assert not hm.needs_grad(torch.zeros(2, requires_grad=True))


def test_growth_ode_einstein_de_sitter_is_exact():
    """Omega_m = 1: D_1 = a and D_2 = -3/7 a^2 exactly, so the integrated
    state (G1, G1', G2, G2') stays (1, 0, 3/7, 0) at every output point."""
    import ctypes
    from pmwd_gb300 import _lib
    lib = _lib.load()
    prm = np.array([1.0, 0.0, -1.0, 0.0])
    lna = np.linspace(np.log(1e-5), 0.0, 40)
    y = np.empty((40, 1, 4))
    dy = np.empty((40, 1, 4))
    f = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    assert lib.pmx_growth_ode(f(prm), 1, f(lna), 40, 1e-11, 1e-13, f(y), f(dy)) == 0
    np.testing.assert_allclose(y[:, 0, :], np.tile([1.0, 0.0, 3 / 7, 0.0], (40, 1)), atol=1e-12)
    np.testing.assert_allclose(dy[:, 0, :], 0.0, atol=1e-12)


def test_from_sigma8_reads_only_the_entries_it_needs():
    """Cosmology.from_sigma8 integrates the variance only at the two table
    radii around 8 Mpc/h; sigma8 interpolates between exactly those, so
    A_s equals the one from the whole table (cosmology.py:95-105)."""
    import pmwd_gb300 as pg
    from pmwd_gb300.boltzmann import boltzmann
    conf = pg.Configuration(2.0, (16,) * 3, 2)
    for s8, om in ((0.8, 0.3), (0.72, 0.21), (0.89, 0.39)):
        fast = pg.Cosmology.from_sigma8(conf, s8, n_s=0.96, Omega_m=om, Omega_b=0.05, h=0.7)
        full = boltzmann(pg.Cosmology(conf, 1, n_s=0.96, Omega_m=om, Omega_b=0.05, h=0.7), conf)
        assert abs(float(fast.A_s_1e9) / float((s8 / full.sigma8) ** 2) - 1) < 1e-12
