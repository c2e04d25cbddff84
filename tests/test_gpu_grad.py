"""End-to-end gradients of the squared-density objective with respect to the
white-noise modes and the cosmological parameters (Omega_m, A_s), through
boltzmann -> linear_modes -> 2LPT -> nbody (reversible adjoint) -> scatter,
checked against central finite differences (relative step 1e-3), and the
served gradient against the autograd one."""

import numpy as np
import pytest
import torch

import pmwd_gb300 as pg
from pmwd_gb300 import serving

pytestmark = pytest.mark.gpu


def objective(modes, Om, As, conf):
    cosmo = pg.Cosmology(conf, A_s_1e9=As, n_s=0.965, Omega_m=Om, Omega_b=0.05, h=0.7)
    cosmo = pg.boltzmann(cosmo, conf, varlin=False)
    ptcl, _ = pg.lpt(pg.linear_modes(modes, cosmo, conf), cosmo, conf)
    ptcl, _ = pg.nbody(ptcl, None, cosmo, conf)
    dens = pg.scatter(ptcl, conf)
    return (dens - 1).square().sum()


@pytest.fixture(scope='module')
def case(cuda):
    conf = pg.Configuration(4.0, (16, 16, 16), 2, a_nbody_maxstep=(1 - 1 / 64) / 8)
    modes = pg.white_noise(5, conf, real=True, device=cuda)
    return conf, modes


def test_gradients_vs_central_differences(cuda, case):
    conf, modes = case
    m = modes.clone().requires_grad_(True)
    Om = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    As = torch.tensor(2.1, dtype=torch.float64, requires_grad=True)
    obj = objective(m, Om, As, conf)
    obj.backward()
    g_m, g_Om, g_As = m.grad.clone(), float(Om.grad), float(As.grad)

    def f(dm=None, om=0.3, a_s=2.1):
        with torch.no_grad():
            mm = modes if dm is None else modes + dm
            return float(objective(mm, torch.tensor(om, dtype=torch.float64),
                                   torch.tensor(a_s, dtype=torch.float64), conf))

    def central(fn, h):
        """Central difference at step h, Richardson-extrapolated with h/2
        ((4 D(h/2) - D(h)) / 3: the h^2 truncation term cancels)."""
        d1 = (fn(h) - fn(-h)) / (2 * h)
        d2 = (fn(h / 2) - fn(-h / 2)) / h
        return (4 * d2 - d1) / 3, d1

    for val, g, name in ((0.3, g_Om, 'Om'), (2.1, g_As, 'As')):
        h = 1e-3 * val
        if name == 'Om':
            fd, fd1 = central(lambda e: f(om=val + e), h)
        else:
            fd, fd1 = central(lambda e: f(a_s=val + e), h)
        assert abs(g / fd - 1) < 2e-2, (name, g, fd, fd1)

    # directional derivative along a random unit direction of the modes
    u = torch.randn(modes.shape, device=cuda, generator=torch.Generator(device=cuda).manual_seed(1))
    u = u / u.norm()
    h = 1e-3 * float(modes.norm())
    fd, fd1 = central(lambda e: f(e * u), h)
    ad = float((g_m * u).sum())
    assert abs(ad / fd - 1) < 2e-2, (ad, fd, fd1)


def test_served_gradient_equals_autograd(cuda):
    req = serving.Request(0, 16, 2, 8, dict(A_s_1e9=2.1, n_s=0.965, Omega_m=0.3, Omega_b=0.05,
                                            h=0.7), seed=5, grad=True, ptcl_spacing=4.0)
    (res,), _ = serving.run_sequential([req])
    conf = pg.Configuration(4.0, (16, 16, 16), 2, a_nbody_maxstep=(1 - 1 / 64) / 8)
    m = pg.white_noise(5, conf, real=True, device=cuda).requires_grad_(True)
    Om = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    obj = objective(m, Om, torch.tensor(2.1, dtype=torch.float64), conf)
    obj.backward()
    assert abs(res.obj / float(obj.detach()) - 1) < 1e-4
    assert abs(res.grad_rms / float(m.grad.square().mean().sqrt()) - 1) < 1e-3
    # d obj / d Omega_m sums the force sensitivity over every step: the order
    # of the float32 atomic adds moves it by ~1e-3 between runs
    assert abs(res.dobj_dOm / float(Om.grad) - 1) < 5e-3


def test_quickstart_cosmology_gradients_match_published(cuda):
    """The reference quickstart (docs/examples/quickstart.ipynb) on a GPU:
    256^3 particles, 512^3 mesh, spacing 1 Mpc/h, 63 steps; objective
    var(scatter(nbody(lpt(linear_modes(modes)))) - target) with the target
    from seed 0 and real modes from seed 1; pmwd prints the gradient with
    respect to (A_s_1e9, n_s, Omega_m, Omega_b, h) as (51.601, 121.798,
    569.083, -1422.57, 361.472).  white_noise draws pmwd's own modes for
    these seeds (JAX's Threefry normals), so this is one realisation run by
    both.  The reversible adjoint rebuilds 63 steps of a strongly clustered
    run backward, so the order of the float32 atomic adds moves the
    gradients from run to run: five runs gave A_s 51.49-51.60, n_s
    121.57-121.83, Omega_b -1422.6 to -1419.4, h 360.7-361.5 (all within
    0.25% of pmwd's printed values) and Omega_m, which sums the force
    sensitivity over every step, 560.4-568.5 (mean 565.1, standard
    deviation 0.55%; pmwd's 569.08 is 1.3 standard deviations above; a
    Richardson-extrapolated central difference of the forward model gives
    559).  Held to 0.5%, and 2.5% (4.5 standard deviations) for Omega_m."""
    import pmwd_gb300 as pg
    conf = pg.Configuration(1.0, (256,) * 3, mesh_shape=2)
    base = pg.SimpleLCDM(conf)
    names = ('A_s_1e9', 'n_s', 'Omega_m', 'Omega_b', 'h')
    published = (51.601, 121.798, 569.083, -1422.57, 361.472)

    def model(modes, cosmo):
        cosmo = pg.boltzmann(cosmo, conf)
        ptcl, obs = pg.lpt(pg.linear_modes(modes, cosmo, conf), cosmo, conf)
        return pg.nbody(ptcl, obs, cosmo, conf)[0]

    with torch.no_grad():
        tgt = pg.scatter(model(pg.white_noise(0, conf, device=cuda), base), conf)
    modes = pg.white_noise(1, conf, real=True, device=cuda).requires_grad_(True)
    prm = {k: torch.tensor(float(getattr(base, k)), dtype=torch.float64, requires_grad=True)
           for k in names}
    loss = (pg.scatter(model(modes, base.replace(**prm)), conf) - tgt).var(correction=0)
    loss.backward()
    assert torch.isfinite(modes.grad).all()
    got = {k: float(prm[k].grad) for k in names}
    print('quickstart gradients', got)
    for k, want in zip(names, published):
        tol = 2.5e-2 if k == 'Omega_m' else 5e-3
        assert abs(got[k] / want - 1) < tol, (k, got[k], want)
    del tgt, modes
    torch.cuda.empty_cache()
