"""White noise on the GPU (pmx_random_bits / pmx_normal, the reference's
jax.random.normal draw of pmwd/modes.py:33-36) against the oracle, and the
whole pipeline pinned to outputs pmwd itself published for the same seeds.

* bits: bit-exact with the oracle's Threefry restatement, both of JAX's
  counter layouts, even and odd counts, seeds with a nonzero high word;
* normals: the oracle evaluates the same float32 formula with NumPy's
  log1p and emulates the fused multiply-adds in float64, so a value may
  differ by an ulp or two: held to 4 ulp of 1;
* published pins: with pmwd's own white noise, the quickstart notebook's
  printed statistics (docs/examples/quickstart.ipynb cells 14 and 16) and
  the cosmology gradients of the adjoint paper's gradient run
  (docs/papers/adjoint/grads.txt, 64 repeated adjoint runs on an H100) are
  reproduced.
"""

import numpy as np
import pytest
import torch

import pmwd_gb300 as pg
from oracle import cosmo as oc, ics, prng
from pmwd_gb300 import _lib
from pmwd_gb300.modes import PRNG_LAYOUTS, prng_key

pytestmark = pytest.mark.gpu

NAMES = ('A_s_1e9', 'n_s', 'Omega_m', 'Omega_b', 'h')


def _draw(entry, seed, n, layout, cuda):
    k0, k1 = prng_key(seed)
    out = torch.empty(n, dtype=torch.int32 if entry == 'pmx_random_bits' else torch.float32,
                      device=cuda)
    _lib.call(entry, k0, k1, n, PRNG_LAYOUTS[layout], out, _lib.stream_ptr(cuda))
    return out.cpu().numpy()


@pytest.mark.parametrize('layout', ['original', 'partitionable'])
@pytest.mark.parametrize('seed, n', [(0, 1), (0, 10), (1, 7), ((5 << 32) + 9, 1001),
                                     (-3, 1 << 20), (12345, (1 << 20) + 3)])
def test_bits_and_normals_match_oracle(cuda, layout, seed, n):
    bits = _draw('pmx_random_bits', seed, n, layout, cuda).view(np.uint32)
    np.testing.assert_array_equal(bits, prng.random_bits(prng.prng_key(seed), n, layout))
    x = _draw('pmx_normal', seed, n, layout, cuda)
    xo = prng.normal_f32(seed, (n,), layout)
    np.testing.assert_allclose(x, xo, rtol=4 * 2.0 ** -23, atol=4 * 2.0 ** -24)


def test_documented_draws_of_seed_0(cuda):
    """JAX's documented normal(PRNGKey(0), (10,)) in the original layout."""
    want = np.float32([-0.3721109, 0.26423115, -0.18252768, -0.7368197, -0.44030377,
                       -0.1521442, -0.67135346, -0.5908641, 0.73168886, 0.5673026])
    np.testing.assert_allclose(_draw('pmx_normal', 0, 10, 'original', cuda), want, rtol=3e-7)


def test_empty_draw_and_bad_layout(cuda):
    out = torch.empty(1, dtype=torch.float32, device=cuda)
    _lib.call('pmx_normal', 0, 0, 0, 0, out, _lib.stream_ptr(cuda))
    with pytest.raises(_lib.PmxError):
        _lib.call('pmx_normal', 0, 0, 1, 7, out, _lib.stream_ptr(cuda))


def test_white_noise_matches_oracle(cuda):
    """The public white_noise (real and Fourier modes) against the oracle's
    restatement of modes.py:12-49 on a 24 x 20 x 18 particle grid."""
    conf = pg.Configuration(2.0, (24, 20, 18))
    oconf = oc.OConf(2.0, (24, 20, 18), 1, float_dtype=np.float32)
    r = pg.white_noise(3, conf, real=True, device=cuda).cpu().numpy()
    np.testing.assert_allclose(r, ics.white_noise(3, oconf, real=True), rtol=5e-7, atol=3e-7)
    f = pg.white_noise(3, conf, device=cuda).cpu().numpy()
    fo = ics.white_noise(3, oconf)
    assert np.linalg.norm(f - fo) / np.linalg.norm(fo) < 1e-6


def _model(conf):
    def model(modes, cosmo):
        cosmo = pg.boltzmann(cosmo, conf)
        ptcl, obs = pg.lpt(pg.linear_modes(modes, cosmo, conf), cosmo, conf)
        return pg.nbody(ptcl, obs, cosmo, conf)[0]
    return model


def _cosmo_grads(conf, cuda):
    """jax.grad(obj, argnums=(1, 2)) of the reference's gradient examples:
    target density from white_noise(0), real modes from white_noise(1),
    objective var(scatter(nbody(lpt(linear_modes(modes)))) - target)."""
    base = pg.SimpleLCDM(conf)
    model = _model(conf)
    with torch.no_grad():
        tgt = pg.scatter(model(pg.white_noise(0, conf, device=cuda), base), conf)
    modes = pg.white_noise(1, conf, real=True, device=cuda).requires_grad_(True)
    prm = {k: torch.tensor(float(getattr(base, k)), dtype=torch.float64, requires_grad=True)
           for k in NAMES}
    loss = (pg.scatter(model(modes, base.replace(**prm)), conf) - tgt).var(correction=0)
    loss.backward()
    assert torch.isfinite(modes.grad).all()
    return np.array([float(prm[k].grad) for k in NAMES])


def _published():
    import json
    import os
    with open(os.path.join(os.path.dirname(__file__), 'golden', 'published_pmwd.json')) as f:
        return json.load(f)


def test_grads_txt_cosmology_gradients(cuda):
    """The adjoint paper's gradient run (docs/papers/adjoint/grads.py:36-56:
    128^3 particles, 256^3 mesh, spacing 1 Mpc/h, a from 1/16 in 15 steps)
    with pmwd's own white noise.  grads.txt holds the cosmology gradients of
    64 repeated adjoint runs on an H100, which spread by the order of the
    float32 atomic adds: each of our five gradients lies within 4 standard
    deviations of their mean (0.3% at most; the published runs themselves
    range over 0.4%)."""
    pub = _published()['grads_txt']
    runs = np.array(pub['adjoint'])
    mean, std = runs.mean(0), runs.std(0)
    c = pub['config']
    conf = pg.Configuration(c['ptcl_spacing'], tuple(c['ptcl_grid_shape']), c['mesh_shape'],
                            a_start=c['a_start'], a_nbody_maxstep=c['a_nbody_maxstep'])
    assert conf.a_nbody_num == 15
    got = _cosmo_grads(conf, cuda)
    dev = (got - mean) / std
    print('grads.txt run:', dict(zip(NAMES, got.round(3))), 'published mean',
          dict(zip(NAMES, mean.round(3))), 'deviation in sigmas', dev.round(2))
    assert np.all(np.abs(dev) < 4), dev


def test_quickstart_statistics(cuda):
    """The quickstart notebook's printed standard deviations of disp and vel
    after 2LPT (0.105, 0.007) and after 63 N-body steps (5.318, 3.286), for
    white_noise(0) on 256^3 particles / 512^3 mesh: equal to the 3 printed
    decimals (a different realisation of the noise moves the N-body values
    in the second decimal)."""
    pub = _published()['quickstart']
    c = pub['config']
    conf = pg.Configuration(c['ptcl_spacing'], tuple(c['ptcl_grid_shape']), c['mesh_shape'])
    cosmo = pg.boltzmann(pg.Cosmology(conf, **pub['cosmo']), conf)
    with torch.no_grad():
        ptcl, obs = pg.lpt(pg.linear_modes(pg.white_noise(0, conf, device=cuda), cosmo, conf),
                           cosmo, conf)
        s_lpt = [float(ptcl.disp.std(correction=0)), float(ptcl.vel.std(correction=0))]
        ptcl, obs = pg.nbody(ptcl, obs, cosmo, conf)
        s_nb = [float(ptcl.disp.std(correction=0)), float(ptcl.vel.std(correction=0))]
    print('quickstart: 2LPT std', s_lpt, 'N-body std', s_nb)
    half = 0.5 * 10.0 ** -pub['decimals'] + 1e-4
    np.testing.assert_allclose(s_lpt, pub['lpt_disp_vel_std'], rtol=0, atol=half)
    np.testing.assert_allclose(s_nb, pub['nbody_disp_vel_std'], rtol=0, atol=half)
