"""The reproducibility and reversibility tables pmwd published in
docs/examples/adjoint.ipynb (cells 5 and 11, single precision), rerun with
pmwd's own white noise: 384^3 particles, white_noise(0), SimpleLCDM,
ptcl_spacing 0.5 / 1 Mpc/h, mesh_shape 2 / 1, a_nbody_maxstep 1/64 / 1/128
(63 / 126 steps from a = 1/64 to 1).  Printed values in
tests/golden/published_pmwd.json.

Each row checks
* the configuration: step count, mesh cells per particle, particle mass;
* the standard deviations of disp and vel, of the 2LPT state and after the
  N-body run: equal to the 2 printed significant digits (they follow from
  the seed and the physics; the order of float32 rounding moves them by
  far less than a printed digit);
* reversibility, forward to a = 1 then ``reverse=True`` back: the relative
  differences sigma(s_rev - s_LPT) / sigma(s_LPT) and the same for p are
  float32 rounding amplified by the loss of small-scale information, so
  they depend on the rounding of each operation, not only on the physics.
  pmwd's own two printings of the same table differ by up to 18%.  Held to
  the published value within a factor of 3 either way;
* reproducibility, two forward runs from the same state: their relative
  difference comes from the order of float32 atomic adds in the deposits.
  Held to at most 10 times the published value (bit-identical runs pass).
"""

import json
import os

import pytest
import torch

import pmwd_gb300 as pg

pytestmark = pytest.mark.gpu

FACTOR_REV = 3.0
FACTOR_REPRO = 10.0


def _published():
    with open(os.path.join(os.path.dirname(__file__), 'golden', 'published_pmwd.json')) as f:
        return json.load(f)['adjoint_notebook']


def _rows():
    pub = _published()
    return list(zip(pub['reproducibility'], pub['reversibility']))


def _digits_equal(x, printed, digits=2):
    """x rounds to ``printed`` at ``digits`` significant digits: within half
    a unit of the last printed digit (plus 1e-3 of that unit for the
    printing's own rounding)."""
    import math
    unit = 10.0 ** (math.floor(math.log10(abs(printed))) - (digits - 1))
    return abs(x - printed) <= 0.5 * unit * 1.001


def _rel(a, b, ref):
    return float((a - b).std(correction=0) / ref.std(correction=0))


@pytest.mark.parametrize('repro, rev', _rows(),
                         ids=[f"sp{r['ptcl_spacing']}-m{r['mesh_shape']}-{r['steps']}"
                              for r, _ in _rows()])
def test_adjoint_notebook_tables(cuda, repro, rev):
    assert all(repro[k] == rev[k] for k in ('ptcl_spacing', 'mesh_shape', 'a_nbody_maxstep_inv'))
    conf = pg.Configuration(repro['ptcl_spacing'], (384,) * 3, repro['mesh_shape'],
                            a_nbody_maxstep=1 / repro['a_nbody_maxstep_inv'])
    assert conf.a_nbody_num == repro['steps']
    assert repro['mesh_shape'] ** 3 == repro['cells_per_ptcl']
    cosmo = pg.boltzmann(pg.SimpleLCDM(conf), conf)
    assert round(float(cosmo.ptcl_mass)) == repro['ptcl_mass_1e10']
    with torch.no_grad():
        modes = pg.linear_modes(pg.white_noise(0, conf, device=cuda), cosmo, conf)
        p0, obs = pg.lpt(modes, cosmo, conf)
        p1, obs1 = pg.nbody(p0, obs, cosmo, conf)
        p2, _ = pg.nbody(p0, obs, cosmo, conf)
        pr, _ = pg.nbody(p1, obs1, cosmo, conf, reverse=True)
    got = {
        'lpt_std': (float(p0.disp.std(correction=0)), float(p0.vel.std(correction=0))),
        'nbody_std': (float(p1.disp.std(correction=0)), float(p1.vel.std(correction=0))),
        'repro': (_rel(p1.disp, p2.disp, p1.disp), _rel(p1.vel, p2.vel, p1.vel)),
        'rev': (_rel(pr.disp, p0.disp, p0.disp), _rel(pr.vel, p0.vel, p0.vel)),
    }
    print(f"adjoint.ipynb row {conf.a_nbody_num} steps, spacing {repro['ptcl_spacing']}, mesh "
          f"{repro['mesh_shape']}: 2LPT std {got['lpt_std']} (printed {rev['disp_std']}, "
          f"{rev['vel_std']}); N-body std {got['nbody_std']} (printed {repro['disp_std']}, "
          f"{repro['vel_std']}); reproducibility {got['repro']} (printed "
          f"{repro['disp_rel_diff']}, {repro['vel_rel_diff']}); reversibility {got['rev']} "
          f"(printed {rev['disp_rel_diff']}, {rev['vel_rel_diff']})")
    assert _digits_equal(got['lpt_std'][0], rev['disp_std'])
    assert _digits_equal(got['lpt_std'][1], rev['vel_std'])
    assert _digits_equal(got['nbody_std'][0], repro['disp_std'])
    assert _digits_equal(got['nbody_std'][1], repro['vel_std'])
    for x, want in zip(got['rev'], (rev['disp_rel_diff'], rev['vel_rel_diff'])):
        assert want / FACTOR_REV <= x <= want * FACTOR_REV, (x, want)
    for x, want in zip(got['repro'], (repro['disp_rel_diff'], repro['vel_rel_diff'])):
        assert x <= want * FACTOR_REPRO, (x, want)
