"""The published-output fixture (tests/golden/published_pmwd.json) against the
host side of this package: every configuration it records must be the one
pmwd printed it for (step counts, mesh cells per particle, particle mass),
so that the GPU tests that reproduce the printed values run the same
workloads."""

import json
import os

import numpy as np
import pytest

import pmwd_gb300 as pg


def _published():
    with open(os.path.join(os.path.dirname(__file__), 'golden', 'published_pmwd.json')) as f:
        return json.load(f)


def test_grads_txt_runs_and_config():
    pub = _published()['grads_txt']
    assert len(pub['adjoint']) == len(pub['ad']) == 64
    c = pub['config']
    conf = pg.Configuration(c['ptcl_spacing'], tuple(c['ptcl_grid_shape']), c['mesh_shape'],
                            a_start=c['a_start'], a_nbody_maxstep=c['a_nbody_maxstep'])
    assert conf.a_nbody_num == 15
    adj, ad = np.array(pub['adjoint']), np.array(pub['ad'])
    # the two methods agree to the spread of the repeated runs
    assert np.all(np.abs(adj.mean(0) / ad.mean(0) - 1) < 5 * adj.std(0) / np.abs(adj.mean(0)))


def test_quickstart_config():
    pub = _published()['quickstart']
    c = pub['config']
    conf = pg.Configuration(c['ptcl_spacing'], tuple(c['ptcl_grid_shape']), c['mesh_shape'])
    assert conf.a_nbody_num == 63 and conf.mesh_shape == (512, 512, 512)
    assert len(pub['cosmo_grad']) == 5 and pub['decimals'] == 3


@pytest.mark.parametrize('table', ['reproducibility', 'reversibility'])
def test_adjoint_notebook_rows(table):
    rows = _published()['adjoint_notebook'][table]
    assert len(rows) == 8
    seen = set()
    for r in rows:
        conf = pg.Configuration(r['ptcl_spacing'], (384,) * 3, r['mesh_shape'],
                                a_nbody_maxstep=1 / r['a_nbody_maxstep_inv'])
        assert conf.a_nbody_num == r['steps']
        assert r['mesh_shape'] ** 3 == r['cells_per_ptcl']
        cosmo = pg.SimpleLCDM(conf)
        assert round(float(cosmo.ptcl_mass)) == r['ptcl_mass_1e10']
        seen.add((r['ptcl_spacing'], r['mesh_shape'], r['steps']))
        assert 0 < r['disp_rel_diff'] < 1 and 0 < r['vel_rel_diff'] < 1
    assert len(seen) == 8
