"""Generates the golden fixtures in this folder from the CPU oracle.

    python tests/golden/make_golden.py

The reference (JAX) cannot be imported where this repository is built, so
the fixtures are the oracle's outputs on small seeded inputs; they pin the
oracle across NumPy/SciPy versions and machines (the tests recompute them)
and give the GPU tests fixed expected values.  Each case is one .npz file.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import cosmo as oc, ics, nbody as onb, pm  # noqa: E402


def ptcl(conf, std, seed):
    pmid, disp = ics.gen_grid(conf)
    rng = np.random.default_rng(seed)
    disp = (disp + rng.normal(0, std, disp.shape)).astype(conf.float_dtype)
    return pmid, disp


def cases():
    out = {}
    # enmesh: default and float64 branches, with an offset
    conf = oc.OConf(1.5, (6, 5, 4), 2, float_dtype=np.float32)
    pmid, disp = ptcl(conf, 4.0, 1)
    for name, off, cs in (('enmesh_default', 0, None), ('enmesh_offset', (0.3, -1.1, 2.0), None),
                          ('enmesh_cell', 0.25, conf.cell_size / 2)):
        shape = conf.mesh_shape if cs is None else tuple(2 * s for s in conf.mesh_shape)
        ind, frac, fg = pm.enmesh(pmid, disp, conf.cell_size, conf.mesh_shape, off, cs, shape, True)
        out[name] = dict(pmid=pmid, disp=disp, ind=ind, frac=frac, frac_grad=fg,
                         conf=np.array([conf.ptcl_spacing, conf.cell_size]),
                         wrap=np.array(conf.mesh_shape), shape=np.array(shape),
                         offset=np.broadcast_to(np.asarray(off, np.float64), (3,)).copy(),
                         cell_size=np.array(-1.0 if cs is None else cs))
    # scatter / gather / gravity and its VJP on a 12^3 grid, 24^3 mesh
    conf = oc.OConf(2.0, (12, 12, 12), 2, float_dtype=np.float32)
    pmid, disp = ptcl(conf, 2.0, 2)
    rng = np.random.default_rng(3)
    mesh = rng.normal(size=conf.mesh_shape).astype(np.float32)
    cot = rng.normal(size=disp.shape).astype(np.float32)
    acc, dcot, omc = pm.gravity_vjp(pmid, disp, 0.3, conf, cot)
    out['pm_12'] = dict(pmid=pmid, disp=disp, mesh=mesh, cot=cot,
                        dens=pm.scatter(pmid, disp, conf),
                        gathered=pm.gather(pmid, disp, conf, mesh),
                        acc=acc, acc_vjp_disp=dcot, acc_vjp_Om=np.array(omc),
                        conf=np.array([conf.ptcl_spacing, conf.cell_size]))
    # a 4-step leapfrog run (8^3 particles, 16^3 mesh), float32
    conf = oc.OConf(4.0, (8, 8, 8), 2, float_dtype=np.float32, a_nbody_maxstep=1 / 4)
    cos = oc.with_tables(oc.simple_lcdm(), conf)
    pmid, disp = ptcl(conf, 0.5, 4)
    vel = np.random.default_rng(5).normal(0, 0.05, disp.shape).astype(np.float32)
    log = []
    st = onb.nbody(onb.State(pmid, disp, vel), cos, conf, log=log)
    out['nbody_8'] = dict(pmid=pmid, disp0=disp, vel0=vel, disp=st.disp, vel=st.vel, acc=st.acc,
                          factors=np.array([f for *_, f in log]),
                          growth=cos.growth)
    return out


def main():
    for name, arrs in cases().items():
        np.savez_compressed(os.path.join(HERE, name + '.npz'), **arrs)
        print('wrote', name)


if __name__ == '__main__':
    main()
