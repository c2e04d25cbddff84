"""NumPy restatement of pmwd's leapfrog and its reversible adjoint
(test infrastructure only).

* ``drift``/``kick``/``force``           pmwd/nbody.py:39-46, 70-77, 102-105
* ``drift_adj``/``kick_adj``/``force_adj`` pmwd/nbody.py:49-67, 80-99, 108-118
* ``integrate``/``integrate_adj``        pmwd/nbody.py:121-162
* ``nbody``/``nbody_adj``                pmwd/nbody.py:193-276

The cosmology cotangent of the reference is a pytree gradient through the
time-step factors (``value_and_grad(drift_factor/kick_factor)``) plus the
``Omega_m`` dependence of ``gravity``.  Here ``nbody_adj`` returns the
equivalent scalar sensitivities: ``factor_cot[name]`` is dL/d(factor) for each
time-step factor in the order the reference evaluates them, and
``Omega_m_force`` is the direct ``gravity`` term; ``cosmo_grad`` chains them to
parameter gradients by central differences of the factor functions.
"""

from dataclasses import dataclass, replace

import numpy as np

from . import cosmo as oc
from . import pm


@dataclass
class State:
    pmid: np.ndarray
    disp: np.ndarray
    vel: np.ndarray
    acc: np.ndarray = None


def _f(x, conf):
    return np.dtype(conf.float_dtype).type(x)


def force(a, st, cosmo, conf):
    acc = pm.gravity(st.pmid, st.disp, cosmo.Omega_m, conf)
    return replace(st, acc=acc.astype(conf.float_dtype))


def drift(a_vel, a_prev, a_next, st, cosmo, conf, log=None):
    D = oc.drift_factor(a_vel, a_prev, a_next, cosmo, conf)
    if log is not None:
        log.append(('drift', (a_vel, a_prev, a_next), D))
    return replace(st, disp=(st.disp + st.vel * _f(D, conf)).astype(conf.float_dtype))


def kick(a_acc, a_prev, a_next, st, cosmo, conf, log=None):
    K = oc.kick_factor(a_acc, a_prev, a_next, cosmo, conf)
    if log is not None:
        log.append(('kick', (a_acc, a_prev, a_next), K))
    return replace(st, vel=(st.vel + st.acc * _f(K, conf)).astype(conf.float_dtype))


def integrate(a_prev, a_next, st, cosmo, conf, log=None):
    """One symplectic step, nbody.py:121-140."""
    D = K = 0
    a_disp = a_vel = a_acc = a_prev
    for d, k in conf.symp_splits:
        if d != 0:
            D += d
            a_disp_next = a_prev * (1 - D) + a_next * D
            st = drift(a_vel, a_disp, a_disp_next, st, cosmo, conf, log)
            a_disp = a_disp_next
            st = force(a_disp, st, cosmo, conf)
            a_acc = a_disp
        if k != 0:
            K += k
            a_vel_next = a_prev * (1 - K) + a_next * K
            st = kick(a_acc, a_vel, a_vel_next, st, cosmo, conf, log)
            a_vel = a_vel_next
    return st


def nbody(st, cosmo, conf, reverse=False, log=None):
    """nbody.py:215-223."""
    a_nbody = conf.a_nbody[::-1] if reverse else conf.a_nbody
    st = force(a_nbody[0], st, cosmo, conf)
    for a_prev, a_next in zip(a_nbody[:-1], a_nbody[1:]):
        st = integrate(a_prev, a_next, st, cosmo, conf, log)
    return st


# --------------------------------------------------------------------------
# adjoint
# --------------------------------------------------------------------------

@dataclass
class Cot:
    disp: np.ndarray
    vel: np.ndarray
    acc: np.ndarray = None


def force_adj(a, st, cot, cosmo, conf):
    """nbody.py:108-118: forward gravity plus its VJP against vel_cot."""
    acc, disp_cot, Om_cot = pm.gravity_vjp(st.pmid, st.disp, cosmo.Omega_m, conf, cot.vel)
    st = replace(st, acc=acc.astype(conf.float_dtype))
    cot = replace(cot, acc=disp_cot.astype(conf.float_dtype))
    return st, cot, Om_cot


def kick_adj(a_acc, a_prev, a_next, st, cot, cosmo, Om_force, conf, sens):
    """nbody.py:80-99."""
    fdt = conf.float_dtype
    K = oc.kick_factor(a_acc, a_prev, a_next, cosmo, conf)
    Kf = _f(K, conf)
    st = replace(st, vel=(st.vel + st.acc * Kf).astype(fdt))
    cot = replace(cot, disp=(cot.disp - cot.acc * Kf).astype(fdt))
    dot = float(np.sum(cot.vel.astype(np.float64) * st.acc.astype(np.float64)))
    # cosmo_cot -= grad(K) * dot + Om_force * K
    sens['factors'].append(('kick', (a_acc, a_prev, a_next), K, -dot))
    sens['Omega_m'] -= Om_force * float(Kf)
    return st, cot


def drift_adj(a_vel, a_prev, a_next, st, cot, cosmo, conf, sens):
    """nbody.py:49-67."""
    fdt = conf.float_dtype
    D = oc.drift_factor(a_vel, a_prev, a_next, cosmo, conf)
    Df = _f(D, conf)
    st = replace(st, disp=(st.disp + st.vel * Df).astype(fdt))
    cot = replace(cot, vel=(cot.vel - cot.disp * Df).astype(fdt))
    dot = float(np.sum(cot.disp.astype(np.float64) * st.vel.astype(np.float64)))
    sens['factors'].append(('drift', (a_vel, a_prev, a_next), D, -dot))
    return st, cot


def integrate_adj(a_prev, a_next, st, cot, cosmo, Om_force, conf, sens):
    """nbody.py:143-162."""
    K = D = 0
    a_disp = a_vel = a_acc = a_prev
    for d, k in reversed(conf.symp_splits):
        if k != 0:
            K += k
            a_vel_next = a_prev * (1 - K) + a_next * K
            st, cot = kick_adj(a_acc, a_vel, a_vel_next, st, cot, cosmo, Om_force, conf, sens)
            a_vel = a_vel_next
        if d != 0:
            D += d
            a_disp_next = a_prev * (1 - D) + a_next * D
            st, cot = drift_adj(a_vel, a_disp, a_disp_next, st, cot, cosmo, conf, sens)
            a_disp = a_disp_next
            st, cot, Om_force = force_adj(a_disp, st, cot, cosmo, conf)
            a_acc = a_disp
    return st, cot, Om_force


def nbody_adj(st, cot, cosmo, conf, reverse=False):
    """nbody.py:251-260.  ``st`` is the final forward state, ``cot`` carries
    (disp_cot, vel_cot) of the final state.  Returns the reconstructed initial
    state, the cotangents at the start (``cot.acc`` is pmwd's alpha) and the
    sensitivities ``sens``."""
    a_nbody = conf.a_nbody[::-1] if reverse else conf.a_nbody
    sens = {'factors': [], 'Omega_m': 0.0}
    st, cot, Om_force = force_adj(a_nbody[-1], st, cot, cosmo, conf)
    for a_prev, a_next in zip(a_nbody[:0:-1], a_nbody[-2::-1]):
        st, cot, Om_force = integrate_adj(a_prev, a_next, st, cot, cosmo, Om_force, conf, sens)
    return st, cot, sens


def cosmo_grad(sens, cosmo, conf, params=('Omega_m', 'Omega_k', 'w_0', 'w_a'), rel=1e-5):
    """Chain factor sensitivities to parameter gradients by central
    differences of the (re-tabulated) factor functions."""
    out = {}
    for p in params:
        v0 = getattr(cosmo, p)
        h = rel * max(abs(v0), 1.0)
        vals = []
        for sgn in (+1, -1):
            c = replace(cosmo, **{p: v0 + sgn * h})
            c.growth = oc.growth_table(c, conf)
            tot = 0.0
            for kind, args, _, s in sens['factors']:
                fn = oc.kick_factor if kind == 'kick' else oc.drift_factor
                tot += s * float(fn(*args, c, conf))
            vals.append(tot)
        out[p] = (vals[0] - vals[1]) / (2 * h)
    out['Omega_m'] = out.get('Omega_m', 0.0) + sens['Omega_m']
    return out
