"""N-body time integration and its reversible adjoint (pmwd/nbody.py:1-276).

The host computes every time-step factor in float64 with torch (so autograd
reaches the cosmological parameters through the growth tables), casts them
to float32, and drives the GPU:

* default splits ((0, .5), (1, .5)) -- one fused ``pmx_nbody_step`` per step
  (kick + drift + density deposit, r2c, Fourier kernel, batched c2r,
  3-component gather + kick) and one fused ``pmx_nbody_adj_step`` per
  reverse step;
* any other ``symp_splits`` -- the reference's op sequence of ``integrate``
  / ``integrate_adj`` (nbody.py:121-162) with the single-op kernels.

``nbody`` is a ``torch.autograd.Function`` whose backward is pmwd's
memory-free adjoint: it starts from the final state and integrates backward
in time together with the adjoint equations (nbody.py:251-276); nothing of
the forward trajectory is stored.  Cosmology cotangents arrive as
d(objective)/d(factor) = -dot for every adjoint factor (the reference's
``cosmo_cot -= grad(factor) * dot``) plus the Omega_m term of each force,
and torch autograd chains them through the factor functions.
"""

import ctypes

import numpy as np
import torch

from . import _lib
from .boltzmann import growth
from .cosmology import E2, H_deriv

DEFAULT_SPLITS = ((0, 0.5), (1, 0.5))


def _G_D(a, cosmo, conf):
    """Growth factor of ZA canonical velocity in [H_0] (nbody.py:12-14)."""
    return a ** 2 * torch.sqrt(E2(a, cosmo)) * growth(a, cosmo, conf, deriv=1)


def _G_K(a, cosmo, conf):
    """Growth factor of ZA accelerations in [H_0^2] (nbody.py:17-22)."""
    return a ** 3 * E2(a, cosmo) * (growth(a, cosmo, conf, deriv=2)
                                    + (2 + H_deriv(a, cosmo)) * growth(a, cosmo, conf, deriv=1))


def drift_factor(a_vel, a_prev, a_next, cosmo, conf):
    """Drift time-step factor in [1/H_0] (nbody.py:25-29), float64."""
    a_vel, a_prev, a_next = (torch.as_tensor(x, dtype=torch.float64) for x in (a_vel, a_prev, a_next))
    return (growth(a_next, cosmo, conf) - growth(a_prev, cosmo, conf)) / _G_D(a_vel, cosmo, conf)


def kick_factor(a_acc, a_prev, a_next, cosmo, conf):
    """Kick time-step factor in [1/H_0] (nbody.py:32-36), float64."""
    a_acc, a_prev, a_next = (torch.as_tensor(x, dtype=torch.float64) for x in (a_acc, a_prev, a_next))
    return (_G_D(a_next, cosmo, conf) - _G_D(a_prev, cosmo, conf)) / _G_K(a_acc, cosmo, conf)


# ---------------------------------------------------------------------------
# schedules: the reference's op sequence with its scale-factor arguments
# ---------------------------------------------------------------------------

def forward_ops(conf, reverse=False):
    """[('force', a) | ('drift', a_vel, a_prev, a_next) | ('kick', a_acc,
    a_prev, a_next)] of nbody (nbody.py:193-223, 121-140)."""
    a = conf.a_nbody.tolist()
    if reverse:
        a = a[::-1]
    ops = [('force', a[0])]
    for a_prev, a_next in zip(a[:-1], a[1:]):
        D = K = 0
        a_disp = a_vel = a_acc = a_prev
        for d, k in conf.symp_splits:
            if d != 0:
                D += d
                a_disp_next = a_prev * (1 - D) + a_next * D
                ops.append(('drift', a_vel, a_disp, a_disp_next))
                a_disp = a_disp_next
                ops.append(('force', a_disp))
                a_acc = a_disp
            if k != 0:
                K += k
                a_vel_next = a_prev * (1 - K) + a_next * K
                ops.append(('kick', a_acc, a_vel, a_vel_next))
                a_vel = a_vel_next
    return ops


def adjoint_ops(conf, reverse=False):
    """[('force_adj', a) | ('kick_adj', ...) | ('drift_adj', ...)] of
    nbody_adj (nbody.py:226-260, 143-162)."""
    a = conf.a_nbody.tolist()
    if reverse:
        a = a[::-1]
    ops = [('force_adj', a[-1])]
    for a_prev, a_next in zip(a[:0:-1], a[-2::-1]):
        K = D = 0
        a_disp = a_vel = a_acc = a_prev
        for d, k in reversed(conf.symp_splits):
            if k != 0:
                K += k
                a_vel_next = a_prev * (1 - K) + a_next * K
                ops.append(('kick_adj', a_acc, a_vel, a_vel_next))
                a_vel = a_vel_next
            if d != 0:
                D += d
                a_disp_next = a_prev * (1 - D) + a_next * D
                ops.append(('drift_adj', a_vel, a_disp, a_disp_next))
                a_disp = a_disp_next
                ops.append(('force_adj', a_disp))
                a_acc = a_disp
    return ops


def op_factors(ops, cosmo, conf):
    """float64 factor of every kick/drift op (vectorised), in op order."""
    kick = [o[1:] for o in ops if o[0] in ('kick', 'kick_adj')]
    drift = [o[1:] for o in ops if o[0] in ('drift', 'drift_adj')]
    kf = kick_factor(*torch.tensor(kick, dtype=torch.float64).T, cosmo, conf) if kick else None
    df = drift_factor(*torch.tensor(drift, dtype=torch.float64).T, cosmo, conf) if drift else None
    out, ik, idd = [], 0, 0
    for o in ops:
        if o[0] in ('kick', 'kick_adj'):
            out.append(kf[ik])
            ik += 1
        elif o[0] in ('drift', 'drift_adj'):
            out.append(df[idd])
            idd += 1
    if not out:
        return torch.zeros(0, dtype=torch.float64)
    return torch.stack(out)


def _is_fused(conf):
    fused = tuple(tuple(s) for s in conf.symp_splits) == DEFAULT_SPLITS
    if conf.kahan and not fused:
        raise NotImplementedError('Kahan-compensated updates need the default symp_splits')
    return fused


# ---------------------------------------------------------------------------
# device loops
# ---------------------------------------------------------------------------

def _spec(conf):
    return _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)


def run_forward(pmid, disp, vel, acc, ops, factors32, Om, conf, ws=None):
    """Integrate in place on the GPU following ``ops``."""
    n = pmid.shape[0]
    ws = ws or _lib.workspace(conf.mesh_shape, adjoint=False)
    spec = _spec(conf)
    st = _lib.stream_ptr(disp.device)
    P = lambda t: _lib.ptr(t)
    lib = _lib.load()
    if _is_fused(conf):
        _lib.check(lib.pmx_force(ws.handle, spec, P(pmid), P(disp), n, conf.ptcl_num, Om, P(acc),
                                 st), 'pmx_force')
        f = factors32.reshape(-1, 3)
        if not conf.kahan:
            # all steps in one call: consecutive steps share a particle pass
            fac = np.ascontiguousarray(f, dtype=np.float32)
            _lib.check(lib.pmx_nbody_steps(ws.handle, spec, P(pmid), P(disp), P(vel), P(acc), n,
                                           conf.ptcl_num, f.shape[0],
                                           fac.ctypes.data_as(ctypes.c_void_p), Om, st),
                       'pmx_nbody_steps')
            return
        dcomp, vcomp = torch.zeros_like(disp), torch.zeros_like(vel)
        for i in range(f.shape[0]):
            fac = (_lib.c_f * 3)(*f[i])
            _lib.check(lib.pmx_nbody_step_kahan(ws.handle, spec, P(pmid), P(disp), P(vel),
                                                P(acc), P(dcomp), P(vcomp), n, conf.ptcl_num,
                                                fac, Om, st), 'pmx_nbody_step_kahan')
        return
    j = 0
    for o in ops:
        if o[0] == 'force':
            _lib.check(lib.pmx_force(ws.handle, spec, P(pmid), P(disp), n, conf.ptcl_num, Om,
                                     P(acc), st), 'pmx_force')
        elif o[0] == 'kick':
            _lib.check(lib.pmx_kick(P(vel), P(acc), 3 * n, float(factors32[j]), st), 'pmx_kick')
            j += 1
        else:
            _lib.check(lib.pmx_drift(P(disp), P(vel), 3 * n, float(factors32[j]), st), 'pmx_drift')
            j += 1


def run_adjoint(pmid, disp, vel, acc, disp_cot, vel_cot, acc_cot, ops, factors32, Om, conf,
                ws=None):
    """Reverse integration with the adjoint equations, in place.  Returns
    (dots (n_factor_ops,) = the reference's per-factor dot products,
    om_grad = -sum_kicks Om_force * K) as host float64 tensors."""
    n = pmid.shape[0]
    ws = ws or _lib.workspace(conf.mesh_shape, adjoint=True)
    spec = _spec(conf)
    dev = disp.device
    st = _lib.stream_ptr(dev)
    P = lambda t: _lib.ptr(t)
    lib = _lib.load()
    nfac = len(factors32)
    if _is_fused(conf):
        nsteps = nfac // 3
        dd = torch.zeros((nsteps + 1, 4), dtype=torch.float64, device=dev)
        # force_adj at the final time: acc, alpha and its Omega_m term
        _lib.check(lib.pmx_force_vjp(ws.handle, spec, P(pmid), P(disp), n, conf.ptcl_num, Om,
                                     P(vel_cot), P(acc), P(acc_cot), P(dd[nsteps, 3:]), st),
                   'pmx_force_vjp')
        f = factors32.reshape(-1, 3)
        if not conf.kahan:
            fac = np.ascontiguousarray(f, dtype=np.float32)
            _lib.check(lib.pmx_nbody_adj_steps(ws.handle, spec, P(pmid), P(disp), P(vel), P(acc),
                                               P(disp_cot), P(vel_cot), P(acc_cot), n,
                                               conf.ptcl_num, nsteps,
                                               fac.ctypes.data_as(ctypes.c_void_p), Om, P(dd),
                                               st), 'pmx_nbody_adj_steps')
        else:
            dcomp, vcomp = torch.zeros_like(disp), torch.zeros_like(vel)
            for i in range(nsteps):
                fac = (_lib.c_f * 3)(*f[i])
                _lib.check(lib.pmx_nbody_adj_step_kahan(
                    ws.handle, spec, P(pmid), P(disp), P(vel), P(acc), P(disp_cot), P(vel_cot),
                    P(acc_cot), P(dcomp), P(vcomp), n, conf.ptcl_num, fac, Om, P(dd[i]), st),
                    'pmx_nbody_adj_step_kahan')
        dd = dd.cpu()
        # factor order per step: K1_adj (dot0), D_adj (dot1), K2_adj (dot2)
        dots = dd[:nsteps, :3].reshape(-1)
        om_force = torch.cat((dd[nsteps:, 3], dd[:nsteps, 3]))  # force before K1 of step i, then K2
        f64 = torch.tensor(factors32.reshape(-1, 3), dtype=torch.float64)
        om_grad = -(om_force[:nsteps] * f64[:, 0]).sum() - (om_force[1:] * f64[:, 2]).sum()
        return dots, om_grad
    # generic: the reference's op sequence
    dots = torch.zeros(max(nfac, 1), dtype=torch.float64, device=dev)
    om = torch.zeros(len(ops) + 1, dtype=torch.float64, device=dev)
    om_of_kick = []
    j = 0
    last_force = None
    for i, o in enumerate(ops):
        if o[0] == 'force_adj':
            _lib.check(lib.pmx_force_vjp(ws.handle, spec, P(pmid), P(disp), n, conf.ptcl_num, Om,
                                         P(vel_cot), P(acc), P(acc_cot), P(om[i:]), st),
                       'pmx_force_vjp')
            last_force = i
        elif o[0] == 'kick_adj':
            _lib.check(lib.pmx_kick_adj(P(vel), P(acc), P(disp_cot), P(acc_cot), P(vel_cot), 3 * n,
                                        float(factors32[j]), P(dots[j:]), st), 'pmx_kick_adj')
            om_of_kick.append((j, last_force))
            j += 1
        else:
            _lib.check(lib.pmx_drift_adj(P(disp), P(vel), P(vel_cot), P(disp_cot), 3 * n,
                                         float(factors32[j]), P(dots[j:]), st), 'pmx_drift_adj')
            j += 1
    dots = dots.cpu()[:nfac]
    om = om.cpu()
    om_grad = torch.zeros((), dtype=torch.float64)
    for jk, fi in om_of_kick:
        om_grad = om_grad - om[fi] * float(factors32[jk])
    return dots, om_grad


class _NbodyFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, disp, vel, fwd_factors, adj_factors, Om, pmid, conf, reverse):
        disp = disp.contiguous().clone()
        vel = vel.contiguous().clone()
        acc = torch.empty_like(disp)
        ops = forward_ops(conf, reverse)
        f32 = fwd_factors.detach().to(torch.float32).numpy()
        run_forward(pmid, disp, vel, acc, ops, f32, float(Om), conf)
        ctx.save_for_backward(pmid, disp, vel, acc)
        ctx.conf, ctx.reverse = conf, reverse
        ctx.adj32 = adj_factors.detach().to(torch.float32).numpy()
        ctx.Om = float(Om)
        return disp, vel, acc

    @staticmethod
    def backward(ctx, disp_cot, vel_cot, acc_cot):
        pmid, disp, vel, acc = ctx.saved_tensors
        conf = ctx.conf
        disp, vel, acc = disp.clone(), vel.clone(), acc.clone()
        dc = (disp_cot if disp_cot is not None else torch.zeros_like(disp)).contiguous().clone()
        vc = (vel_cot if vel_cot is not None else torch.zeros_like(vel)).contiguous().clone()
        alpha = torch.zeros_like(disp)
        ops = adjoint_ops(conf, ctx.reverse)
        dots, om_grad = run_adjoint(pmid, disp, vel, acc, dc, vc, alpha, ops, ctx.adj32, ctx.Om,
                                    conf)
        return dc, vc, None, -dots, om_grad, None, None, None


def nbody(ptcl, obsvbl, cosmo, conf, reverse=False):
    """N-body time integration (nbody.py:215-223) with pmwd's reversible
    adjoint as its VJP.  Returns (ptcl, obsvbl); ``obsvbl`` passes through
    (the reference's observation hooks are no-ops)."""
    if ptcl.vel is None:
        raise ValueError('nbody needs particle velocities')
    Om = cosmo.Omega_m
    if not torch.is_tensor(Om):
        Om = torch.tensor(float(Om), dtype=torch.float64)
    fwd = op_factors(forward_ops(conf, reverse), cosmo, conf)
    adj = op_factors(adjoint_ops(conf, reverse), cosmo, conf)
    disp, vel, acc = _NbodyFn.apply(ptcl.disp, ptcl.vel, fwd, adj, Om, ptcl.pmid.contiguous(),
                                    conf, reverse)
    return ptcl.replace(disp=disp, vel=vel, acc=acc), obsvbl


def nbody_adj(ptcl, ptcl_cot, obsvbl_cot, cosmo, conf, reverse=False):
    """Explicit reverse integration with the adjoint equations
    (nbody.py:251-260): returns (ptcl at the start, ptcl_cot with pmwd's
    alpha in ``acc``, dL/dfactor per adjoint op, dL/dOmega_m force term)."""
    adj = op_factors(adjoint_ops(conf, reverse), cosmo, conf).detach()
    disp, vel = ptcl.disp.clone(), ptcl.vel.clone()
    acc = ptcl.acc.clone() if ptcl.acc is not None else torch.zeros_like(disp)
    dc, vc = ptcl_cot.disp.clone(), ptcl_cot.vel.clone()
    alpha = torch.zeros_like(disp)
    dots, om_grad = run_adjoint(ptcl.pmid, disp, vel, acc, dc, vc, alpha,
                                adjoint_ops(conf, reverse), adj.to(torch.float32).numpy(),
                                float(cosmo.Omega_m), conf)
    return (ptcl.replace(disp=disp, vel=vel, acc=acc), ptcl_cot.replace(disp=dc, vel=vc, acc=alpha),
            -dots, om_grad)
