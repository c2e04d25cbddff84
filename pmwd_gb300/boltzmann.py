"""Background tables in float64 on the host: transfer function, growth
functions, linear power and top-hat variance (pmwd/boltzmann.py:1-455).

* ``transfer_fit``  Eisenstein & Hu (1998) fit, boltzmann.py:32-123.
* ``growth_integ``  the 1st/2nd-order LPT growth ODEs of boltzmann.py:163-229.
  The reference integrates them with its own adaptive Dormand-Prince
  ``odeint`` (ode_util.py) and differentiates through an adjoint ODE; here
  libpmx's host Dormand-Prince 5(4) integrator (``pmx_growth_ode``, the same
  method in C++) integrates all the systems needed at once -- the nominal
  parameters plus +/- perturbations of (Omega_m, Omega_k, w_0, w_a) on a
  shared step sequence -- and the table's parameter Jacobian is the central
  difference of those solutions.  ``GrowthTable`` exposes that Jacobian to
  torch autograd.
* ``growth``, ``linear_power``, ``varlin``, ``boltzmann`` as in the reference.
"""

import ctypes
import math

import numpy as np
import torch

from . import _lib

DT = torch.float64


def interp(x, xp, fp):
    """``jnp.interp`` (linear, clamped at both ends), differentiable in fp
    and x."""
    x = torch.as_tensor(x, dtype=DT, device=fp.device)
    xp = xp.to(device=fp.device, dtype=DT)
    n = xp.shape[0]
    i = torch.clamp(torch.searchsorted(xp, x.detach().reshape(-1).contiguous(), right=True),
                    1, n - 1)
    i = i.reshape(x.shape)
    df = fp[i] - fp[i - 1]
    dx = xp[i] - xp[i - 1]
    delta = x - xp[i - 1]
    f = torch.where(dx == 0, fp[i], fp[i - 1] + (delta / torch.where(dx == 0, 1, dx)) * df)
    f = torch.where(x < xp[0], fp[0], f)
    f = torch.where(x > xp[-1], fp[-1], f)
    return f


# ---------------------------------------------------------------------------
# transfer function
# ---------------------------------------------------------------------------

def transfer_integ(cosmo, conf):
    """Tabulate the transfer function at conf.transfer_k (boltzmann.py:8-28)."""
    if not conf.transfer_fit:
        raise NotImplementedError('TODO')
    return cosmo.replace(transfer=transfer_fit(conf.transfer_k, cosmo, conf))


def transfer_fit(k, cosmo, conf):
    """Eisenstein & Hu fit of the matter transfer function (boltzmann.py:32-123)."""
    k = torch.as_tensor(k, dtype=DT)
    k = k * cosmo.h / conf.L * conf.Mpc_SI
    T2n = (conf.T_cmb / 2.7) ** 2
    h2 = cosmo.h ** 2
    w_m = cosmo.Omega_m * h2
    w_b = cosmo.Omega_b * h2
    f_b = cosmo.Omega_b / cosmo.Omega_m
    f_c = cosmo.Omega_c / cosmo.Omega_m
    z_eq = 2.50e4 * w_m / T2n ** 2
    k_eq = 7.46e-2 * w_m / T2n
    b1 = 0.313 * w_m ** -0.419 * (1 + 0.607 * w_m ** 0.674)
    b2 = 0.238 * w_m ** 0.223
    z_d = 1291 * w_m ** 0.251 / (1 + 0.659 * w_m ** 0.828) * (1 + b1 * w_b ** b2)
    R_d = 31.5 * w_b / T2n ** 2 * (1e3 / z_d)
    R_eq = 31.5 * w_b / T2n ** 2 * (1e3 / z_eq)
    s = (2 / (3 * k_eq) * torch.sqrt(6 / R_eq)
         * torch.log((torch.sqrt(1 + R_d) + torch.sqrt(R_eq + R_d)) / (1 + torch.sqrt(R_eq))))
    k_silk = 1.6 * w_b ** 0.52 * w_m ** 0.73 * (1 + (10.4 * w_m) ** -0.95)

    if conf.transfer_fit_nowiggle:
        alpha_gamma = (1 - 0.328 * torch.log(431 * w_m) * f_b
                       + 0.38 * torch.log(22.3 * w_m) * f_b ** 2)
        gamma_eff_ratio = alpha_gamma + (1 - alpha_gamma) / (1 + (0.43 * k * s) ** 4)
        q_eff = k / (13.41 * k_eq * gamma_eff_ratio)
        L0 = torch.log(2 * math.e + 1.8 * q_eff)
        C0 = 14.2 + 731 / (1 + 62.5 * q_eff)
        return L0 / (L0 + C0 * q_eff ** 2)

    a1 = (46.9 * w_m) ** 0.670 * (1 + (32.1 * w_m) ** -0.532)
    a2 = (12.0 * w_m) ** 0.424 * (1 + (45.0 * w_m) ** -0.582)
    alpha_c = a1 ** -f_b * a2 ** -f_b ** 3
    bb1 = 0.944 / (1 + (458 * w_m) ** -0.708)
    bb2 = (0.395 * w_m) ** -0.0266
    beta_c = 1 / (1 + bb1 * (f_c ** bb2 - 1))

    def T0_tilde(k, alpha_c, beta_c):
        q = k / (13.41 * k_eq)
        L = torch.log(math.e + 1.8 * beta_c * q)
        C = 14.2 / alpha_c + 386 / (1 + 69.9 * q ** 1.08)
        return L / (L + C * q ** 2)

    f = 1 / (1 + (k * s / 5.4) ** 4)
    T_c = f * T0_tilde(k, 1, beta_c) + (1 - f) * T0_tilde(k, alpha_c, beta_c)
    y = (1 + z_eq) / (1 + z_d)
    x = torch.sqrt(1 + y)
    G = y * (-6 * x + (2 + 3 * y) * torch.log((x + 1) / (x - 1)))
    alpha_b = 2.07 * k_eq * s * (1 + R_d) ** -0.75 * G
    beta_node = 8.41 * w_m ** 0.435
    beta_b = 0.5 + f_b + (3 - 2 * f_b) * torch.sqrt(1 + (17.2 * w_m) ** 2)
    ks = k * s
    T_b = (T0_tilde(k, 1, 1) / (1 + (ks / 5.2) ** 2)
           + alpha_b * ks ** 3 / (beta_b ** 3 + ks ** 3) * torch.exp(-(k / k_silk) ** 1.4)
           ) * torch.sinc(ks ** 2 / (math.pi * torch.pow(beta_node ** 3 + ks ** 3, 1 / 3)))
    return f_c * T_c + f_b * T_b


def transfer(k, cosmo, conf):
    """Interpolated transfer function (boltzmann.py:126-160)."""
    if cosmo.transfer is None:
        raise ValueError('Transfer table is empty. Call transfer_integ or boltzmann first.')
    if not conf.transfer_fit:
        raise NotImplementedError('TODO')
    k = torch.as_tensor(k)
    tab = cosmo.transfer.to(k.device if k.is_cuda else 'cpu')
    return interp(k.to(DT), conf.transfer_k, tab)


# ---------------------------------------------------------------------------
# growth
# ---------------------------------------------------------------------------

_GROWTH_PARAMS = ('Omega_m', 'Omega_k', 'w_0', 'w_a')


def _growth_tables_np(params, conf, rtol=1e-11, atol=1e-13):
    """Tables (P, 2, 3, num_a) for P parameter rows (Om, Ok, w0, wa)."""
    params = np.asarray(params, dtype=np.float64)
    eps = np.finfo(np.float64).eps
    a_ic = 0.5 * np.cbrt(eps)
    if a_ic >= conf.a_lpt_step:
        a_ic = 0.1 * conf.a_lpt_step
    a = conf.growth_a.numpy().copy()
    a[0] = a_ic
    lna = np.log(a)
    P = params.shape[0]
    # Dormand-Prince 5(4) in libpmx (host code): y and dy/dlna at every lna
    Y = np.empty((len(lna), P, 4))                                       # (num_a, P, 4)
    Yd = np.empty((len(lna), P, 4))
    prm = np.ascontiguousarray(params)
    lna = np.ascontiguousarray(lna)
    f = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    _lib.check(_lib.load().pmx_growth_ode(f(prm), P, f(lna), len(lna), rtol, atol, f(Y), f(Yd)),
               'pmx_growth_ode')
    G = np.stack([Y[..., 0:2], Y[..., 2:4]], axis=2)                      # (num_a, P, 2, 2)
    Gpp = np.stack([Yd[..., 1], Yd[..., 3]], axis=2)[..., None]          # (num_a, P, 2, 1)
    G = np.concatenate((G, Gpp), axis=3)                                  # (num_a, P, 2, 3)
    G = np.moveaxis(G, 0, 3)                                              # (P, 2, 3, num_a)
    m = np.array([1.0, 2.0])[:, None]
    table = np.stack((G[:, :, 0],
                      m * G[:, :, 0] + G[:, :, 1],
                      m ** 2 * G[:, :, 0] + 2 * m * G[:, :, 1] + G[:, :, 2]), axis=2)
    return table


class GrowthTable(torch.autograd.Function):
    """(Omega_m, Omega_k, w_0, w_a) -> growth table (2, 3, num_a)."""

    @staticmethod
    def forward(ctx, conf, Om, Ok, w0, wa):
        x = np.array([float(Om), float(Ok), float(w0), float(wa)])
        need = any(ctx.needs_input_grad[1:])
        rows = [x]
        hs = []
        if need:
            for i in range(4):
                h = 1e-5 * max(1.0, abs(x[i]))
                hs.append(h)
                for sgn in (1, -1):
                    r = x.copy()
                    r[i] += sgn * h
                    rows.append(r)
        tabs = _growth_tables_np(np.stack(rows), conf)
        if need:
            jac = np.stack([(tabs[1 + 2 * i] - tabs[2 + 2 * i]) / (2 * hs[i]) for i in range(4)])
            ctx.save_for_backward(torch.from_numpy(jac))
        else:
            ctx.save_for_backward(None)
        return torch.from_numpy(tabs[0])

    @staticmethod
    def backward(ctx, g):
        (jac,) = ctx.saved_tensors
        if jac is None:
            return None, None, None, None, None
        grads = (jac * g).reshape(4, -1).sum(1)
        return None, grads[0], grads[1], grads[2], grads[3]


def growth_integ(cosmo, conf):
    """Integrate and tabulate the growth functions at conf.growth_a
    (boltzmann.py:163-229): shape (2 orders, 3 derivatives, num_a)."""
    table = GrowthTable.apply(conf, cosmo.Omega_m, cosmo.Omega_k, cosmo.w_0, cosmo.w_a)
    return cosmo.replace(growth=table)


def growth(a, cosmo, conf, order=1, deriv=0):
    """d^n D_m / dlna^n at scale factors a (boltzmann.py:232-269)."""
    if cosmo.growth is None:
        raise ValueError('Growth table is empty. Call growth_integ or boltzmann first.')
    a = torch.as_tensor(a, dtype=DT)
    tab = cosmo.growth[order - 1][deriv]
    return a ** order * interp(a, conf.growth_a, tab.to(a.device))


# ---------------------------------------------------------------------------
# linear power and variance
# ---------------------------------------------------------------------------

def _safe_power(x, e):
    pos = x > 0
    xs = torch.where(pos, x, torch.ones_like(x))
    return torch.where(pos, xs ** e, torch.zeros_like(x))


def linear_power(k, a, cosmo, conf):
    """Linear matter power spectrum in [L^3] (boltzmann.py:399-455)."""
    if conf.dim != 3:
        raise ValueError(f'dim={conf.dim} not supported')
    k = torch.as_tensor(k).to(DT)
    T = transfer(k, cosmo, conf)
    kp = cosmo.k_pivot.to(k.device)
    Plin = (0.32 * cosmo.A_s.to(k.device) * kp * _safe_power(k / kp, cosmo.n_s.to(k.device))
            * (math.pi * (conf.c / conf.H_0) ** 2 / cosmo.Omega_m.to(k.device) * T) ** 2)
    if a is not None:
        D = growth(torch.as_tensor(a, dtype=DT), cosmo, conf)
        Plin = Plin * D.to(k.device) ** 2
    return Plin


def varlin_integ(cosmo, conf, only=None):
    """Tabulate the linear variance in top-hat spheres at conf.varlin_R
    (boltzmann.py:272-291).  Direct quadrature over ln k replaces mcfit's
    FFTLog transform.

    ``only``: radii at which the table will be read; only the table entries
    that linear interpolation at those radii uses are computed (each entry's
    quadrature is independent of the others), the rest are left at zero."""
    lnk = torch.linspace(math.log(1e-5), math.log(1e3), 8001, dtype=DT)
    k = torch.exp(lnk)
    P = linear_power(k, None, cosmo, conf)
    R = conf.varlin_R
    rows = None
    if only is not None:
        x = torch.as_tensor(only, dtype=DT).reshape(-1)
        i = torch.clamp(torch.searchsorted(R, x, right=True), 1, len(R) - 1)
        rows = torch.unique(torch.cat((i - 1, i)))
        R = R[rows]
    x = k[None, :] * R[:, None]
    W = 3 * (torch.sin(x) - x * torch.cos(x)) / x ** 3
    integrand = k ** 3 * P * W ** 2 / (2 * math.pi ** 2)
    var = torch.trapezoid(integrand, lnk, dim=1)
    if rows is not None:
        full = torch.zeros(len(conf.varlin_R), dtype=var.dtype)
        var = full.index_put((rows,), var)
    return cosmo.replace(varlin=var)


def varlin(R, a, cosmo, conf):
    """Linear variance in top-hat spheres of radius R (boltzmann.py:294-335)."""
    if cosmo.varlin is None:
        raise ValueError('Linear matter overdensity variance table is empty. '
                         'Call varlin_integ or boltzmann first.')
    s2 = interp(torch.as_tensor(R, dtype=DT), conf.varlin_R, cosmo.varlin)
    if a is not None:
        s2 = s2 * growth(a, cosmo, conf) ** 2
    return s2


def boltzmann(cosmo, conf, transfer=True, growth=True, varlin=True):
    """Transfer, growth and variance tables (boltzmann.py:338-374)."""
    cosmo = transfer_integ(cosmo, conf) if transfer else cosmo.replace(transfer=None)
    cosmo = growth_integ(cosmo, conf) if growth else cosmo.replace(growth=None)
    cosmo = varlin_integ(cosmo, conf) if varlin else cosmo.replace(varlin=None)
    return cosmo
