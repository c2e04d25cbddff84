"""Float64 host arithmetic for calls that need no gradient.

The initial-condition path evaluates a few hundred scalars per call: the
linear power spectrum on the table of distinct |k| (modes.py:67-117 via
boltzmann.py:399-455) and the growth factors at a_start (lpt.py:197-210).
As torch CPU tensors these are ~10^2 dispatched ops (about a millisecond);
when nothing needs a gradient they are evaluated here in NumPy with the
same formulas and the same order of operations as the torch code in
``boltzmann`` and ``cosmology``, so both give the same float32 results.
"""

import math

import numpy as np
import torch


def _f(x):
    return float(x.detach()) if torch.is_tensor(x) else float(x)


def interp(x, xp, fp):
    """boltzmann.interp (``jnp.interp``, clamped) on NumPy float64 arrays."""
    x = np.asarray(x, np.float64)
    n = xp.shape[0]
    i = np.clip(np.searchsorted(xp, x, side='right'), 1, n - 1)
    df = fp[i] - fp[i - 1]
    dx = xp[i] - xp[i - 1]
    delta = x - xp[i - 1]
    f = np.where(dx == 0, fp[i], fp[i - 1] + (delta / np.where(dx == 0, 1, dx)) * df)
    f = np.where(x < xp[0], fp[0], f)
    return np.where(x > xp[-1], fp[-1], f)


def needs_grad(*objs):
    """Whether autograd has to see any tensor of these objects (tensors,
    or dataclasses such as Cosmology holding tensors)."""
    if not torch.is_grad_enabled():
        return False
    for o in objs:
        if torch.is_tensor(o):
            if o.requires_grad:
                return True
        elif hasattr(o, '__dict__'):
            if any(torch.is_tensor(v) and v.requires_grad for v in vars(o).values()):
                return True
    return False


def growth(a, cosmo, conf, order=1, deriv=0, tables=None):
    """boltzmann.growth at a scalar a; tables = (conf.growth_a, cosmo.growth)
    as NumPy arrays when the caller already has them."""
    xp, tab = tables if tables is not None else (conf.growth_a.numpy(),
                                                 cosmo.growth.detach().cpu().numpy())
    return a ** order * float(interp(a, xp, tab[order - 1][deriv]))


def E2(a, cosmo):
    """cosmology.E2 at a scalar a."""
    Om, Ok, w0, wa = (_f(cosmo.Omega_m), _f(cosmo.Omega_k), _f(cosmo.w_0), _f(cosmo.w_a))
    Ode = 1 - (Om + Ok)
    de_a = a ** (-3 * (1 + w0 + wa)) * math.exp(-3 * wa * (1 - a))
    return Om * a ** -3 + Ok * a ** -2 + Ode * de_a


def lpt_factors(cosmo, conf):
    """(lpt_order, 2) float32 array of (D_m, a^2 H dD_m/dlna) at a_start."""
    a = conf.a_start
    tables = (conf.growth_a.numpy(), cosmo.growth.detach().cpu().numpy())
    e2 = E2(a, cosmo)
    rows = []
    for order in range(1, 1 + conf.lpt_order):
        D = growth(a, cosmo, conf, order=order, tables=tables)
        dD_dlna = growth(a, cosmo, conf, order=order, deriv=1, tables=tables)
        rows.append((D, a ** 2 * math.sqrt(e2) * dD_dlna))
    return np.asarray(rows, np.float64).astype(np.float32)


def mode_amplitude(k, a, cosmo, conf):
    """sqrt(V P_lin(k)) in float32 (modes.py:102-112 with
    boltzmann.linear_power) at float64 wavenumbers k."""
    T = interp(k, conf.transfer_k.numpy(), cosmo.transfer.detach().cpu().numpy())
    kp = _f(cosmo.k_pivot)
    x = k / kp
    pos = x > 0
    pw = np.where(pos, np.power(np.where(pos, x, 1.0), _f(cosmo.n_s)), 0.0)
    Plin = (0.32 * _f(cosmo.A_s) * kp * pw
            * (math.pi * (conf.c / conf.H_0) ** 2 / _f(cosmo.Omega_m) * T) ** 2)
    if a is not None:
        Plin = Plin * growth(a, cosmo, conf) ** 2
    P32 = Plin.astype(np.float32)
    return np.sqrt(P32 * np.float32(conf.box_vol))
