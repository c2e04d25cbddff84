"""Lagrangian perturbation theory initial conditions (pmwd/lpt.py:1-212),
torch on the GPU (cuFFT through torch.fft; autograd gives its VJP)."""

import math
from itertools import combinations, permutations

import torch

from .boltzmann import growth
from .cosmology import E2
from .gravity import laplace, neg_grad
from .particles import Particles
from .pm_util import fftfreq, fftfwd, fftinv


def _strain(kvec, i, j, pot, conf):
    """LPT strain component from a scalar potential (lpt.py:13-37); the
    Nyquist planes are zeroed only when i != j."""
    k_i, k_j = kvec[i], kvec[j]
    nyquist = math.pi / conf.ptcl_spacing
    eps = nyquist * torch.finfo(torch.float32).eps
    if i != j:
        k_i = torch.where(torch.abs(torch.abs(k_i) - nyquist) <= eps, torch.zeros_like(k_i), k_i)
        k_j = torch.where(torch.abs(torch.abs(k_j) - nyquist) <= eps, torch.zeros_like(k_j), k_j)
    strain = -k_i * k_j * pot
    return fftinv(strain, shape=conf.ptcl_grid_shape).to(torch.float32)


def _nyq_zeroed(k, conf):
    nyquist = math.pi / conf.ptcl_spacing
    eps = nyquist * torch.finfo(torch.float32).eps
    return torch.where(torch.abs(torch.abs(k) - nyquist) <= eps, torch.zeros_like(k), k)


def _L3(kvec, pot, conf):
    """2nd-order source of one potential in 3-D (lpt.py:40-76 with m = n):
    the six strain fields come from one batched inverse FFT (each diagonal
    strain once), and the products are summed in the reference's order,
    L = phi_00 phi_22 + phi_00 phi_11 + phi_11 phi_22
        - phi_01^2 - phi_02^2 - phi_12^2."""
    kz = [_nyq_zeroed(k, conf) for k in kvec]
    pairs = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))
    spec = torch.stack([-(kvec[i] if i == j else kz[i]) * (kvec[j] if i == j else kz[j]) * pot
                        for i, j in pairs])
    phi = fftinv(spec, shape=conf.ptcl_grid_shape, axes=(-3, -2, -1)).to(torch.float32)
    L = phi[0] * phi[2]
    L = torch.addcmul(L, phi[0], phi[1])
    L = torch.addcmul(L, phi[1], phi[2])
    for c in (3, 4, 5):
        L = torch.addcmul(L, phi[c], phi[c], value=-1)
    return L


def _L(kvec, pot_m, pot_n, conf):
    """2nd-order source (lpt.py:40-76)."""
    m_eq_n = pot_n is None
    if m_eq_n and conf.dim == 3:
        return _L3(kvec, pot_m, conf)
    if m_eq_n:
        pot_n = pot_m
    L = torch.zeros(conf.ptcl_grid_shape, dtype=torch.float32, device=pot_m.device)
    for i in range(conf.dim):
        strain_m = _strain(kvec, i, i, pot_m, conf)
        for j in range(conf.dim - 1, i, -1):
            L = L + strain_m * _strain(kvec, j, j, pot_n, conf)
        if not m_eq_n:
            for j in range(i - 1, -1, -1):
                L = L + strain_m * _strain(kvec, j, j, pot_n, conf)
    if not m_eq_n:
        L = L * 0.5
    for i in range(conf.dim - 1):
        for j in range(i + 1, conf.dim):
            strain_m = _strain(kvec, i, j, pot_m, conf)
            strain_n = strain_m if m_eq_n else _strain(kvec, j, i, pot_n, conf)
            L = L - strain_m * strain_n
    return L


def levi_civita(indices):
    """Levi-Civita symbol (lpt.py:79-100)."""
    indices = list(indices)
    eps = 1
    for lo, hi in combinations(range(len(indices)), 2):
        d = indices[hi] - indices[lo]
        eps *= (d > 0) - (d < 0)
    return eps


def _M(kvec, pot, conf):
    """3rd-order determinant source (lpt.py:103-116)."""
    M = torch.zeros(conf.ptcl_grid_shape, dtype=torch.float32, device=pot.device)
    for i, j, k in permutations(range(conf.dim), r=3):
        M = M + (levi_civita((i, j, k)) * _strain(kvec, 0, i, pot, conf)
                 * _strain(kvec, 1, j, pot, conf) * _strain(kvec, 2, k, pot, conf))
    return M


def lpt(modes, cosmo, conf):
    """LPT displacements and velocities at conf.a_start (lpt.py:136-212).

    Returns ``(ptcl, None)`` with particles on the Lagrangian grid.
    """
    if conf.dim not in (1, 2, 3):
        raise ValueError(f'dim={conf.dim} not supported')
    if conf.lpt_order not in (0, 1, 2, 3):
        raise ValueError(f'lpt_order={conf.lpt_order} not supported')
    dev = modes.device
    modes = modes / conf.ptcl_cell_vol
    kvec = fftfreq(conf.ptcl_grid_shape, conf.ptcl_spacing, dtype=torch.float32, device=dev)
    pot = []
    if conf.lpt_order > 0:
        pot.append(laplace(kvec, modes, cosmo))
    if conf.lpt_order > 1:
        src_2 = fftfwd(_L(kvec, pot[0], None, conf))
        pot.append(laplace(kvec, src_2, cosmo))
    if conf.lpt_order > 2:
        raise NotImplementedError('TODO')

    a = conf.a_start
    ptcl = Particles.gen_grid(conf, vel=True, device=dev)
    if conf.lpt_order == 0:
        return ptcl, None
    # every displacement field of every order from one batched inverse FFT
    grads = torch.stack([neg_grad(k, pot[o], conf.ptcl_spacing)
                         for o in range(conf.lpt_order) for k in kvec])
    grads = fftinv(grads, shape=conf.ptcl_grid_shape,
                   axes=tuple(range(-conf.dim, 0))).to(torch.float32)
    grads = grads.reshape(conf.lpt_order, conf.dim, -1)
    # columns (dim, n): disp_i += D_m g_mi, vel_i += a^2 H dD_m/dlna g_mi,
    # order by order as the reference accumulates them
    disp, vel = ptcl.disp.t(), ptcl.vel.t()
    for order in range(1, 1 + conf.lpt_order):
        D = growth(a, cosmo, conf, order=order)
        dD_dlna = growth(a, cosmo, conf, order=order, deriv=1)
        a2HDp = a ** 2 * torch.sqrt(E2(a, cosmo)) * dD_dlna
        D = D.to(torch.float32).to(dev)
        a2HDp = a2HDp.to(torch.float32).to(dev)
        g = grads[order - 1]
        disp = disp + D * g
        vel = vel + a2HDp * g
    return ptcl.replace(disp=disp.t().contiguous(), vel=vel.t().contiguous()), None
