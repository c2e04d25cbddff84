"""Float64 torch restatement of pmwd's forward operators, differentiated by
torch autograd (test infrastructure only).

pmwd checks its hand-written VJPs against JAX autodiff of the same forward
code (pmwd/test_util.py:88-149 ``check_custom_vjp``; the gradient study in
docs/papers/adjoint/grads.py compares the adjoint against AD).  This module is
the AD side of that comparison: plain autograd through scatter (scatter.py:60-83),
gather (gather.py:69-77), gravity (gravity.py:47-72) and the leapfrog
(nbody.py:111-140), default enmesh branch only (pm_util.py:119-137).
"""

import math

import numpy as np
import torch

DT = torch.float64


def _enmesh(pmid, disp, cell, wrap_shape):
    """8 neighbours: flat index (N, 8) and differentiable fractions (N, 8)."""
    d = disp / cell
    fl = torch.floor(d.detach())
    idxs, fracs = [], []
    shape = torch.tensor(wrap_shape, dtype=torch.int64)
    for n in range(8):
        nb = torch.tensor([(n >> a) & 1 for a in range(3)], dtype=DT)
        i2 = fl + nb
        d2 = d - i2
        f = 1 - torch.abs(d2)
        i = (i2.to(torch.int64) + pmid.to(torch.int64)) % shape
        flat = (i[:, 0] * wrap_shape[1] + i[:, 1]) * wrap_shape[2] + i[:, 2]
        idxs.append(flat)
        fracs.append(f[:, 0] * f[:, 1] * f[:, 2])
    return torch.stack(idxs, 1), torch.stack(fracs, 1)


def scatter(pmid, disp, mesh_shape, cell, val, mesh=None):
    idx, frac = _enmesh(pmid, disp, cell, mesh_shape)
    size = int(np.prod(mesh_shape))
    out = torch.zeros(size, dtype=DT) if mesh is None else mesh.reshape(-1)
    v = val if torch.is_tensor(val) and val.ndim else torch.as_tensor(val, dtype=DT)
    contrib = (v.reshape(-1, 1) * frac) if v.ndim else v * frac
    out = out.index_add(0, idx.reshape(-1), contrib.reshape(-1))
    return out.reshape(mesh_shape)


def gather(pmid, disp, mesh_shape, cell, mesh):
    idx, frac = _enmesh(pmid, disp, cell, mesh_shape)
    return (mesh.reshape(-1)[idx] * frac).sum(1)


def fftfreq(shape, spacing):
    period = 2 * math.pi / spacing
    ks = [torch.fft.fftfreq(s, dtype=DT) * period for s in shape[:-1]]
    ks.append(torch.fft.rfftfreq(shape[-1], dtype=DT) * period)
    return torch.meshgrid(*ks, indexing='ij')


def gravity(pmid, disp, Omega_m, mesh_shape, cell, ptcl_num):
    """gravity.py:47-72 in float64 autograd."""
    val = float(np.prod(mesh_shape)) / ptcl_num
    dens = scatter(pmid, disp, mesh_shape, cell, val)
    dens = (dens - 1) * (1.5 * Omega_m)
    F = torch.fft.rfftn(dens)
    kvec = fftfreq(mesh_shape, cell)
    k2 = sum(k ** 2 for k in kvec)
    pot = torch.where(k2 != 0, -F / torch.where(k2 != 0, k2, 1), 0)
    acc = []
    nyq = math.pi / cell
    for k in kvec:
        m = torch.where(torch.abs(torch.abs(k) - nyq) <= nyq * 2.2e-16, 0, k)
        g = torch.fft.irfftn(-1j * m * pot, s=mesh_shape)
        acc.append(gather(pmid, disp, mesh_shape, cell, g))
    return torch.stack(acc, -1)
