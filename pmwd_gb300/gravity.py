"""Poisson gravity (pmwd/gravity.py:1-72).

``gravity`` runs the fused CUDA force (``pmx_force``): CIC density,
cuFFT r2c, one Fourier kernel for the Green's function and the three
spectral gradients, batched cuFFT c2r and one 3-component CIC gather.  Its
VJP (``pmx_force_vjp``) recomputes the forward force and applies the exact
transpose of every stage, with no mesh kept between forward and backward.

``laplace`` and ``neg_grad`` are the small Fourier-space helpers the
reference exposes (also used by ``lpt``); they are torch elementwise ops.
"""

import math

import torch

from . import _lib
from .scatter import _check_ptcl


class _LaplaceFn(torch.autograd.Function):
    """-src/k^2 with k = 0 -> 0; self-adjoint VJP avoids NaN gradients
    (gravity.py:9-34)."""

    @staticmethod
    def forward(ctx, src, k2):
        ctx.save_for_backward(k2)
        return _laplace(src, k2)

    @staticmethod
    def backward(ctx, g):
        (k2,) = ctx.saved_tensors
        return _laplace(g, k2), None


def _laplace(src, k2):
    safe = torch.where(k2 != 0, k2, torch.ones_like(k2))
    return torch.where(k2 != 0, -src / safe, torch.zeros((), dtype=src.dtype, device=src.device))


def laplace(kvec, src, cosmo=None):
    """Laplace kernel in Fourier space (gravity.py:9-16)."""
    k2 = sum(k ** 2 for k in kvec)
    return _LaplaceFn.apply(src, k2)


def neg_grad(k, pot, spacing):
    """-i k pot with the Nyquist plane zeroed (gravity.py:37-44)."""
    nyquist = math.pi / spacing
    eps = nyquist * torch.finfo(k.dtype).eps
    k = torch.where(torch.abs(torch.abs(k) - nyquist) <= eps, torch.zeros_like(k), k)
    return (-1j * k) * pot


class _GravityFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, disp, Omega_m, pmid, conf):
        n = pmid.shape[0]
        ws = _lib.workspace(conf.mesh_shape, adjoint=False)
        spec = _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)
        acc = torch.empty_like(disp)
        _lib.call('pmx_force', ws.handle, spec, _lib.ptr(pmid), _lib.ptr(disp), n, conf.ptcl_num,
                  float(Omega_m), _lib.ptr(acc), _lib.stream_ptr(disp.device))
        ctx.save_for_backward(pmid, disp)
        ctx.conf = conf
        ctx.Om = float(Omega_m)
        return acc

    @staticmethod
    def backward(ctx, acc_cot):
        pmid, disp = ctx.saved_tensors
        conf = ctx.conf
        n = pmid.shape[0]
        ws = _lib.workspace(conf.mesh_shape, adjoint=True)
        spec = _lib.make_spec(3, conf.mesh_shape, conf.mesh_shape, conf.cell_size)
        acc = torch.empty_like(disp)
        disp_cot = torch.empty_like(disp)
        om = torch.empty((), dtype=torch.float64, device=disp.device)
        _lib.call('pmx_force_vjp', ws.handle, spec, _lib.ptr(pmid), _lib.ptr(disp), n,
                  conf.ptcl_num, ctx.Om, acc_cot.contiguous(), _lib.ptr(acc),
                  _lib.ptr(disp_cot), _lib.ptr(om), _lib.stream_ptr(disp.device))
        om_cot = om.cpu() if ctx.needs_input_grad[1] else None
        return disp_cot, om_cot, None, None


def gravity(a, ptcl, cosmo, conf):
    """Gravitational accelerations of particles in [H_0^2] (gravity.py:47-72).

    Differentiable in ``ptcl.disp`` and ``cosmo.Omega_m``.
    """
    pmid, disp = ptcl.pmid, ptcl.disp
    _check_ptcl(pmid, disp)
    if conf.dim != 3:
        raise ValueError('the GPU force is 3-D')
    Om = cosmo.Omega_m
    if not torch.is_tensor(Om):
        Om = torch.tensor(float(Om), dtype=torch.float64)
    return _GravityFn.apply(disp.contiguous(), Om, pmid.contiguous(), conf)
