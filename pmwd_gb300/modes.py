"""White noise and linear modes (pmwd/modes.py:1-117), torch on the GPU.

White noise is drawn from NumPy's PCG64 generator on the host (float32
standard normals, then uploaded), so a seed gives the same field on every
machine; the reference draws JAX threefry normals instead, so realisations
differ from the reference's while the distribution is the same.
"""

import numpy as np
import torch

from .boltzmann import linear_power
from .pm_util import fftfreq, fftfwd, fftinv


def white_noise(seed, conf, real=False, unit_abs=False, device=None):
    """White noise Fourier or real modes (modes.py:12-49)."""
    dev = device if device is not None else torch.device('cuda', torch.cuda.current_device())
    rng = np.random.default_rng(seed)
    modes = torch.from_numpy(rng.standard_normal(conf.ptcl_grid_shape, dtype=np.float32)).to(dev)
    if real and not unit_abs:
        return modes
    modes = fftfwd(modes, norm='ortho')
    if unit_abs:
        modes = modes / torch.abs(modes)
    if real:
        modes = fftinv(modes, shape=conf.ptcl_grid_shape, norm='ortho')
    return modes


class _SafeSqrt(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        y = torch.sqrt(x)
        ctx.save_for_backward(y)
        return y

    @staticmethod
    def backward(ctx, g):
        (y,) = ctx.saved_tensors
        return torch.where(y != 0, 0.5 / torch.where(y != 0, y, torch.ones_like(y)) * g,
                           torch.zeros_like(g))


def linear_modes(modes, cosmo, conf, a=None, real=False):
    """Linear matter overdensity modes (modes.py:67-117): Fourier modes times
    sqrt(V P_lin(k)); optionally back to real space (dimensionless)."""
    dev = modes.device
    kvec = fftfreq(conf.ptcl_grid_shape, conf.ptcl_spacing, dtype=torch.float32, device=dev)
    k = torch.sqrt(sum(kk ** 2 for kk in kvec))
    Plin = linear_power(k, a, cosmo, conf).to(torch.float32)
    if not torch.is_complex(modes):
        modes = fftfwd(modes, norm='ortho')
    modes = modes * _SafeSqrt.apply(Plin * conf.box_vol)
    if real:
        modes = fftinv(modes, shape=conf.ptcl_grid_shape, norm=conf.ptcl_spacing)
    return modes
