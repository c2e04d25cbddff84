"""FFT helpers of pmwd/pm_util.py:159-344 on torch tensors (cuFFT through
torch.fft on the GPU).  They serve the initial conditions and analysis; the
N-body force calls cuFFT directly from libpmx."""

import math

import numpy as np
import torch


def fftfreq(shape, spacing, dtype=torch.float64, sparse=True, device=None):
    """Angular wavevectors, sparse ij grids (pm_util.py:159-199).  Computed
    in float64 and cast, like the reference."""
    period = 1.0 if spacing is None else 2 * math.pi / spacing
    ks = [np.fft.fftfreq(s) * period for s in shape[:-1]]
    ks.append(np.fft.rfftfreq(shape[-1]) * period)
    ks = [torch.from_numpy(k).to(dtype=dtype, device=device) for k in ks]
    if not sparse:
        return list(torch.meshgrid(*ks, indexing='ij'))
    d = len(ks)
    return [k.reshape((1,) * i + (-1,) + (1,) * (d - i - 1)) for i, k in enumerate(ks)]


def fftfwd(f, shape=None, axes=None, norm=None):
    """rfftn with optional grid-spacing normalisation (pm_util.py:236-289)."""
    if torch.is_complex(f):
        raise ValueError('input field must be real')
    dim = axes if axes is not None else None
    if norm is None or isinstance(norm, str):
        return torch.fft.rfftn(f, s=shape, dim=dim, norm=norm)
    d = f.ndim
    if shape is not None:
        d = len(shape)
    if axes is not None:
        d = len(axes)
    return norm ** d * torch.fft.rfftn(f, s=shape, dim=dim, norm='backward')


def fftinv(f, shape=None, axes=None, norm=None):
    """irfftn with optional grid-spacing normalisation (pm_util.py:292-344)."""
    if not torch.is_complex(f):
        raise ValueError('input field must be Hermitian complex')
    dim = axes if axes is not None else None
    if norm is None or isinstance(norm, str):
        return torch.fft.irfftn(f, s=shape, dim=dim, norm=norm)
    d = f.ndim
    if shape is not None:
        d = len(shape)
    if axes is not None:
        d = len(axes)
    return norm ** -d * torch.fft.irfftn(f, s=shape, dim=dim, norm='backward')


def fft(f, shape=None, axes=None, norm=None):
    """fftfwd for real input, fftinv for complex (pm_util.py:209-233)."""
    if torch.is_complex(f):
        return fftinv(f, shape, axes, norm)
    return fftfwd(f, shape, axes, norm)
