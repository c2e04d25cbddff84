"""White noise and linear modes (pmwd/modes.py:1-117), torch on the GPU.

White noise is drawn on the GPU by libpmx's ``pmx_normal``, which restates
the draw of the reference, ``jax.random.normal(jax.random.PRNGKey(seed),
shape, float32)`` (modes.py:33-36): Threefry-2x32 bits in JAX's counter
layout, a uniform in [nextafter(-1, 0), 1) and sqrt(2) erfinv(u).  A seed
therefore gives pmwd's own realisation.  JAX changed its default counter
layout in version 0.5 (``jax_threefry_partitionable``); the default here,
``'original'``, is the layout of pmwd's published outputs.
"""

import math
import threading
from collections import OrderedDict

import numpy as np
import torch

from . import _hostmath
from .boltzmann import linear_power
from .pm_util import fftfreq, fftfwd, fftinv


PRNG_LAYOUTS = {'original': 0, 'partitionable': 1}


def prng_key(seed):
    """jax.random.PRNGKey of an int64 seed (64-bit JAX types, as pmwd turns
    on): the uint32 pair (seed >> 32, seed & 0xffffffff)."""
    s = int(np.int64(seed)) & 0xFFFFFFFFFFFFFFFF
    return s >> 32, s & 0xFFFFFFFF


def white_noise(seed, conf, real=False, unit_abs=False, device=None, prng_layout='original'):
    """White noise Fourier or real modes (modes.py:12-49), the reference's
    own draw for the same seed (``prng_layout``: JAX's Threefry counter
    layout, 'original' before JAX 0.5 or 'partitionable' after)."""
    from . import _lib
    dev = device if device is not None else torch.device('cuda', torch.cuda.current_device())
    if prng_layout not in PRNG_LAYOUTS:
        raise ValueError(f'{prng_layout=} not in {tuple(PRNG_LAYOUTS)}')
    k0, k1 = prng_key(seed)
    modes = torch.empty(conf.ptcl_grid_shape, dtype=torch.float32, device=dev)
    with torch.cuda.device(dev):
        _lib.call('pmx_normal', k0, k1, modes.numel(), PRNG_LAYOUTS[prng_layout], modes,
                  _lib.stream_ptr(dev))
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


_MODE_INDEX = OrderedDict()   # (shape, device) -> index; the 4 most recent
_MODE_LOCK = threading.Lock()


def _mode_index(shape, device):
    key = (tuple(shape), str(device))
    with _MODE_LOCK:
        if key in _MODE_INDEX:
            _MODE_INDEX.move_to_end(key)
            return _MODE_INDEX[key]
    val = _mode_index_build(shape, device)
    with _MODE_LOCK:
        _MODE_INDEX[key] = val
        while len(_MODE_INDEX) > 4:
            _MODE_INDEX.popitem(last=False)
    return val


def _mode_index_build(shape, device):
    """For power-of-two grids: the integer m with k^2 = (2 pi / spacing)^2 m / D,
    D = max(n)^2, of every rfft mode, and D.  fftfreq values are i / n_a, so
    k^2 (2 pi / spacing)^-2 = sum_a i_a^2 / n_a^2 = m / D exactly.  None for
    other grids."""
    if not all(n > 1 and n & (n - 1) == 0 for n in shape):
        return None
    D = max(shape) ** 2
    idx = []
    for ax, n in enumerate(shape):
        i = torch.arange(n // 2 + 1 if ax == len(shape) - 1 else n, device=device)
        if ax < len(shape) - 1:
            i = torch.where(i < (n + 1) // 2, i, i - n)
        m = (i * i * (D // (n * n))).to(torch.int32)   # dim D / 4 < 2^31 up to 2^15 per side
        idx.append(m.reshape((1,) * ax + (-1,) + (1,) * (len(shape) - ax - 1)))
    # the largest index, |i_a| = n_a / 2 on every axis, is dim D / 4
    return sum(idx), D, len(shape) * D // 4


def linear_modes(modes, cosmo, conf, a=None, real=False):
    """Linear matter overdensity modes (modes.py:67-117): Fourier modes times
    sqrt(V P_lin(k)); optionally back to real space (dimensionless).

    P_lin depends on |k| only: on power-of-two grids sqrt(V P_lin) is
    evaluated once per distinct k^2 (float64 math, float32 result, as per
    mode) and gathered, instead of evaluating the float64 transfer function
    and power law at every mode."""
    dev = modes.device
    mi = _mode_index(conf.ptcl_grid_shape, dev)
    if mi is not None:
        # the table is small (dim D / 4 + 1 entries): evaluated on the host,
        # where the cosmology's tables and parameters live, then gathered;
        # in NumPy when no gradient is needed
        m, D, mmax = mi
        # NumPy is faster for small tables (no per-op dispatch), torch's
        # threaded CPU ops for large ones (197K entries at 512^3)
        if mmax < (1 << 16) and not _hostmath.needs_grad(modes, cosmo, a):
            kn = (2 * math.pi / conf.ptcl_spacing) * np.sqrt(np.arange(mmax + 1) / D)
            an = None if a is None else float(a)
            tab = torch.from_numpy(_hostmath.mode_amplitude(kn, an, cosmo, conf))
        else:
            mv = torch.arange(mmax + 1, dtype=torch.float64)
            k = (2 * math.pi / conf.ptcl_spacing) * torch.sqrt(mv / D)
            Plin = linear_power(k, a, cosmo, conf).to(torch.float32)
            tab = _SafeSqrt.apply(Plin * conf.box_vol)
        amp = tab.to(dev)[m]
    else:
        kvec = fftfreq(conf.ptcl_grid_shape, conf.ptcl_spacing, dtype=torch.float32, device=dev)
        k = torch.sqrt(sum(kk ** 2 for kk in kvec))
        Plin = linear_power(k, a, cosmo, conf).to(torch.float32)
        amp = _SafeSqrt.apply(Plin * conf.box_vol)
    if not torch.is_complex(modes):
        modes = fftfwd(modes, norm='ortho')
    modes = modes * amp
    if real:
        modes = fftinv(modes, shape=conf.ptcl_grid_shape, norm=conf.ptcl_spacing)
    return modes
