"""Power spectrum estimator (pmwd/spec_util.py:1-147), torch on the GPU."""

import math

import torch

from .pm_util import fftfreq, fftfwd


def _getbins(grid_shape, bins, cut_nyq):
    """Bin edges in units of 2x Nyquist (spec_util.py:10-47)."""
    kfun = 1 / max(grid_shape)
    knyq = 0.5
    kmax = knyq * math.sqrt(3)
    if isinstance(bins, (int, float)):
        w = bins * kfun
        bnum = 1 + math.ceil(kmax / w)
        bcut = 1 + math.ceil(knyq / w) if cut_nyq else bnum
        edges = w * torch.arange(bnum, dtype=torch.float64)
        right = True
    elif isinstance(bins, complex):
        kmaxable = all(s % 2 == 0 for s in grid_shape)
        bnum = 1 + math.ceil(math.log2(kmax / kfun) / bins.imag) + kmaxable
        bcut = 1 + math.ceil(math.log2(knyq / kfun) / bins.imag) if cut_nyq else bnum
        edges = kfun * 2 ** (bins.imag * torch.arange(bnum, dtype=torch.float64))
        right = False
    elif isinstance(bins, tuple):
        if bins[0] != 0:
            raise ValueError(f'{bins=} must starts from 0')
        bnum = len(bins)
        if cut_nyq:
            for bcut, edge in enumerate(bins, start=1):
                if edge >= knyq:
                    break
        else:
            bcut = bnum
        edges = torch.tensor(bins, dtype=torch.float64)
        right = True
    else:
        raise ValueError(f'{bins=} not supported')
    return bnum, bcut, edges, right


def powspec(f, spacing, bins=1j / 3, g=None, deconv=None, cut_zero=True, cut_nyq=True,
            dtype=torch.float64):
    """Auto or cross power spectrum in spherical bins (spec_util.py:50-147).
    Returns (k, P, N, bins)."""
    f = torch.as_tensor(f)
    if g is not None and f.shape != g.shape:
        raise ValueError(f'shape mismatch: {f.shape} != {g.shape}')
    grid_shape = tuple(f.shape[-3:])
    bnum, bcut, edges, right = _getbins(grid_shape, bins, cut_nyq)
    dev = f.device
    F = fftfwd(f, axes=(-3, -2, -1))
    if g is None:
        P = F.real.to(dtype) ** 2 + F.imag.to(dtype) ** 2
    else:
        G = fftfwd(torch.as_tensor(g), axes=(-3, -2, -1))
        P = (F * G.conj()).to(torch.complex128)
    if P.ndim > 3:
        P = P.sum(tuple(range(P.ndim - 3)))
    kvec = fftfreq(grid_shape, None, dtype=torch.float64, device=dev)
    k = torch.sqrt(sum(kk ** 2 for kk in kvec))
    if deconv is not None:
        for kk in kvec:
            P = P * torch.sinc(kk) ** -deconv
    N = torch.full(P.shape, 2.0, dtype=torch.float64, device=dev)
    N[..., 0] = 1
    if grid_shape[-1] % 2 == 0:
        N[..., -1] = 1
    k = torch.broadcast_to(k, P.shape).reshape(-1)
    P = P.reshape(-1)
    N = N.reshape(-1)
    e = edges.to(dev)
    b = torch.bucketize(k, e, right=not right)  # numpy digitize semantics
    keep = b < bnum  # bincount(length=bnum) drops the rest
    b, k, P, N = b[keep], k[keep], P[keep], N[keep]
    kk = torch.zeros(bnum, dtype=dtype, device=dev).index_add_(0, b, (k * N).to(dtype))
    PP = torch.zeros(bnum, dtype=P.dtype, device=dev).index_add_(0, b, P * N.to(P.dtype))
    NN = torch.zeros(bnum, dtype=torch.float64, device=dev).index_add_(0, b, N)
    sl = slice(int(cut_zero), bcut)
    kk, PP, NN, edges = kk[sl], PP[sl], NN[sl], e[:bcut]
    kk = kk / NN * 2 * math.pi / spacing
    PP = PP / NN * spacing ** 3 / math.prod(grid_shape)
    return kk, PP, NN, edges * 2 * math.pi / spacing
