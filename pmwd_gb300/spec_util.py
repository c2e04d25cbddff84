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
    if F.is_cuda and F.dtype == torch.complex64:
        G = None if g is None else fftfwd(torch.as_tensor(g, device=dev), axes=(-3, -2, -1))
        kk, PP, NN = _bin_cuda(F, G, grid_shape, edges, right, bnum, deconv)
        return _finish(kk, PP, NN, edges.to(dev), bcut, cut_zero, spacing, grid_shape, dtype,
                       g is not None)
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
    return _finish(kk, PP, NN, e, bcut, cut_zero, spacing, grid_shape, dtype, g is not None)


def _bin_cuda(F, G, grid_shape, edges, right, bnum, deconv):
    """One pass of the pmx_powspec_bin kernel over the complex64 spectra:
    per-bin sums of k N, P N and N in float64."""
    from . import _lib
    dev = F.device
    nb = math.prod(F.shape[:-3])
    if G is not None:
        G = G.to(torch.complex64)
        if G.shape != F.shape:
            raise ValueError(f'shape mismatch: {G.shape} != {F.shape}')
    # torch's CUDA rfftn returns (..., n0, n1, n2h) stored half-axis major,
    # (..., n2h, n0, n1) contiguous: bin it in place instead of transposing
    zm = (_pow2_grid(grid_shape) and bnum <= 2048
          and not F.is_contiguous() and F.movedim(-1, -3).is_contiguous()
          and (G is None or (G.stride() == F.stride())))
    if zm:
        F = F.movedim(-1, -3)
        G = None if G is None else G.movedim(-1, -3)
    else:
        F = F.contiguous()
        G = None if G is None else G.contiguous()
    kx, ky, kz = (k.reshape(-1).contiguous() for k in
                  fftfreq(grid_shape, None, dtype=torch.float64, device=dev))
    e = edges.to(device=dev, dtype=torch.float64).contiguous()
    psum = torch.zeros(bnum, 2, dtype=torch.float64, device=dev)
    # the per-bin sums of k N and N depend on the grid and bins only: for
    # power-of-two grids they are computed on the first call and reused
    key = (dev, grid_shape, tuple(edges.tolist()), bool(right), bnum)
    cached = _GEOMETRY.get(key) if _pow2_grid(grid_shape) else None
    if cached is None:
        ksum = torch.zeros(bnum, dtype=torch.float64, device=dev)
        nsum = torch.zeros(bnum, dtype=torch.float64, device=dev)
    else:
        ksum = nsum = None
    shape = (_lib.c_i64 * 3)(*grid_shape)
    _lib.call('pmx_powspec_bin_zmajor' if zm else 'pmx_powspec_bin', torch.view_as_real(F),
              None if G is None else torch.view_as_real(G),
              nb, shape, kx, ky, kz, e, len(e), int(right), bnum, float(deconv or 0.0), ksum, psum,
              nsum, _lib.stream_ptr(dev))
    if cached is None:
        if _pow2_grid(grid_shape):
            _GEOMETRY[key] = (ksum, nsum)
    else:
        ksum, nsum = cached[0].clone(), cached[1].clone()
    PP = psum[:, 0] if G is None else torch.complex(psum[:, 0], psum[:, 1])
    return ksum, PP, nsum


_GEOMETRY = {}


def _pow2_grid(grid_shape):
    return all(s > 0 and s & (s - 1) == 0 for s in grid_shape) and max(grid_shape) <= 2048


def _finish(kk, PP, NN, e, bcut, cut_zero, spacing, grid_shape, dtype, cross):
    """Cut to [cut_zero, bcut) and normalise (spec_util.py:141-147)."""
    sl = slice(int(cut_zero), bcut)
    kk, PP, NN, edges = kk[sl], PP[sl], NN[sl], e[:bcut]
    kk = kk.to(dtype) / NN * 2 * math.pi / spacing
    PP = (PP if cross else PP.to(dtype)) / NN * spacing ** 3 / math.prod(grid_shape)
    return kk, PP, NN, edges * 2 * math.pi / spacing
