"""NumPy restatement of pmwd's mesh operators (test infrastructure only).

Follows, function by function:

* ``enmesh``            pmwd/pm_util.py:33-156
* ``fftfreq``           pmwd/pm_util.py:159-199
* ``fftfwd``/``fftinv`` pmwd/pm_util.py:236-344
* ``scatter`` + VJP     pmwd/scatter.py:8-150
* ``gather``  + VJP     pmwd/gather.py:8-144
* ``laplace``, ``neg_grad``, ``gravity`` pmwd/gravity.py:9-72

Floating point follows the reference's dtypes (float32 or float64 particle
data, int16 or wider mesh indices).  Scatter-adds accumulate in float64 with
``np.bincount`` and are cast back, which is at least as accurate as the
reference's float32 XLA scatter-add; everything else keeps the reference's
operation order.
"""

import math

import numpy as np
import scipy.fft as sfft

FFT_WORKERS = -1


# ----------------------------------------------------------------------------
# JAX-compatible scalar helpers (jax.numpy semantics the reference relies on)
# ----------------------------------------------------------------------------

def _float_divmod(x1, x2):
    """jnp.divmod for floats: CPython float_divmod, as used by jnp.floor_divide
    and jnp.divmod (the reference calls both in pm_util.py:108,120)."""
    x1 = np.asarray(x1, dtype=np.float64)
    x2 = np.asarray(x2, dtype=np.float64)
    mod = np.fmod(x1, x2)
    div = (x1 - mod) / x2
    ind = (mod != 0) & (np.sign(x2) != np.sign(mod))
    mod = np.where(ind, mod + x2, mod)
    div = np.where(ind, div - 1, div)
    # lax.round rounds half away from zero
    div = np.where(div >= 0, np.floor(div + 0.5), np.ceil(div - 0.5))
    return div, mod


def _float_remainder(x1, x2):
    """jnp.remainder for floats (result takes the divisor's sign)."""
    trunc = np.fmod(x1, x2)
    do_plus = ((trunc < 0) != (x2 < 0)) & (trunc != 0)
    return np.where(do_plus, trunc + x2, trunc)


# ----------------------------------------------------------------------------
# enmesh  (pm_util.py:33-156)
# ----------------------------------------------------------------------------

def enmesh(i1, d1, a1, s1, b12, a2, s2, grad):
    """Multilinear mesh indices and fractions, pm_util.py:33-156.

    Returns ``i2 (num, 2**dim, dim)`` of ``i1.dtype``, ``f2 (num, 2**dim)`` of
    ``d1.dtype`` and, if ``grad``, ``f2g (num, 2**dim, dim)``.
    """
    i1 = np.asarray(i1)
    d1 = np.asarray(d1)
    idt = i1.dtype
    fdt = d1.dtype
    dim = i1.shape[1]
    neighbors = ((np.arange(2**dim, dtype=idt)[:, None]
                  >> np.arange(dim, dtype=idt)) & 1).astype(idt)

    if s1 is not None:
        s1 = np.asarray(s1, dtype=idt)
    if s2 is not None:
        s2 = np.asarray(s2, dtype=idt)
    b12 = np.broadcast_to(np.asarray(b12, dtype=np.float64), (dim,))

    if a2 is not None:                                   # pm_util.py:99-118
        a1 = np.float64(a1)
        a2 = np.float64(a2)
        P = i1.astype(np.float64) * a1 + d1.astype(np.float64) - b12
        P = P[:, None]
        i2 = P + neighbors.astype(np.float64) * a2
        if s1 is not None:
            L = s1.astype(np.float64) * a1
            i2 = _float_remainder(i2, L)
        i2 = _float_divmod(i2, a2)[0]
        d2 = P - i2 * a2
        if s1 is not None:
            d2 = d2 - np.rint(d2 / L) * L
        i2 = i2.astype(idt)
        d2 = d2.astype(fdt)
        d2 = d2 / fdt.type(a2)
    else:                                                # pm_util.py:119-137
        a1 = fdt.type(a1)
        i12, d12 = _float_divmod(b12, np.float64(a1))
        i1 = (i1 - i12.astype(idt)).astype(idt)
        d1 = (d1 - d12.astype(fdt)).astype(fdt)
        i1 = i1[:, None]
        d1 = d1[:, None]
        d1 = d1 / a1
        i2 = np.floor(d1).astype(idt)
        i2 = (i2 + neighbors).astype(idt)
        d2 = d1 - i2.astype(fdt)
        i2 = (i2 + i1).astype(idt)
        if s1 is not None:
            i2 = np.remainder(i2, s1).astype(idt)

    f2 = (1 - np.abs(d2)).astype(fdt)

    if s1 is None and s2 is not None:
        i2 = np.where(i2 < 0, s2, i2).astype(idt)

    def prod(f):
        out = f[..., 0]
        for j in range(1, f.shape[-1]):
            out = out * f[..., j]
        return out

    if grad:
        sign = np.sign(-d2)
        f2g = []
        for i in range(dim):
            not_i = tuple(range(i + 1, dim)) + tuple(range(0, i))
            if not_i:
                f2g.append(sign[..., i] * prod(f2[..., not_i]))
            else:
                f2g.append(sign[..., i])
        f2g = np.stack(f2g, axis=-1).astype(fdt)
        return i2, prod(f2).astype(fdt), f2g

    return i2, prod(f2).astype(fdt)


def _axis_default(i1, d1, a1, s1):
    """Per-axis neighbour indices (num, dim, 2) and fractions of the default
    branch (pm_util.py:119-137), with the same float32 operations as
    ``enmesh``; the 2**dim combinations are formed by ``_combine``."""
    fdt = d1.dtype
    a1 = fdt.type(a1)
    x = d1 / a1
    fl = np.floor(x)
    i0 = fl.astype(np.int64)
    w = np.empty(x.shape + (2,), dtype=fdt)
    ii = np.empty(x.shape + (2,), dtype=np.int64)
    for nb in (0, 1):
        d2 = x - (fl + fdt.type(nb)).astype(fdt)
        w[..., nb] = (1 - np.abs(d2)).astype(fdt)
        ii[..., nb] = np.remainder(i0 + nb + i1.astype(np.int64), np.asarray(s1, np.int64))
    return ii, w


def _combine(ii, w, shape):
    """Flat indices (num, 2**dim) and fraction products in the neighbour
    order of pm_util.py:95-97, dropping indices >= shape."""
    num, dim = ii.shape[:2]
    nk = 2 ** dim
    flat = None
    frac = None
    ok = None
    for a in range(dim):
        # neighbour bit a varies along broadcast axis (dim - a), so the
        # final reshape orders neighbours as k = sum_a bit_a << a
        bshape = (num,) + (1,) * (dim - 1 - a) + (2,) + (1,) * a
        ia = ii[:, a, :].reshape(bshape)
        fa = w[:, a, :].reshape(bshape)
        oka = ia < shape[a]
        flat = ia if flat is None else flat * shape[a] + ia
        frac = fa if frac is None else frac * fa
        ok = oka if ok is None else ok & oka
    flat = np.broadcast_to(flat, (num,) + (2,) * dim).reshape(num, nk)
    ok = np.broadcast_to(ok, (num,) + (2,) * dim).reshape(num, nk)
    frac = np.broadcast_to(frac, (num,) + (2,) * dim).reshape(num, nk)
    return np.where(ok, flat, -1), frac


def _enmesh_flat(pmid, disp, conf, offset, cell_size, spatial_shape):
    """(flat index, frac) as scatter/gather use them; the per-axis fast path
    gives results identical to ``enmesh`` + ``_flat_index`` for the default
    branch and zero offset."""
    if cell_size is None and np.all(np.asarray(offset) == 0):
        ii, w = _axis_default(pmid, disp, conf.cell_size, conf.mesh_shape)
        return _combine(ii, w, spatial_shape)
    ind, frac = enmesh(pmid, disp, conf.cell_size, conf.mesh_shape, offset, cell_size,
                       spatial_shape, False)
    return _flat_index(ind, spatial_shape), frac


def _flat_index(ind, shape):
    """Raveled mesh index with jax ``.at[]`` FILL_OR_DROP semantics: negative
    indices are normalised once by adding the size, anything still out of
    bounds is dropped (returned as -1)."""
    ind = ind.astype(np.int64)
    shape = np.asarray(shape, dtype=np.int64)
    ind = np.where(ind < 0, ind + shape, ind)
    ok = np.all((ind >= 0) & (ind < shape), axis=-1)
    flat = np.zeros(ind.shape[:-1], dtype=np.int64)
    for d in range(ind.shape[-1]):
        flat = flat * shape[d] + ind[..., d]
    return np.where(ok, flat, -1)


# ----------------------------------------------------------------------------
# scatter (scatter.py:8-150)
# ----------------------------------------------------------------------------

def scatter(pmid, disp, conf, mesh=None, val=None, offset=0, cell_size=None):
    """Multilinear scatter, scatter.py:33-83 (all chunks at once)."""
    fdt = np.dtype(conf.float_dtype)
    num, dim = pmid.shape
    if val is None:
        val = conf.mesh_size / conf.ptcl_num                # scatter.py:37-38
    val = np.asarray(val, dtype=fdt)
    if mesh is None:
        mesh = np.zeros(tuple(conf.mesh_shape) + val.shape[1:], dtype=fdt)
    mesh = np.array(mesh, dtype=fdt, copy=True)
    if mesh.shape[dim:] != val.shape[1:]:
        raise ValueError('channel shape mismatch: '
                         f'{mesh.shape[dim:]} != {val.shape[1:]}')
    spatial_shape = mesh.shape[:dim]
    chan = int(np.prod(mesh.shape[dim:], dtype=np.int64))

    flat, frac = _enmesh_flat(pmid, disp, conf, offset, cell_size, spatial_shape)
    if val.ndim != 0:
        v = val.reshape(num, 1, chan)
    else:
        v = val.reshape(1, 1, 1)
    contrib = (v * frac[..., None]).astype(fdt)             # (num, 2**dim, chan)

    ok = flat >= 0
    m = mesh.reshape(-1, chan)
    size = m.shape[0]
    for c in range(chan):
        w = np.broadcast_to(contrib[..., c], flat.shape)[ok]
        acc = np.bincount(flat[ok], weights=w.astype(np.float64), minlength=size)
        m[:, c] = (m[:, c].astype(np.float64) + acc).astype(fdt)
    return m.reshape(mesh.shape)


def scatter_vjp(pmid, disp, conf, mesh_cot, val=None, offset=0, cell_size=None):
    """Scatter VJP, scatter.py:86-148: returns (disp_cot, mesh_cot, val_cot)."""
    fdt = np.dtype(conf.float_dtype)
    num, dim = pmid.shape
    if val is None:
        val = conf.mesh_size / conf.ptcl_num
    val = np.asarray(val, dtype=fdt)
    mesh_cot = np.asarray(mesh_cot, dtype=fdt)
    spatial_shape = mesh_cot.shape[:dim]
    chan = int(np.prod(mesh_cot.shape[dim:], dtype=np.int64))

    ind, frac, frac_grad = enmesh(pmid, disp, conf.cell_size, conf.mesh_shape,
                                  offset, cell_size, spatial_shape, True)
    flat = _flat_index(ind, spatial_shape)
    m = mesh_cot.reshape(-1, chan)
    g = np.where((flat >= 0)[..., None], m[np.maximum(flat, 0)], 0).astype(fdt)

    if val.ndim != 0:
        v = val.reshape(num, 1, chan)
    else:
        v = val.reshape(1, 1, 1)
    dc = (g * v).sum(axis=-1, dtype=fdt)                    # (num, 2**dim)
    disp_cot = (dc[..., None] * frac_grad).sum(axis=1, dtype=fdt)
    disp_cot = (disp_cot / fdt.type(cell_size if cell_size is not None
                                    else conf.cell_size)).astype(fdt)
    val_cot = (g * frac[..., None]).sum(axis=1, dtype=fdt)  # (num, chan)
    val_cot = val_cot.reshape((num,) + mesh_cot.shape[dim:])
    return disp_cot, mesh_cot, val_cot


# ----------------------------------------------------------------------------
# gather (gather.py:8-144)
# ----------------------------------------------------------------------------

def gather(pmid, disp, conf, mesh, val=0, offset=0, cell_size=None):
    """Multilinear gather, gather.py:33-77."""
    fdt = np.dtype(conf.float_dtype)
    num, dim = pmid.shape
    mesh = np.asarray(mesh, dtype=fdt)
    val = np.asarray(val, dtype=fdt)
    if mesh.shape[dim:] != val.shape[1:]:
        raise ValueError('channel shape mismatch: '
                         f'{mesh.shape[dim:]} != {val.shape[1:]}')
    spatial_shape = mesh.shape[:dim]
    chan_shape = mesh.shape[dim:]
    chan = int(np.prod(chan_shape, dtype=np.int64))

    flat, frac = _enmesh_flat(pmid, disp, conf, offset, cell_size, spatial_shape)
    m = mesh.reshape(-1, chan)
    g = np.where((flat >= 0)[..., None], m[np.maximum(flat, 0)], 0).astype(fdt)
    s = (g * frac[..., None]).sum(axis=1, dtype=fdt)        # (num, chan)
    s = s.reshape((num,) + chan_shape)
    return (val + s).astype(fdt)


def gather_vjp(pmid, disp, conf, mesh, val_cot, offset=0, cell_size=None):
    """Gather VJP, gather.py:80-142: returns (disp_cot, mesh_cot, val_cot)."""
    fdt = np.dtype(conf.float_dtype)
    num, dim = pmid.shape
    mesh = np.asarray(mesh, dtype=fdt)
    val_cot = np.asarray(val_cot, dtype=fdt)
    spatial_shape = mesh.shape[:dim]
    chan = int(np.prod(mesh.shape[dim:], dtype=np.int64))

    ind, frac, frac_grad = enmesh(pmid, disp, conf.cell_size, conf.mesh_shape,
                                  offset, cell_size, spatial_shape, True)
    flat = _flat_index(ind, spatial_shape)
    m = mesh.reshape(-1, chan)
    g = np.where((flat >= 0)[..., None], m[np.maximum(flat, 0)], 0).astype(fdt)
    vc = val_cot.reshape(num, 1, chan) if val_cot.ndim != 0 else val_cot.reshape(1, 1, 1)

    dc = (vc * g).sum(axis=-1, dtype=fdt)
    disp_cot = (dc[..., None] * frac_grad).sum(axis=1, dtype=fdt)
    disp_cot = (disp_cot / fdt.type(cell_size if cell_size is not None
                                    else conf.cell_size)).astype(fdt)

    contrib = np.broadcast_to(vc * frac[..., None], g.shape)
    ok = flat >= 0
    mc = np.zeros((m.shape[0], chan), dtype=np.float64)
    for c in range(chan):
        mc[:, c] = np.bincount(flat[ok], weights=contrib[..., c][ok].astype(np.float64),
                               minlength=m.shape[0])
    mesh_cot = mc.astype(fdt).reshape(mesh.shape)
    return disp_cot, mesh_cot, val_cot


# ----------------------------------------------------------------------------
# FFT helpers (pm_util.py:159-344)
# ----------------------------------------------------------------------------

def fftfreq(shape, spacing, dtype=np.float64):
    """Angular wavevectors, sparse ij grids, pm_util.py:159-199."""
    period = 1.0 if spacing is None else 2 * math.pi / spacing
    kvec = []
    for s in shape[:-1]:
        kvec.append((np.fft.fftfreq(s) * period).astype(dtype))
    kvec.append((np.fft.rfftfreq(shape[-1]) * period).astype(dtype))
    return np.meshgrid(*kvec, sparse=True, indexing='ij')


def fftfwd(f, norm=None):
    """rfftn, pm_util.py:236-289 (float norm = grid spacing)."""
    if norm is None or isinstance(norm, str):
        return sfft.rfftn(f, norm=norm, workers=FFT_WORKERS)
    d = f.ndim
    out = sfft.rfftn(f, norm='backward', workers=FFT_WORKERS)
    return (norm**d * out).astype(out.dtype)


def fftinv(f, shape=None, norm=None):
    """irfftn, pm_util.py:292-344."""
    if norm is None or isinstance(norm, str):
        return sfft.irfftn(f, s=shape, norm=norm, workers=FFT_WORKERS)
    d = f.ndim if shape is None else len(shape)
    out = sfft.irfftn(f, s=shape, norm='backward', workers=FFT_WORKERS)
    return (norm**-d * out).astype(out.dtype)


def laplace(kvec, src):
    """-src/k^2 with the k=0 mode zeroed, gravity.py:9-16 (self-adjoint,
    gravity.py:23-32)."""
    k2 = kvec[0] ** 2
    for k in kvec[1:]:
        k2 = k2 + k ** 2
    with np.errstate(divide='ignore', invalid='ignore'):
        pot = np.where(k2 != 0, -src / k2, 0)
    return pot.astype(src.dtype)


def neg_grad(k, pot, spacing):
    """-i k pot with the Nyquist plane zeroed, gravity.py:37-44."""
    nyquist = np.pi / spacing
    eps = nyquist * np.finfo(k.dtype).eps
    neg_ik = np.where(np.abs(np.abs(k) - nyquist) <= eps, 0, -1j * k)
    return (neg_ik * pot).astype(pot.dtype)


# ----------------------------------------------------------------------------
# gravity (gravity.py:47-72) and its VJP
# ----------------------------------------------------------------------------

def gravity_meshes(pmid, disp, Omega_m, conf):
    """Forward Poisson solve up to the three real acceleration meshes."""
    fdt = np.dtype(conf.float_dtype)
    kvec = fftfreq(conf.mesh_shape, conf.cell_size, dtype=fdt)
    dens = scatter(pmid, disp, conf)
    dens = (dens - 1).astype(fdt)
    dens = (dens * fdt.type(1.5 * fdt.type(Omega_m))).astype(fdt)
    dens_k = fftfwd(dens)
    pot = laplace(kvec, dens_k)
    meshes = []
    for k in kvec:
        g = neg_grad(k, pot, conf.cell_size)
        g = fftinv(g, shape=conf.mesh_shape).astype(fdt)
        meshes.append(g)
    return meshes


def gravity(pmid, disp, Omega_m, conf):
    """Particle accelerations, gravity.py:47-72 -> (num, dim)."""
    meshes = gravity_meshes(pmid, disp, Omega_m, conf)
    acc = [gather(pmid, disp, conf, g) for g in meshes]
    return np.stack(acc, axis=-1)


def _irfftn_adjoint(t, shape):
    """Real transpose of ``irfftn(., s=shape)`` (backward norm) as a map from
    the Hermitian half spectrum, paired with Re(sum(conj(a) b)) there:
    mask*rfftn(t)/N with the de-duplicated planes weighted by 2."""
    n = int(np.prod(shape))
    x = sfft.rfftn(t, workers=FFT_WORKERS)
    mask = np.full(x.shape[-1], 2.0)
    mask[0] = 1
    if shape[-1] % 2 == 0:
        mask[-1] = 1
    return (x * mask / n).astype(x.dtype)


def _rfftn_adjoint_direct(t, shape):
    """x -> Re(sum_{k in half} conj(t_k) X_k) gradient, X = rfftn(x): equal to
    N * irfftn(w * t) with w = 1 on the planes rfftn stores once per pair
    of conjugates and 1/2 on the self-conjugate planes (kz = 0, kz = Nyq).
    irfftn symmetrises those planes itself, so halving them is exact."""
    n = int(np.prod(shape))
    w = np.ones(t.shape[-1])
    w[0] = 2.0
    if shape[-1] % 2 == 0:
        w[-1] = 2.0
    # irfftn(u) = (1/N) sum_full u_k e^{ikx} with u Hermitian-completed; the
    # gradient of Re(sum_half conj(t) X) is sum_half Re(t_k e^{ikx}) which
    # equals (N/2) irfftn(t') where t' doubles the self-conjugate planes.
    return (0.5 * n * sfft.irfftn(t * w, s=shape, workers=FFT_WORKERS)).astype(
        np.real(t).dtype)


def gravity_vjp(pmid, disp, Omega_m, conf, acc_cot):
    """VJP of ``gravity`` w.r.t. disp and Omega_m.

    pmwd obtains this by JAX autodiff through gravity.py:47-72 (using the
    custom VJPs of scatter, gather and laplace).  Here each adjoint is
    written out: gather VJP per axis (gather.py:98-113), transpose of irfftn,
    neg_grad (its own transpose), laplace (self-adjoint, gravity.py:23-32),
    transpose of rfftn, the 1.5*Omega_m scale and scatter VJP
    (scatter.py:104-119).  Returns (acc, disp_cot, Omega_m_cot).
    """
    fdt = np.dtype(conf.float_dtype)
    shape = tuple(conf.mesh_shape)
    kvec = fftfreq(shape, conf.cell_size, dtype=fdt)
    rho = scatter(pmid, disp, conf)
    delta = (rho - 1).astype(fdt)
    s = fdt.type(1.5 * fdt.type(Omega_m))
    dens_k = fftfwd((delta * s).astype(fdt))
    pot = laplace(kvec, dens_k)

    acc = []
    disp_cot = np.zeros(disp.shape, dtype=np.float64)
    pot_cot = np.zeros(pot.shape, dtype=np.complex128)
    for i, k in enumerate(kvec):
        g = neg_grad(k, pot, conf.cell_size)
        g = fftinv(g, shape=shape).astype(fdt)
        acc.append(gather(pmid, disp, conf, g))
        dcot, mcot, _ = gather_vjp(pmid, disp, conf, g, acc_cot[:, i])
        disp_cot += dcot
        # real-space cot of g -> half-spectrum cot of the neg_grad output
        gk_cot = _irfftn_adjoint(mcot.astype(np.float64), shape)
        # neg_grad is multiplication by m = -ik (masked); its adjoint under
        # Re(conj(a) b) is multiplication by conj(m)
        nyquist = np.pi / conf.cell_size
        eps = nyquist * np.finfo(k.dtype).eps
        m = np.where(np.abs(np.abs(k) - nyquist) <= eps, 0, -1j * k.astype(np.float64))
        pot_cot += np.conj(m) * gk_cot
    acc = np.stack(acc, axis=-1)

    k2 = sum(k.astype(np.float64) ** 2 for k in kvec)
    with np.errstate(divide='ignore', invalid='ignore'):
        dens_k_cot = np.where(k2 != 0, -pot_cot / k2, 0)
    dens_cot = _rfftn_adjoint_direct(dens_k_cot, shape)      # real, float64
    Om_cot = 1.5 * float(np.sum(delta.astype(np.float64) * dens_cot))
    rho_cot = (dens_cot * float(s)).astype(fdt)
    dcot, _, _ = scatter_vjp(pmid, disp, conf, rho_cot)
    disp_cot += dcot
    return acc, disp_cot.astype(fdt), Om_cot
