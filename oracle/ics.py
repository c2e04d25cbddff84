"""NumPy restatement of pmwd's particle grid, initial conditions and power
spectrum (test infrastructure only).

* ``gen_grid``       pmwd/particles.py:109-154
* ``pos``            pmwd/particles.py:184-209
* ``linear_modes``   pmwd/modes.py:67-117
* ``lpt`` (2LPT)     pmwd/lpt.py:13-76, 136-212
* ``powspec``        pmwd/spec_util.py:10-147

* ``white_noise``    pmwd/modes.py:12-49, with JAX's Threefry normal draw
  restated in ``oracle/prng.py`` (the reference's realisation of a seed)
"""

import math

import numpy as np

from . import cosmo as oc
from . import pm
from . import prng


def gen_grid(conf):
    """Particles on the Lagrangian grid: (pmid, disp), particles.py:109-144."""
    pmid, disp = [], []
    for sp, sm in zip(conf.ptcl_grid_shape, conf.mesh_shape):
        p1 = oc.jax_linspace(0, sm, sp, endpoint=False)
        p1 = np.rint(p1).astype(conf.pmid_dtype)
        pmid.append(p1)
        d1 = np.arange(sp, dtype=np.int64) * sm - p1.astype(np.int64) * sp
        d1 = d1 * (conf.cell_size / sp)
        disp.append(d1.astype(conf.float_dtype))
    pmid = np.stack(np.meshgrid(*pmid, indexing='ij'), axis=-1).reshape(-1, conf.dim)
    disp = np.stack(np.meshgrid(*disp, indexing='ij'), axis=-1).reshape(-1, conf.dim)
    return pmid, disp


def pos(pmid, disp, conf, wrap=True):
    p = pmid.astype(np.float64) * conf.cell_size + disp.astype(np.float64)
    if wrap:
        p = np.remainder(p, np.array(conf.box_size))
    return p


def white_noise(seed, conf, real=False, layout='original'):
    """modes.py:12-49 (Fourier or real modes; ``unit_abs`` not restated)."""
    modes = prng.normal_f32(seed, conf.ptcl_grid_shape, layout).astype(conf.float_dtype)
    if real:
        return modes
    return pm.fftfwd(modes, norm='ortho')


def linear_modes(modes, cosmo, conf, a=None):
    """modes.py:67-86 (Fourier output)."""
    fdt = conf.float_dtype
    kvec = pm.fftfreq(conf.ptcl_grid_shape, conf.ptcl_spacing, dtype=fdt)
    k = np.sqrt(sum(kk ** 2 for kk in kvec)).astype(fdt)
    Plin = oc.linear_power(k.astype(np.float64), a, cosmo, conf).astype(fdt)
    if np.isrealobj(modes):
        modes = pm.fftfwd(modes, norm='ortho')
    return (modes * np.sqrt(Plin * fdt.type(conf.box_vol))).astype(modes.dtype)


def _strain(kvec, i, j, pot, conf):
    """lpt.py:13-37."""
    fdt = conf.float_dtype
    k_i, k_j = kvec[i], kvec[j]
    nyquist = np.pi / conf.ptcl_spacing
    eps = nyquist * np.finfo(fdt).eps
    if i != j:
        k_i = np.where(np.abs(np.abs(k_i) - nyquist) <= eps, 0, k_i)
        k_j = np.where(np.abs(np.abs(k_j) - nyquist) <= eps, 0, k_j)
    strain = (-k_i * k_j * pot).astype(pot.dtype)
    return pm.fftinv(strain, shape=conf.ptcl_grid_shape).astype(fdt)


def _L(kvec, pot, conf):
    """lpt.py:40-76 with m == n."""
    L = np.zeros(conf.ptcl_grid_shape, dtype=conf.float_dtype)
    for i in range(conf.dim):
        sm = _strain(kvec, i, i, pot, conf)
        for j in range(conf.dim - 1, i, -1):
            L += sm * _strain(kvec, j, j, pot, conf)
    for i in range(conf.dim - 1):
        for j in range(i + 1, conf.dim):
            s = _strain(kvec, i, j, pot, conf)
            L -= s * s
    return L


def lpt(modes, cosmo, conf):
    """2LPT displacements and velocities at a_start, lpt.py:136-212.
    Returns (pmid, disp, vel)."""
    fdt = conf.float_dtype
    modes = (modes / fdt.type(conf.ptcl_cell_vol)).astype(modes.dtype)
    kvec = pm.fftfreq(conf.ptcl_grid_shape, conf.ptcl_spacing, dtype=fdt)
    pot = [pm.laplace(kvec, modes)]
    if conf.lpt_order > 1:
        src2 = pm.fftfwd(_L(kvec, pot[0], conf))
        pot.append(pm.laplace(kvec, src2))
    a = conf.a_start
    pmid, disp = gen_grid(conf)
    vel = np.zeros_like(disp)
    for order in range(1, 1 + conf.lpt_order):
        D = oc.growth(a, cosmo, conf, order=order)
        dD = oc.growth(a, cosmo, conf, order=order, deriv=1)
        a2HDp = a ** 2 * np.sqrt(oc.E2(a, cosmo)) * dD
        D, a2HDp = fdt.type(D), fdt.type(a2HDp)
        for i, k in enumerate(kvec):
            g = pm.neg_grad(k, pot[order - 1], conf.ptcl_spacing)
            g = pm.fftinv(g, shape=conf.ptcl_grid_shape).astype(fdt).ravel()
            disp[:, i] += D * g
            vel[:, i] += a2HDp * g
    return pmid, disp, vel


def powspec(f, spacing, bins=1j / 3, cut_zero=True, cut_nyq=True, deconv=None):
    """Spherically binned auto power spectrum, spec_util.py:10-147 (log bins
    or linear bins; float64 accumulation; ``deconv``: the sinc^-deconv
    window of each axis, spec_util.py:115-116)."""
    f = np.asarray(f)
    grid_shape = f.shape[-3:]
    kfun = 1 / max(grid_shape)
    knyq = 0.5
    kmax = knyq * math.sqrt(3)
    if isinstance(bins, complex):
        kmaxable = all(s % 2 == 0 for s in grid_shape)
        bnum = 1 + math.ceil(math.log2(kmax / kfun) / bins.imag) + kmaxable
        bcut = 1 + math.ceil(math.log2(knyq / kfun) / bins.imag) if cut_nyq else bnum
        edges = kfun * 2 ** (bins.imag * np.arange(bnum))
        right = False
    else:
        w = bins * kfun
        bnum = 1 + math.ceil(kmax / w)
        bcut = 1 + math.ceil(knyq / w) if cut_nyq else bnum
        edges = w * np.arange(bnum)
        right = True
    F = pm.fftfwd(f)
    P = F.real.astype(np.float64) ** 2 + F.imag.astype(np.float64) ** 2
    kvec = pm.fftfreq(grid_shape, None, dtype=np.float64)
    k = np.sqrt(sum(kk ** 2 for kk in kvec))
    if deconv is not None:
        for kk in kvec:
            P = P * np.sinc(kk) ** -deconv   # numpy's sinc has the pi
    k = np.broadcast_to(k, P.shape)
    N = np.full(P.shape, 2.0)
    N[..., 0] = 1
    if grid_shape[-1] % 2 == 0:
        N[..., -1] = 1
    b = np.digitize(k.ravel(), edges, right=right)
    kk = np.bincount(b, weights=(k * N).ravel(), minlength=bnum)[:bnum]
    PP = np.bincount(b, weights=(P * N).ravel(), minlength=bnum)[:bnum]
    NN = np.bincount(b, weights=N.ravel(), minlength=bnum)[:bnum]
    sl = slice(int(cut_zero), bcut)
    kk, PP, NN, edges = kk[sl], PP[sl], NN[sl], edges[:bcut]
    with np.errstate(invalid='ignore', divide='ignore'):   # empty bins: NaN, as the reference
        kk = kk / NN * 2 * math.pi / spacing
        PP = PP / NN * spacing ** 3 / math.prod(grid_shape)
    return kk, PP, NN, edges * 2 * math.pi / spacing
