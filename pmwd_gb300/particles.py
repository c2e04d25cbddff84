"""Particle state, mirroring pmwd/particles.py:18-346.

``pmid`` is int16 (n, dim) -- the nearest mesh point of each particle's
Lagrangian position -- and ``disp``/``vel``/``acc`` are float32 (n, dim),
all torch tensors resident on the GPU in the reference's row-major layout.
"""

import dataclasses
from dataclasses import dataclass, field
from itertools import accumulate
from operator import mul
from typing import Any, Optional

import numpy as np
import torch

from . import _lib
from .configuration import Configuration, jax_linspace
from .cosmology import E2


def _device(device=None):
    if device is not None:
        return torch.device(device)
    return torch.device('cuda', torch.cuda.current_device())


@dataclass(frozen=True)
class Particles:
    """Particle state (particles.py:18-76)."""

    conf: Configuration = field(repr=False)

    pmid: torch.Tensor
    disp: torch.Tensor
    vel: Optional[torch.Tensor] = None
    acc: Optional[torch.Tensor] = None

    attr: Any = None

    def __post_init__(self):
        conf = self.conf
        for name in ('pmid', 'disp', 'vel', 'acc'):
            v = getattr(self, name)
            if v is None:
                continue
            dt = conf.pmid_dtype if name == 'pmid' else conf.float_dtype
            if not torch.is_tensor(v):
                v = torch.as_tensor(np.asarray(v))
            if v.dtype != dt:
                v = v.to(dt)
            object.__setattr__(self, name, v)

    def replace(self, **changes):
        return dataclasses.replace(self, **changes)

    def __len__(self):
        return len(self.pmid)

    def __getitem__(self, key):
        kw = {n: (getattr(self, n)[key] if getattr(self, n) is not None else None)
              for n in ('pmid', 'disp', 'vel', 'acc')}
        return self.replace(**kw)

    @classmethod
    def from_pos(cls, conf, pos, wrap=True):
        """pmid and disp from positions (particles.py:81-107)."""
        pos = torch.as_tensor(pos, dtype=torch.float64)
        pmid = torch.round(pos / conf.cell_size)
        disp = pos - pmid * conf.cell_size
        pmid = pmid.to(conf.pmid_dtype)
        disp = disp.to(conf.float_dtype)
        if wrap:
            shape = torch.tensor(conf.mesh_shape, dtype=conf.pmid_dtype, device=pmid.device)
            pmid = torch.remainder(pmid, shape)
        return cls(conf, pmid, disp)

    @classmethod
    def gen_grid(cls, conf, vel=False, acc=False, device=None):
        """Particles on the uniform Lagrangian grid (particles.py:109-154)."""
        dev = _device(device)
        pmid, disp = [], []
        for sp, sm in zip(conf.ptcl_grid_shape, conf.mesh_shape):
            p1 = np.rint(jax_linspace(0, sm, sp, endpoint=False)).astype(np.int16)
            d1 = np.arange(sp, dtype=np.int64) * sm - p1.astype(np.int64) * sp
            d1 = (d1 * (conf.cell_size / sp)).astype(np.float32)
            pmid.append(torch.from_numpy(p1).to(dev))
            disp.append(torch.from_numpy(d1).to(dev))
        pmid = torch.stack(torch.meshgrid(*pmid, indexing='ij'), dim=-1).reshape(-1, conf.dim)
        disp = torch.stack(torch.meshgrid(*disp, indexing='ij'), dim=-1).reshape(-1, conf.dim)
        v = torch.zeros_like(disp) if vel else None
        a = torch.zeros_like(disp) if acc else None
        return cls(conf, pmid.contiguous(), disp.contiguous(), vel=v, acc=a)

    def raveled_id(self, dtype=torch.int64, wrap=False):
        """Raveled particle IDs from pmid (particles.py:156-182)."""
        conf = self.conf
        pmid = self.pmid.to(torch.int64)
        if wrap:
            pmid = torch.remainder(pmid, torch.tensor(conf.mesh_shape, device=pmid.device))
        strides = tuple(accumulate((1,) + conf.mesh_shape[:0:-1], mul))[::-1]
        return sum(pmid[:, i] * s for i, s in enumerate(strides)).to(dtype)

    def pos(self, dtype=torch.float64, wrap=True):
        """Particle positions in [L] (particles.py:184-209)."""
        conf = self.conf
        p = self.pmid.to(dtype) * conf.cell_size + self.disp.to(dtype)
        if wrap:
            p = torch.remainder(p, torch.tensor(conf.box_size, dtype=dtype, device=p.device))
        return p


def ptcl_enmesh(ptcl, conf, offset=0, cell_size=None, mesh_shape=None, wrap=True, drop=True,
                grad=False):
    """Multilinear mesh indices, fractions and fraction gradients
    (particles.py:212-254) computed by the CUDA ``pmx_enmesh`` kernel.

    ``wrap``: wrap around the periodic boundaries (``conf.mesh_shape``);
    without wrapping the indices are the reference's int16 sums, and with
    ``drop`` the negative ones are replaced by ``mesh_shape`` (with wrapping
    no index is negative, so ``drop`` has no effect).
    """
    if mesh_shape is None:
        mesh_shape = conf.mesh_shape
    n, dim = ptcl.pmid.shape
    spec = _lib.make_spec(dim, conf.mesh_shape if wrap else None, mesh_shape, conf.cell_size,
                          offset, cell_size, drop=drop)
    dev = ptcl.disp.device
    nk = 2 ** dim
    ind = torch.empty((n, nk, dim), dtype=torch.int32, device=dev)
    frac = torch.empty((n, nk), dtype=torch.float32, device=dev)
    fg = torch.empty((n, nk, dim), dtype=torch.float32, device=dev) if grad else None
    _lib.call('pmx_enmesh', spec, ptcl.pmid.contiguous(),
              ptcl.disp.contiguous(), n, _lib.ptr(ind), _lib.ptr(frac), _lib.ptr(fg),
              _lib.stream_ptr(dev))
    ind = ind.to(conf.pmid_dtype)
    return (ind, frac, fg) if grad else (ind, frac)


def ptcl_pos(ptcl, conf, dtype=float, wrap=True):
    raise RuntimeError('Deprecated and replaced by ptcl.pos')


def ptcl_rpos(ptcl, ref, conf, wrap=True):
    """Positions relative to reference points or particles (particles.py:261-291)."""
    if not isinstance(ref, Particles):
        ref = Particles.from_pos(conf, ref, wrap=False)
    rpos = (ptcl.pmid - ref.pmid.to(ptcl.pmid.device)).to(conf.float_dtype)
    rpos = rpos * conf.cell_size + (ptcl.disp - ref.disp.to(ptcl.disp.device))
    if wrap:
        box = torch.tensor(conf.box_size, dtype=conf.float_dtype, device=rpos.device)
        rpos = rpos - torch.round(rpos / box) * box
    return rpos


def ptcl_rsd(ptcl, los, a, cosmo):
    """Redshift-space distortion displacements (particles.py:294-324)."""
    conf = cosmo.conf
    dev = ptcl.vel.device
    los = torch.as_tensor(los, dtype=conf.float_dtype, device=dev)
    a = torch.as_tensor(a, dtype=conf.float_dtype, device=dev)
    E = torch.sqrt(E2(a.double().cpu(), cosmo)).to(conf.float_dtype).to(dev)
    rsd = (ptcl.vel * los).sum(dim=1, keepdim=True)
    return rsd * los / (a ** 2 * E)


def ptcl_los(ptcl, obs, conf):
    """Line-of-sight unit vectors (particles.py:327-346)."""
    los = ptcl_rpos(ptcl, obs, conf, wrap=False)
    return los / torch.linalg.norm(los, dim=1, keepdim=True)
