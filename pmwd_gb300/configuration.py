"""Configuration: the static simulation parameters, mirroring
pmwd/configuration.py:21-325 field by field.

Differences from the reference, by design:

* dtypes are torch dtypes; the particle-mesh kernels compute in float32 with
  int16 ``pmid``, so ``float_dtype`` must be float32 and ``pmid_dtype`` int16
  (the reference also allows float64/other ints on its XLA path);
* the top-hat variance tables (``mcfit.TophatVar`` in the reference) are
  replaced by direct quadrature in ``boltzmann.varlin``;
* ``kahan`` (default False) turns on compensated float32 updates of disp and
  vel in the N-body loop; it is off by default so results follow pmwd.
"""

import dataclasses
import math
from dataclasses import dataclass, field
from typing import ClassVar, Optional, Tuple, Union

import numpy as np
import torch


def jax_linspace(start, stop, num, endpoint=True):
    """``jnp.linspace`` in float64: ``start*(1-t) + stop*t``, ``t = i/div``."""
    div = (num - 1) if endpoint else num
    if num == 1:
        return np.array([start], dtype=np.float64)
    t = np.arange(num, dtype=np.float64) / div
    return start * (1 - t) + stop * t


@dataclass(frozen=True)
class Configuration:
    """Configuration parameters, immutable (pmwd/configuration.py:21-196).

    Parameters are those of the reference: ``ptcl_spacing``,
    ``ptcl_grid_shape``, ``mesh_shape`` (int/float ratio or tuple),
    ``cosmo_dtype``, ``pmid_dtype``, ``float_dtype``, ``k_pivot_Mpc``,
    ``T_cmb``, units ``M``/``L``/``T``, transfer and growth settings,
    ``lpt_order``, ``a_start``/``a_stop``, ``a_lpt_maxstep``,
    ``a_nbody_maxstep``, ``symp_splits`` and ``chunk_size``.
    """

    ptcl_spacing: float
    ptcl_grid_shape: Tuple[int, ...]

    mesh_shape: Union[float, Tuple[int, ...]] = 1

    cosmo_dtype: torch.dtype = torch.float64
    pmid_dtype: torch.dtype = torch.int16
    float_dtype: torch.dtype = torch.float32

    k_pivot_Mpc: float = 0.05

    T_cmb: float = 2.7255

    M_sun_SI: ClassVar[float] = 1.98847e30
    Mpc_SI: ClassVar[float] = 3.0856775815e22
    H_0_SI: ClassVar[float] = 1e5 / Mpc_SI
    c_SI: ClassVar[int] = 299792458
    G_SI: ClassVar[float] = 6.67430e-11

    M: float = 1e10 * M_sun_SI
    L: float = Mpc_SI
    T: float = 1 / H_0_SI

    transfer_fit: bool = True
    transfer_fit_nowiggle: bool = False
    transfer_lgk_min: float = -4
    transfer_lgk_max: float = 3
    transfer_lgk_maxstep: float = 1 / 128

    growth_rtol: Optional[float] = None
    growth_atol: Optional[float] = None
    growth_inistep: Union[float, None, Tuple[Optional[float], Optional[float]]] = (1, None)

    lpt_order: int = 2

    a_start: float = 1 / 64
    a_stop: float = 1
    a_lpt_maxstep: float = 1 / 128
    a_nbody_maxstep: float = 1 / 64

    symp_splits: Tuple[Tuple[float, float], ...] = ((0, 0.5), (1, 0.5))

    chunk_size: int = 2 ** 24

    kahan: bool = False

    def __post_init__(self):
        object.__setattr__(self, 'ptcl_grid_shape', tuple(int(s) for s in self.ptcl_grid_shape))
        if isinstance(self.mesh_shape, (int, float)):
            mesh_shape = tuple(round(s * self.mesh_shape) for s in self.ptcl_grid_shape)
            object.__setattr__(self, 'mesh_shape', mesh_shape)
        object.__setattr__(self, 'mesh_shape', tuple(int(s) for s in self.mesh_shape))
        if len(self.ptcl_grid_shape) != len(self.mesh_shape):
            raise ValueError('particle and mesh grid dimensions differ')
        if any(sm < sp for sp, sm in zip(self.ptcl_grid_shape, self.mesh_shape)):
            raise ValueError('mesh grid cannot be smaller than particle grid')
        if any(self.ptcl_grid_shape[0] * sm != self.mesh_shape[0] * sp
               for sp, sm in zip(self.ptcl_grid_shape[1:], self.mesh_shape[1:])):
            raise ValueError('particle and mesh grid aspect ratios differ')
        if not self.cosmo_dtype.is_floating_point:
            raise ValueError('cosmo_dtype must be floating point numbers')
        if self.pmid_dtype not in (torch.int8, torch.int16, torch.int32, torch.int64):
            raise ValueError('pmid_dtype must be signed integers')
        if not self.float_dtype.is_floating_point:
            raise ValueError('float_dtype must be floating point numbers')
        if self.float_dtype != torch.float32 or self.pmid_dtype != torch.int16:
            raise ValueError('the GB300 kernels compute with float32 disp/vel/acc and int16 '
                             'pmid; float_dtype must be float32 and pmid_dtype int16')
        if max(self.mesh_shape) > 32767:
            raise ValueError('mesh_shape must fit int16 pmid')

        growth_tol = math.sqrt(np.finfo(np.float64).eps)
        if self.growth_rtol is None:
            object.__setattr__(self, 'growth_rtol', growth_tol)
        if self.growth_atol is None:
            object.__setattr__(self, 'growth_atol', growth_tol)

        if any(len(s) != 2 for s in self.symp_splits):
            raise ValueError(f'symp_splits={self.symp_splits} not supported')
        symp_splits_sum = tuple(sum(s) for s in zip(*self.symp_splits))
        if symp_splits_sum != (1, 1):
            raise ValueError(f'sum of symplectic splits = {symp_splits_sum} != (1, 1)')

    def replace(self, **changes):
        return dataclasses.replace(self, **changes)

    @property
    def dim(self):
        return len(self.ptcl_grid_shape)

    @property
    def ptcl_cell_vol(self):
        return self.ptcl_spacing ** self.dim

    @property
    def ptcl_num(self):
        return int(np.prod(self.ptcl_grid_shape, dtype=np.int64))

    @property
    def box_size(self):
        return tuple(self.ptcl_spacing * s for s in self.ptcl_grid_shape)

    @property
    def box_vol(self):
        return float(np.prod(self.box_size))

    @property
    def cell_size(self):
        return self.ptcl_spacing * self.ptcl_grid_shape[0] / self.mesh_shape[0]

    @property
    def cell_vol(self):
        return self.cell_size ** self.dim

    @property
    def mesh_size(self):
        return int(np.prod(self.mesh_shape, dtype=np.int64))

    @property
    def V(self):
        return self.L / self.T

    @property
    def H_0(self):
        return self.H_0_SI * self.T

    @property
    def c(self):
        return self.c_SI / self.V

    @property
    def G(self):
        return self.G_SI * self.M / (self.L * self.V ** 2)

    @property
    def rho_crit(self):
        return 3 * self.H_0 ** 2 / (8 * math.pi * self.G)

    @property
    def transfer_k_num(self):
        return 1 + math.ceil((self.transfer_lgk_max - self.transfer_lgk_min)
                             / self.transfer_lgk_maxstep) + 1

    @property
    def transfer_lgk_step(self):
        return ((self.transfer_lgk_max - self.transfer_lgk_min) / (self.transfer_k_num - 2))

    @property
    def transfer_k(self):
        lg = jax_linspace(self.transfer_lgk_min, self.transfer_lgk_max, self.transfer_k_num - 1)
        return torch.from_numpy(np.concatenate(([0.0], 10.0 ** lg)))

    @property
    def a_lpt_num(self):
        return math.ceil(self.a_start / self.a_lpt_maxstep)

    @property
    def a_lpt_step(self):
        return self.a_start / self.a_lpt_num

    @property
    def a_nbody_num(self):
        return math.ceil((self.a_stop - self.a_start) / self.a_nbody_maxstep)

    @property
    def a_nbody_step(self):
        return (self.a_stop - self.a_start) / self.a_nbody_num

    @property
    def a_lpt(self):
        return torch.from_numpy(jax_linspace(0, self.a_start, self.a_lpt_num + 1))

    @property
    def a_nbody(self):
        return torch.from_numpy(jax_linspace(self.a_start, self.a_stop, 1 + self.a_nbody_num))

    @property
    def growth_a(self):
        return torch.cat((self.a_lpt, self.a_nbody[1:]))

    @property
    def varlin_R(self):
        """Radii of the tabulated linear variance in [L]."""
        return torch.logspace(-2, 3, 256, dtype=torch.float64)
