"""Cosmology parameters and background functions in float64 on the host,
mirroring pmwd/cosmology.py:15-269.

Parameters are 0-d float64 CPU tensors so that torch autograd gives the
cosmological gradients (the reference gets them from JAX AD through the same
functions).  ``Cosmology`` supports the reference's linear operations
(``+``, ``-``, scalar ``*``) for tangents and cotangents.
"""

import dataclasses
from dataclasses import dataclass, field
from functools import partial
from typing import ClassVar, Optional

import torch

from .configuration import Configuration

_PARAMS = ('A_s_1e9', 'n_s', 'Omega_m', 'Omega_b', 'h', 'Omega_k_', 'w_0_', 'w_a_')


def _f64(x):
    if x is None:
        return None
    if torch.is_tensor(x):
        return x.to(torch.float64) if x.dtype != torch.float64 else x
    return torch.tensor(float(x), dtype=torch.float64)


@dataclass(frozen=True)
class Cosmology:
    """Cosmological parameters (pmwd/cosmology.py:15-162).

    Trailing-underscore parameters may be None and then take the fixed
    values ``Omega_k_fixed``, ``w_0_fixed``, ``w_a_fixed``.  ``transfer``,
    ``growth`` and ``varlin`` hold the tables filled by ``boltzmann``.
    """

    conf: Configuration = field(repr=False)

    A_s_1e9: torch.Tensor
    n_s: torch.Tensor
    Omega_m: torch.Tensor
    Omega_b: torch.Tensor
    h: torch.Tensor

    Omega_k_: Optional[torch.Tensor] = None
    Omega_k_fixed: ClassVar[float] = 0
    w_0_: Optional[torch.Tensor] = None
    w_0_fixed: ClassVar[float] = -1
    w_a_: Optional[torch.Tensor] = None
    w_a_fixed: ClassVar[float] = 0

    transfer: Optional[torch.Tensor] = field(default=None, compare=False, repr=False)
    growth: Optional[torch.Tensor] = field(default=None, compare=False, repr=False)
    varlin: Optional[torch.Tensor] = field(default=None, compare=False, repr=False)

    def __post_init__(self):
        for name in _PARAMS:
            object.__setattr__(self, name, _f64(getattr(self, name)))

    def replace(self, **changes):
        return dataclasses.replace(self, **changes)

    def params(self):
        """(name, tensor) of the parameters that are set."""
        return [(n, getattr(self, n)) for n in _PARAMS if getattr(self, n) is not None]

    def _map(self, fn, other=None):
        kw = {}
        for n in _PARAMS:
            x = getattr(self, n)
            if x is None:
                continue
            kw[n] = fn(x) if other is None else fn(x, getattr(other, n))
        return self.replace(**kw, transfer=None, growth=None, varlin=None)

    def __add__(self, other):
        return self._map(lambda a, b: a + b, other)

    def __sub__(self, other):
        return self._map(lambda a, b: a - b, other)

    def __mul__(self, other):
        return self._map(lambda a: a * other)

    __rmul__ = __mul__

    @classmethod
    def from_sigma8(cls, conf, sigma8, *args, **kwargs):
        """Cosmology with sigma8 instead of A_s (cosmology.py:95-105)."""
        from .boltzmann import boltzmann, varlin_integ
        cosmo = cls(conf, 1, *args, **kwargs)
        # only the variance entries around R = 8 Mpc/h are read
        cosmo = boltzmann(cosmo, conf, varlin=False)
        cosmo = varlin_integ(cosmo, conf, only=8 * conf.Mpc_SI / conf.L)
        A_s_1e9 = (sigma8 / cosmo.sigma8) ** 2
        return cls(conf, A_s_1e9, *args, **kwargs)

    def astype(self, dtype):
        return self

    @property
    def k_pivot(self):
        return self.conf.k_pivot_Mpc / (self.h * self.conf.Mpc_SI) * self.conf.L

    @property
    def A_s(self):
        return self.A_s_1e9 * 1e-9

    @property
    def Omega_c(self):
        return self.Omega_m - self.Omega_b

    @property
    def Omega_k(self):
        return _f64(self.Omega_k_fixed) if self.Omega_k_ is None else self.Omega_k_

    @property
    def Omega_de(self):
        return 1 - (self.Omega_m + self.Omega_k)

    @property
    def w_0(self):
        return _f64(self.w_0_fixed) if self.w_0_ is None else self.w_0_

    @property
    def w_a(self):
        return _f64(self.w_a_fixed) if self.w_a_ is None else self.w_a_

    @property
    def sigma8(self):
        from .boltzmann import varlin
        R = 8 * self.conf.Mpc_SI / self.conf.L
        return torch.sqrt(varlin(R, 1, self, self.conf))

    @property
    def ptcl_mass(self):
        return self.conf.rho_crit * self.Omega_m * self.conf.ptcl_cell_vol


SimpleLCDM = partial(Cosmology, A_s_1e9=2.0, n_s=0.96, Omega_m=0.3, Omega_b=0.05, h=0.7)
SimpleLCDM.__doc__ = 'Simple LCDM cosmology (cosmology.py:164-172).'

Planck18 = partial(Cosmology, A_s_1e9=2.105, n_s=0.9665, Omega_m=0.3111, Omega_b=0.04897,
                   h=0.6766)
Planck18.__doc__ = 'Planck 2018 cosmology, arXiv:1807.06209 Table 2 last column.'


def _a(a):
    return a.to(torch.float64) if torch.is_tensor(a) else torch.as_tensor(a, dtype=torch.float64)


def E2(a, cosmo):
    """Squared Hubble rate E^2(a) = H^2/H_0^2 (cosmology.py:185-219)."""
    a = _a(a)
    de_a = a ** (-3 * (1 + cosmo.w_0 + cosmo.w_a)) * torch.exp(-3 * cosmo.w_a * (1 - a))
    return cosmo.Omega_m * a ** -3 + cosmo.Omega_k * a ** -2 + cosmo.Omega_de * de_a


def H_deriv(a, cosmo):
    """dlnH/dlna (cosmology.py:222-242), in closed form: a E2'(a) / (2 E2)."""
    a = _a(a)
    p = -3 * (1 + cosmo.w_0 + cosmo.w_a)
    q = -3 * cosmo.w_a
    de_a = a ** p * torch.exp(q * (1 - a))
    a_dE2 = (-3 * cosmo.Omega_m * a ** -3 - 2 * cosmo.Omega_k * a ** -2
             + cosmo.Omega_de * de_a * (p - q * a))
    return 0.5 * a_dE2 / E2(a, cosmo)


def Omega_m_a(a, cosmo):
    """Omega_m(a) = Omega_m a^-3 / E2(a) (cosmology.py:245-269)."""
    a = _a(a)
    return cosmo.Omega_m / (a ** 3 * E2(a, cosmo))
