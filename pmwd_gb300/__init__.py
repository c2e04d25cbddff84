"""pmwd_gb300: pmwd's particle-mesh hot path on one NVIDIA GB300 (sm_103a).

Same public API as pmwd/__init__.py:4-15, with torch tensors on the GPU in
place of JAX arrays.  The CIC scatter/gather, Poisson force, leapfrog and
reversible adjoint run in ``libpmx.so`` (hand-written CUDA behind a C ABI,
``include/pmx.h``); initial conditions and analysis use torch on the GPU;
background tables are float64 on the host.
"""

from .configuration import Configuration
from .cosmology import Cosmology, SimpleLCDM, Planck18, E2, H_deriv, Omega_m_a
from .boltzmann import (transfer_integ, transfer_fit, transfer, growth_integ, growth,
                        varlin_integ, varlin, boltzmann, linear_power)
from .particles import Particles, ptcl_enmesh, ptcl_pos, ptcl_rpos, ptcl_rsd, ptcl_los
from .scatter import scatter
from .gather import gather
from .gravity import laplace, neg_grad, gravity
from .modes import white_noise, linear_modes
from .lpt import lpt
from .nbody import nbody

__version__ = '0.1.0'
