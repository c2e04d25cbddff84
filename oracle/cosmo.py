"""NumPy/SciPy restatement of pmwd's configuration and background cosmology
(test infrastructure only).

* ``OConf``            derived fields of pmwd/configuration.py:148-325
* ``E2``, ``H_deriv``, ``Omega_m_a``   pmwd/cosmology.py:185-269
* ``growth_table``     pmwd/boltzmann.py:163-229 -- the reference integrates
  with its own adaptive Dormand-Prince ``odeint`` (ode_util.py); here
  ``scipy.integrate.solve_ivp`` with the Radau method at tight tolerances
  stands in, so the tables agree to the reference's ODE tolerance (~1e-8).
* ``growth``           pmwd/boltzmann.py:232-269
* ``transfer_fit``     pmwd/boltzmann.py:32-123 (Eisenstein & Hu 1998)
* ``linear_power``     pmwd/boltzmann.py:377-455
* ``sigma2_tophat``    replaces mcfit.TophatVar (configuration.py:173-178)
  by direct quadrature.
* ``drift_factor``, ``kick_factor`` pmwd/nbody.py:12-36
"""

import math
from dataclasses import dataclass, field

import numpy as np
from scipy.integrate import solve_ivp


def jax_linspace(start, stop, num, endpoint=True):
    """jnp.linspace in float64: start*(1-t) + stop*t with t = i/div."""
    div = (num - 1) if endpoint else num
    if num == 1:
        return np.array([start], dtype=np.float64)
    t = np.arange(num, dtype=np.float64) / div
    return start * (1 - t) + stop * t


@dataclass
class OConf:
    """Minimal restatement of pmwd.Configuration's fields and derived
    properties (configuration.py:101-325)."""
    ptcl_spacing: float
    ptcl_grid_shape: tuple
    mesh_shape: object = 1
    float_dtype: object = np.float32
    pmid_dtype: object = np.int16
    a_start: float = 1 / 64
    a_stop: float = 1.0
    a_lpt_maxstep: float = 1 / 128
    a_nbody_maxstep: float = 1 / 64
    lpt_order: int = 2
    k_pivot_Mpc: float = 0.05
    T_cmb: float = 2.7255
    transfer_lgk_min: float = -4
    transfer_lgk_max: float = 3
    transfer_lgk_maxstep: float = 1 / 128
    symp_splits: tuple = ((0, 0.5), (1, 0.5))

    M_sun_SI = 1.98847e30
    Mpc_SI = 3.0856775815e22
    H_0_SI = 1e5 / Mpc_SI
    c_SI = 299792458
    G_SI = 6.67430e-11

    def __post_init__(self):
        self.ptcl_grid_shape = tuple(self.ptcl_grid_shape)
        if isinstance(self.mesh_shape, (int, float)):
            self.mesh_shape = tuple(round(s * self.mesh_shape)
                                    for s in self.ptcl_grid_shape)
        self.mesh_shape = tuple(int(s) for s in self.mesh_shape)
        self.float_dtype = np.dtype(self.float_dtype)
        self.pmid_dtype = np.dtype(self.pmid_dtype)
        self.M = 1e10 * self.M_sun_SI
        self.L = self.Mpc_SI
        self.T = 1 / self.H_0_SI

    dim = property(lambda self: len(self.ptcl_grid_shape))
    ptcl_num = property(lambda self: int(np.prod(self.ptcl_grid_shape)))
    mesh_size = property(lambda self: int(np.prod(self.mesh_shape)))
    box_size = property(lambda self: tuple(self.ptcl_spacing * s for s in self.ptcl_grid_shape))
    box_vol = property(lambda self: float(np.prod(self.box_size)))
    ptcl_cell_vol = property(lambda self: self.ptcl_spacing ** self.dim)
    cell_size = property(lambda self: self.ptcl_spacing * self.ptcl_grid_shape[0] / self.mesh_shape[0])
    V = property(lambda self: self.L / self.T)
    H_0 = property(lambda self: self.H_0_SI * self.T)
    c = property(lambda self: self.c_SI / self.V)
    G = property(lambda self: self.G_SI * self.M / (self.L * self.V ** 2))
    rho_crit = property(lambda self: 3 * self.H_0 ** 2 / (8 * np.pi * self.G))

    @property
    def a_nbody_num(self):
        return math.ceil((self.a_stop - self.a_start) / self.a_nbody_maxstep)

    @property
    def a_lpt_num(self):
        return math.ceil(self.a_start / self.a_lpt_maxstep)

    @property
    def a_lpt_step(self):
        return self.a_start / self.a_lpt_num

    @property
    def a_nbody(self):
        return jax_linspace(self.a_start, self.a_stop, 1 + self.a_nbody_num)

    @property
    def a_lpt(self):
        return jax_linspace(0, self.a_start, self.a_lpt_num + 1)

    @property
    def growth_a(self):
        return np.concatenate((self.a_lpt, self.a_nbody[1:]))

    @property
    def transfer_k_num(self):
        return 1 + math.ceil((self.transfer_lgk_max - self.transfer_lgk_min)
                             / self.transfer_lgk_maxstep) + 1

    @property
    def transfer_k(self):
        n = self.transfer_k_num - 1
        lg = jax_linspace(self.transfer_lgk_min, self.transfer_lgk_max, n)
        return np.concatenate(([0.0], 10.0 ** lg))


@dataclass
class OCosmo:
    """Cosmological parameters (cosmology.py:15-182) plus computed tables."""
    A_s_1e9: float
    n_s: float
    Omega_m: float
    Omega_b: float
    h: float
    Omega_k: float = 0.0
    w_0: float = -1.0
    w_a: float = 0.0
    growth: np.ndarray = field(default=None, repr=False)
    transfer: np.ndarray = field(default=None, repr=False)

    Omega_c = property(lambda self: self.Omega_m - self.Omega_b)
    Omega_de = property(lambda self: 1 - (self.Omega_m + self.Omega_k))
    A_s = property(lambda self: self.A_s_1e9 * 1e-9)

    def k_pivot(self, conf):
        return conf.k_pivot_Mpc / (self.h * conf.Mpc_SI) * conf.L


def simple_lcdm(**kw):
    p = dict(A_s_1e9=2.0, n_s=0.96, Omega_m=0.3, Omega_b=0.05, h=0.7)
    p.update(kw)
    return OCosmo(**p)


# --------------------------------------------------------------------------
# background (cosmology.py:185-269)
# --------------------------------------------------------------------------

def E2(a, cosmo):
    a = np.asarray(a, dtype=np.float64)
    de_a = a ** (-3 * (1 + cosmo.w_0 + cosmo.w_a)) * np.exp(-3 * cosmo.w_a * (1 - a))
    return cosmo.Omega_m * a ** -3 + cosmo.Omega_k * a ** -2 + cosmo.Omega_de * de_a


def H_deriv(a, cosmo):
    """dlnH/dlna = a E2'(a) / (2 E2), closed form of the autodiff in
    cosmology.py:222-242."""
    a = np.asarray(a, dtype=np.float64)
    p = -3 * (1 + cosmo.w_0 + cosmo.w_a)
    q = -3 * cosmo.w_a
    de_a = a ** p * np.exp(q * (1 - a))
    a_dE2 = (-3 * cosmo.Omega_m * a ** -3 - 2 * cosmo.Omega_k * a ** -2
             + cosmo.Omega_de * de_a * (p - q * a))
    return 0.5 * a_dE2 / E2(a, cosmo)


def Omega_m_a(a, cosmo):
    a = np.asarray(a, dtype=np.float64)
    return cosmo.Omega_m / (a ** 3 * E2(a, cosmo))


# --------------------------------------------------------------------------
# growth (boltzmann.py:163-269)
# --------------------------------------------------------------------------

def _growth_rhs(lna, G, cosmo):
    a = math.exp(lna)
    dlnH = float(H_deriv(a, cosmo))
    Of = 1.5 * float(Omega_m_a(a, cosmo))
    G1, G1p, G2, G2p = G
    G1pp = -(3 + dlnH - Of) * G1 - (4 + dlnH) * G1p
    G2pp = Of * G1 ** 2 - (8 + 2 * dlnH - Of) * G2 - (6 + dlnH) * G2p
    return np.array([G1p, G1pp, G2p, G2pp])


def growth_table(cosmo, conf, rtol=1e-12, atol=1e-13):
    """(2 orders, 3 derivatives, len(growth_a)) table, boltzmann.py:163-229."""
    eps = np.finfo(np.float64).eps
    a_ic = 0.5 * np.cbrt(eps)
    if a_ic >= conf.a_lpt_step:
        a_ic = 0.1 * conf.a_lpt_step
    a = conf.growth_a.copy()
    a[0] = a_ic
    lna = np.log(a)
    G_ic = np.array([1.0, 0.0, 3 / 7, 0.0])
    sol = solve_ivp(_growth_rhs, (lna[0], lna[-1]), G_ic, method='Radau',
                    t_eval=lna, rtol=rtol, atol=atol, args=(cosmo,))
    G = sol.y.T                                         # (num_a, 4)
    Gd = np.stack([_growth_rhs(t, g, cosmo) for t, g in zip(lna, G)])
    G = G.reshape(-1, 2, 2)
    Gpp = Gd.reshape(-1, 2, 2)[..., 1:]
    G = np.concatenate((G, Gpp), axis=2)                # (num_a, order, 3)
    G = np.moveaxis(G, 0, 2)                            # (order, 3, num_a)
    m = np.array([1.0, 2.0])[:, None]
    table = np.stack((G[:, 0],
                      m * G[:, 0] + G[:, 1],
                      m ** 2 * G[:, 0] + 2 * m * G[:, 1] + G[:, 2]), axis=1)
    return table


def growth(a, cosmo, conf, order=1, deriv=0):
    a = np.asarray(a, dtype=np.float64)
    return a ** order * np.interp(a, conf.growth_a, cosmo.growth[order - 1][deriv])


def with_tables(cosmo, conf):
    cosmo.growth = growth_table(cosmo, conf)
    cosmo.transfer = transfer_fit(conf.transfer_k, cosmo, conf)
    return cosmo


# --------------------------------------------------------------------------
# time-step factors (nbody.py:12-36)
# --------------------------------------------------------------------------

def G_D(a, cosmo, conf):
    return a ** 2 * np.sqrt(E2(a, cosmo)) * growth(a, cosmo, conf, deriv=1)


def G_K(a, cosmo, conf):
    return a ** 3 * E2(a, cosmo) * (growth(a, cosmo, conf, deriv=2)
                                     + (2 + H_deriv(a, cosmo)) * growth(a, cosmo, conf, deriv=1))


def drift_factor(a_vel, a_prev, a_next, cosmo, conf):
    return (growth(a_next, cosmo, conf) - growth(a_prev, cosmo, conf)) / G_D(a_vel, cosmo, conf)


def kick_factor(a_acc, a_prev, a_next, cosmo, conf):
    return (G_D(a_next, cosmo, conf) - G_D(a_prev, cosmo, conf)) / G_K(a_acc, cosmo, conf)


# --------------------------------------------------------------------------
# transfer function and linear power (boltzmann.py:32-123, 377-455)
# --------------------------------------------------------------------------

def transfer_fit(k, cosmo, conf):
    """Eisenstein & Hu (1998) fitting formula with baryon wiggles."""
    k = np.asarray(k, dtype=np.float64) * cosmo.h / conf.L * conf.Mpc_SI
    T2n = (conf.T_cmb / 2.7) ** 2
    h2 = cosmo.h ** 2
    w_m = cosmo.Omega_m * h2
    w_b = cosmo.Omega_b * h2
    f_b = cosmo.Omega_b / cosmo.Omega_m
    f_c = cosmo.Omega_c / cosmo.Omega_m
    z_eq = 2.50e4 * w_m / T2n ** 2
    k_eq = 7.46e-2 * w_m / T2n
    b1 = 0.313 * w_m ** -0.419 * (1 + 0.607 * w_m ** 0.674)
    b2 = 0.238 * w_m ** 0.223
    z_d = 1291 * w_m ** 0.251 / (1 + 0.659 * w_m ** 0.828) * (1 + b1 * w_b ** b2)
    R_d = 31.5 * w_b / T2n ** 2 * (1e3 / z_d)
    R_eq = 31.5 * w_b / T2n ** 2 * (1e3 / z_eq)
    s = (2 / (3 * k_eq) * math.sqrt(6 / R_eq)
         * math.log((math.sqrt(1 + R_d) + math.sqrt(R_eq + R_d)) / (1 + math.sqrt(R_eq))))
    k_silk = 1.6 * w_b ** 0.52 * w_m ** 0.73 * (1 + (10.4 * w_m) ** -0.95)

    a1 = (46.9 * w_m) ** 0.670 * (1 + (32.1 * w_m) ** -0.532)
    a2 = (12.0 * w_m) ** 0.424 * (1 + (45.0 * w_m) ** -0.582)
    alpha_c = a1 ** -f_b * a2 ** -f_b ** 3
    bb1 = 0.944 / (1 + (458 * w_m) ** -0.708)
    bb2 = (0.395 * w_m) ** -0.0266
    beta_c = 1 / (1 + bb1 * (f_c ** bb2 - 1))

    def T0_tilde(k, alpha_c, beta_c):
        q = k / (13.41 * k_eq)
        L = np.log(np.e + 1.8 * beta_c * q)
        C = 14.2 / alpha_c + 386 / (1 + 69.9 * q ** 1.08)
        return L / (L + C * q ** 2)

    f = 1 / (1 + (k * s / 5.4) ** 4)
    T_c = f * T0_tilde(k, 1, beta_c) + (1 - f) * T0_tilde(k, alpha_c, beta_c)
    y = (1 + z_eq) / (1 + z_d)
    x = math.sqrt(1 + y)
    Gy = y * (-6 * x + (2 + 3 * y) * math.log((x + 1) / (x - 1)))
    alpha_b = 2.07 * k_eq * s * (1 + R_d) ** -0.75 * Gy
    beta_node = 8.41 * w_m ** 0.435
    beta_b = 0.5 + f_b + (3 - 2 * f_b) * math.sqrt(1 + (17.2 * w_m) ** 2)
    ks = k * s
    T_b = (T0_tilde(k, 1, 1) / (1 + (ks / 5.2) ** 2)
           + alpha_b * ks ** 3 / (beta_b ** 3 + ks ** 3) * np.exp(-(k / k_silk) ** 1.4)
           ) * np.sinc(ks ** 2 / (np.pi * np.cbrt(beta_node ** 3 + ks ** 3)))
    return f_c * T_c + f_b * T_b


def linear_power(k, a, cosmo, conf):
    """P_lin(k, a) in [L^3], boltzmann.py:399-455."""
    k = np.asarray(k, dtype=np.float64)
    T = np.interp(k, conf.transfer_k, cosmo.transfer)
    kp = cosmo.k_pivot(conf)
    Plin = (0.32 * cosmo.A_s * kp * (k / kp) ** cosmo.n_s
            * (np.pi * (conf.c / conf.H_0) ** 2 / cosmo.Omega_m * T) ** 2)
    if a is not None:
        Plin = Plin * growth(a, cosmo, conf) ** 2
    return Plin


def sigma2_tophat(R, cosmo, conf, a=None):
    """Linear variance in a top-hat sphere of radius R (direct quadrature)."""
    lnk = np.linspace(np.log(1e-5), np.log(1e3), 20001)
    k = np.exp(lnk)
    x = k * R
    W = 3 * (np.sin(x) - x * np.cos(x)) / x ** 3
    P = linear_power(k, a, cosmo, conf)
    integrand = k ** 3 * P * W ** 2 / (2 * np.pi ** 2)
    return np.trapezoid(integrand, lnk)
