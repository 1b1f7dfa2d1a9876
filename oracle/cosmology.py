"""Background, growth and linear power spectrum in float64 NumPy/SciPy
(test infrastructure only).

JaxPM imports ``Esqr``, ``growth_factor``, ``growth_rate``,
``growth_factor_second``, ``growth_rate_second``, ``_compute_growth_tables``
and ``linear_matter_power`` from jax_cosmo (``jaxpm/growth.py:6-9``,
``jaxpm/pm.py:2,78``, ``tests/conftest.py:91``); jax_cosmo is not in the
reference tree and cannot be imported here, so its published equations are
restated:

* ``Esqr(a) = Om a^-3 + Ok a^-2 + Ode a^f(a)``, with the Linder dark-energy
  exponent ``f(a) = -3(1+w0) + 3 wa ((a-1)/ln(a-1e-5) - 1)``.
* Growth ODEs in the scale factor for D1 and D2,
  ``D'' + q D' - r D = 0`` and ``D2'' + q D2' - r D2 = -r D1^2`` with
  ``q = (2 - (Om(a) + (1+3w) Ode(a))/2)/a`` and ``r = 1.5 Om(a)/a^2``,
  started in matter domination at ``a = 1e-3`` (``D1 = a``,
  ``D2 = -3/7 a^2``), tabulated on ``logspace(-3, 0, 128)`` and normalised
  to 1 at ``a = 1`` (table layout of ``_compute_growth_tables``:
  ``(a, g, f, h, g2, f2, h2)`` with ``f = dlnD/dlna`` and
  ``h = a D''/D``).  This oracle integrates with SciPy's DOP853 at tight
  tolerance; lookups are linear interpolation in ``a``.
* Eisenstein & Hu (1998, ApJ 496, 605) transfer function with baryon
  oscillations, ``P(k) = A k^ns T(k)^2 D(a)^2`` normalised to ``sigma8``
  with a top-hat window of radius 8 Mpc/h.

JaxPM's own formulas (``E``, ``dEa``, ``Gf``, ``Gf2``, ``dGfa``,
``dGf2a``, ``gp``) follow ``jaxpm/growth.py:31-293`` directly.
"""
from dataclasses import dataclass

import numpy as np
from scipy.integrate import solve_ivp

T_CMB = 2.7255


@dataclass(frozen=True)
class Cosmology:
    """Parameters of ``jax_cosmo.Cosmology`` used by the hot path."""
    Omega_c: float = 0.2589
    Omega_b: float = 0.0486
    h: float = 0.6774
    n_s: float = 0.9667
    sigma8: float = 0.8159
    Omega_k: float = 0.0
    w0: float = -1.0
    wa: float = 0.0

    @property
    def Omega_m(self):
        return self.Omega_c + self.Omega_b

    @property
    def Omega_de(self):
        return 1.0 - self.Omega_k - self.Omega_m


def f_de(c, a):
    a = np.asarray(a, dtype=np.float64)
    return -3.0 * (1.0 + c.w0) + 3.0 * c.wa * ((a - 1.0) / np.log(a - 1e-5) - 1.0)


def w(c, a):
    return c.w0 + (1.0 - np.asarray(a, dtype=np.float64)) * c.wa


def Esqr(c, a):
    a = np.asarray(a, dtype=np.float64)
    return (c.Omega_m * a**-3 + c.Omega_k * a**-2 +
            c.Omega_de * np.power(a, f_de(c, a)))


def Omega_m_a(c, a):
    a = np.asarray(a, dtype=np.float64)
    return c.Omega_m * a**-3 / Esqr(c, a)


def Omega_de_a(c, a):
    a = np.asarray(a, dtype=np.float64)
    return c.Omega_de * np.power(a, f_de(c, a)) / Esqr(c, a)


def _growth_rhs(c, a, y):
    d1, d1p, d2, d2p = y
    q = (2.0 - 0.5 * (Omega_m_a(c, a) + (1.0 + 3.0 * w(c, a)) * Omega_de_a(c, a))) / a
    r = 1.5 * Omega_m_a(c, a) / a / a
    return np.array([d1p, -q * d1p + r * d1, d2p, -q * d2p + r * d2 - r * d1 * d1])


_TABLES = {}


def growth_tables(c):
    """``_compute_growth_tables``: ``(a, g, f, h, g2, f2, h2)`` on
    ``logspace(-3, 0, 128)``."""
    if c in _TABLES:
        return _TABLES[c]
    atab = np.logspace(-3, 0, 128)
    a0 = atab[0]
    y0 = [a0, 1.0, -3.0 / 7.0 * a0**2, -6.0 / 7.0 * a0]
    sol = solve_ivp(lambda a, y: _growth_rhs(c, a, y), (a0, 1.0), y0,
                    t_eval=atab, method='DOP853', rtol=1e-12, atol=1e-14)
    y = sol.y
    dy = np.stack([_growth_rhs(c, a, y[:, i]) for i, a in enumerate(atab)], 1)
    g = y[0] / y[0, -1]
    f = y[1] / y[0, -1] * atab / g
    h = dy[1] / y[0, -1] * atab / g
    g2 = y[2] / y[2, -1]
    f2 = y[3] / y[2, -1] * atab / g2
    h2 = dy[3] / y[2, -1] * atab / g2
    out = (atab, g, f, h, g2, f2, h2)
    _TABLES[c] = out
    return out


def growth_factor(c, a):
    t = growth_tables(c)
    return np.clip(np.interp(a, t[0], t[1]), 0.0, 1.0)


def growth_rate(c, a):
    t = growth_tables(c)
    return np.interp(a, t[0], t[2])


def growth_factor_second(c, a):
    t = growth_tables(c)
    return np.interp(a, t[0], t[4])


def growth_rate_second(c, a):
    t = growth_tables(c)
    return np.interp(a, t[0], t[5])


def E(c, a):
    """``jaxpm/growth.py:31-52``."""
    return np.sqrt(Esqr(c, a))


def df_de(c, a, epsilon=1e-5):
    """``jaxpm/growth.py:55-85``."""
    a = np.asarray(a, dtype=np.float64)
    return (3 * c.wa * (np.log(a - epsilon) - (a - 1) / (a - epsilon)) /
            np.power(np.log(a - epsilon), 2))


def dEa(c, a):
    """``jaxpm/growth.py:88-121``."""
    a = np.asarray(a, dtype=np.float64)
    return (0.5 * (-3 * c.Omega_m * a**-4 - 2 * c.Omega_k * a**-3 +
                   df_de(c, a) * c.Omega_de * np.exp(f_de(c, a))) / E(c, a))


def Gf(c, a):
    """``jaxpm/growth.py:124-154``."""
    a = np.asarray(a, dtype=np.float64)
    return growth_rate(c, a) * growth_factor(c, a) / a * a**3 * E(c, a)


def Gf2(c, a):
    """``jaxpm/growth.py:157-187``."""
    a = np.asarray(a, dtype=np.float64)
    return growth_rate_second(c, a) * growth_factor_second(c, a) / a * a**3 * E(c, a)


def dGfa(c, a):
    """``jaxpm/growth.py:190-224``."""
    a = np.asarray(a, dtype=np.float64)
    d1f = growth_rate(c, a) * growth_factor(c, a) / a
    t = growth_tables(c)
    f1p = np.interp(np.log(a), np.log(t[0]), t[3] / t[0] * t[1])
    Ea = E(c, a)
    return f1p * a**3 * Ea + d1f * a**3 * dEa(c, a) + 3 * a**2 * Ea * d1f


def dGf2a(c, a):
    """``jaxpm/growth.py:227-261``."""
    a = np.asarray(a, dtype=np.float64)
    d2f = growth_rate_second(c, a) * growth_factor_second(c, a) / a
    t = growth_tables(c)
    f2p = np.interp(np.log(a), np.log(t[0]), t[6] / t[0] * t[4])
    Ea = E(c, a)
    return f2p * a**3 * Ea + d2f * a**3 * dEa(c, a) + 3 * a**2 * Ea * d2f


def gp(c, a):
    """``jaxpm/growth.py:264-293``."""
    a = np.asarray(a, dtype=np.float64)
    return growth_rate(c, a) * growth_factor(c, a) / a


# --------------------------------------------------------------------------
# Linear matter power spectrum
# --------------------------------------------------------------------------


def eisenstein_hu(c, k):
    """Eisenstein & Hu (1998) transfer function with baryon wiggles;
    ``k`` in h/Mpc."""
    k = np.asarray(k, dtype=np.float64) * c.h  # 1/Mpc
    th = T_CMB / 2.7
    omh2 = c.Omega_m * c.h**2
    obh2 = c.Omega_b * c.h**2
    fb = c.Omega_b / c.Omega_m
    fc = c.Omega_c / c.Omega_m
    z_eq = 2.50e4 * omh2 * th**-4
    k_eq = 7.46e-2 * omh2 * th**-2
    b1 = 0.313 * omh2**-0.419 * (1 + 0.607 * omh2**0.674)
    b2 = 0.238 * omh2**0.223
    z_d = 1291 * omh2**0.251 / (1 + 0.659 * omh2**0.828) * (1 + b1 * obh2**b2)
    R = lambda z: 31.5 * obh2 * th**-4 * (1000.0 / z)
    R_d, R_eq = R(z_d), R(z_eq)
    s = (2.0 / (3.0 * k_eq) * np.sqrt(6.0 / R_eq) *
         np.log((np.sqrt(1 + R_d) + np.sqrt(R_d + R_eq)) / (1 + np.sqrt(R_eq))))
    k_silk = 1.6 * obh2**0.52 * omh2**0.73 * (1 + (10.4 * omh2)**-0.95)
    a1 = (46.9 * omh2)**0.670 * (1 + (32.1 * omh2)**-0.532)
    a2 = (12.0 * omh2)**0.424 * (1 + (45.0 * omh2)**-0.582)
    alpha_c = a1**(-fb) * a2**(-fb**3)
    bb1 = 0.944 / (1 + (458 * omh2)**-0.708)
    bb2 = (0.395 * omh2)**-0.0266
    beta_c = 1.0 / (1 + bb1 * (fc**bb2 - 1))
    q = k / (13.41 * k_eq)

    def T0(alpha, beta):
        L = np.log(np.e + 1.8 * beta * q)
        C = 14.2 / alpha + 386.0 / (1 + 69.9 * q**1.08)
        return L / (L + C * q * q)

    ks = k * s
    f = 1.0 / (1 + (ks / 5.4)**4)
    Tc = f * T0(1.0, beta_c) + (1 - f) * T0(alpha_c, beta_c)
    y = (1 + z_eq) / (1 + z_d)
    Gy = y * (-6 * np.sqrt(1 + y) + (2 + 3 * y) *
              np.log((np.sqrt(1 + y) + 1) / (np.sqrt(1 + y) - 1)))
    alpha_b = 2.07 * k_eq * s * (1 + R_d)**-0.75 * Gy
    beta_node = 8.41 * omh2**0.435
    beta_b = 0.5 + fb + (3 - 2 * fb) * np.sqrt((17.2 * omh2)**2 + 1)
    s_t = s / (1 + (beta_node / ks)**3)**(1.0 / 3.0)
    x = k * s_t
    j0 = np.sinc(x / np.pi)
    Tb = (T0(1.0, 1.0) / (1 + (ks / 5.2)**2) +
          alpha_b / (1 + (beta_b / ks)**3) * np.exp(-(k / k_silk)**1.4)) * j0
    return fb * Tb + fc * Tc


def _sigma_sqr_unnorm(c, R=8.0):
    lk = np.linspace(np.log(1e-4), np.log(1e3), 8193)
    k = np.exp(lk)
    x = k * R
    W = 3 * (np.sin(x) - x * np.cos(x)) / x**3
    integrand = k**3 * k**c.n_s * eisenstein_hu(c, k)**2 * W**2 / (2 * np.pi**2)
    dl = lk[1] - lk[0]
    return dl / 3 * (integrand[0] + integrand[-1] + 4 * integrand[1:-1:2].sum() +
                     2 * integrand[2:-1:2].sum())


def linear_matter_power(c, k, a=1.0):
    """``jax_cosmo.power.linear_matter_power`` restated; ``k`` in h/Mpc,
    ``P`` in (Mpc/h)^3."""
    k = np.asarray(k, dtype=np.float64)
    norm = c.sigma8**2 / _sigma_sqr_unnorm(c)
    return norm * k**c.n_s * eisenstein_hu(c, k)**2 * growth_factor(c, a)**2
