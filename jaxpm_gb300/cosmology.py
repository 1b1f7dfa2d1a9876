"""Cosmological parameters, background expansion and the linear matter
power spectrum used to build initial conditions (host-side, float64).

JaxPM takes these from jax_cosmo (``jaxpm/pm.py:2``, ``jaxpm/growth.py:6-9``,
``tests/conftest.py:57-68,90-94``).  This module implements the same
published equations: the Linder dark-energy background
``E^2(a) = Om a^-3 + Ok a^-2 + Ode a^f(a)``, and the Eisenstein & Hu (1998)
transfer function with baryon oscillations normalised to ``sigma8``.
"""
from dataclasses import dataclass

import numpy as np

T_CMB = 2.7255


@dataclass(frozen=True)
class Cosmology:
    """The ``jax_cosmo.Cosmology`` fields used by the PM step."""
    Omega_c: float
    Omega_b: float
    h: float
    n_s: float
    sigma8: float
    Omega_k: float = 0.0
    w0: float = -1.0
    wa: float = 0.0

    @property
    def Omega_m(self):
        return self.Omega_c + self.Omega_b

    @property
    def Omega_de(self):
        return 1.0 - self.Omega_k - self.Omega_m


def Planck15(**kw):
    """Planck 2015 parameters (the cosmology of the benchmark workloads)."""
    p = dict(Omega_c=0.2589, Omega_b=0.0486, h=0.6774, n_s=0.9667, sigma8=0.8159)
    p.update(kw)
    return Cosmology(**p)


def f_de(c, a):
    """Exponent of ``a`` in the dark-energy density (Linder w0-wa)."""
    a = np.asarray(a, dtype=np.float64)
    return -3.0 * (1.0 + c.w0) + 3.0 * c.wa * ((a - 1.0) / np.log(a - 1e-5) - 1.0)


def w(c, a):
    return c.w0 + (1.0 - np.asarray(a, dtype=np.float64)) * c.wa


def Esqr(c, a):
    a = np.asarray(a, dtype=np.float64)
    return c.Omega_m / a**3 + c.Omega_k / a**2 + c.Omega_de * a**f_de(c, a)


def Omega_m_a(c, a):
    return c.Omega_m / np.asarray(a, dtype=np.float64)**3 / Esqr(c, a)


def Omega_de_a(c, a):
    a = np.asarray(a, dtype=np.float64)
    return c.Omega_de * a**f_de(c, a) / Esqr(c, a)


def _transfer_eh(c, k_hmpc):
    """Eisenstein & Hu (1998) transfer function, ``k`` in h/Mpc."""
    k = np.asarray(k_hmpc, dtype=np.float64) * c.h
    theta = T_CMB / 2.7
    om = c.Omega_m * c.h * c.h
    ob = c.Omega_b * c.h * c.h
    fb, fc = c.Omega_b / c.Omega_m, c.Omega_c / c.Omega_m
    zeq = 2.5e4 * om / theta**4
    keq = 7.46e-2 * om / theta**2
    zd = (1291.0 * om**0.251 / (1.0 + 0.659 * om**0.828) *
          (1.0 + 0.313 * om**-0.419 * (1.0 + 0.607 * om**0.674) * ob**(0.238 * om**0.223)))
    rd = 31.5 * ob / theta**4 * (1000.0 / zd)
    req = 31.5 * ob / theta**4 * (1000.0 / zeq)
    sound = (2.0 / (3.0 * keq)) * np.sqrt(6.0 / req) * np.log(
        (np.sqrt(1.0 + rd) + np.sqrt(rd + req)) / (1.0 + np.sqrt(req)))
    ksilk = 1.6 * ob**0.52 * om**0.73 * (1.0 + (10.4 * om)**-0.95)
    alpha_c = ((46.9 * om)**0.670 * (1.0 + (32.1 * om)**-0.532))**(-fb) * \
              ((12.0 * om)**0.424 * (1.0 + (45.0 * om)**-0.582))**(-fb**3)
    beta_c = 1.0 / (1.0 + (0.944 / (1.0 + (458.0 * om)**-0.708)) *
                    (fc**((0.395 * om)**-0.0266) - 1.0))
    q = k / (13.41 * keq)
    ks = k * sound

    def tilde_t0(alpha, beta):
        lg = np.log(np.e + 1.8 * beta * q)
        return lg / (lg + (14.2 / alpha + 386.0 / (1.0 + 69.9 * q**1.08)) * q * q)

    fsup = 1.0 / (1.0 + (ks / 5.4)**4)
    t_cdm = fsup * tilde_t0(1.0, beta_c) + (1.0 - fsup) * tilde_t0(alpha_c, beta_c)
    y = (1.0 + zeq) / (1.0 + zd)
    sy = np.sqrt(1.0 + y)
    gy = y * (-6.0 * sy + (2.0 + 3.0 * y) * np.log((sy + 1.0) / (sy - 1.0)))
    alpha_b = 2.07 * keq * sound * (1.0 + rd)**-0.75 * gy
    beta_node = 8.41 * om**0.435
    beta_b = 0.5 + fb + (3.0 - 2.0 * fb) * np.sqrt((17.2 * om)**2 + 1.0)
    s_tilde = sound / np.cbrt(1.0 + (beta_node / ks)**3)
    t_bar = (tilde_t0(1.0, 1.0) / (1.0 + (ks / 5.2)**2) +
             alpha_b / (1.0 + (beta_b / ks)**3) * np.exp(-(k / ksilk)**1.4)) * \
        np.sinc(k * s_tilde / np.pi)
    return fb * t_bar + fc * t_cdm


def _sigma8_sq_unit(c):
    """sigma^2(R=8 Mpc/h) of the unnormalised spectrum (Simpson in ln k)."""
    lnk = np.linspace(np.log(1e-4), np.log(1e3), 8193)
    k = np.exp(lnk)
    x = 8.0 * k
    wth = 3.0 * (np.sin(x) - x * np.cos(x)) / x**3
    f = k**(3.0 + c.n_s) * _transfer_eh(c, k)**2 * wth**2 / (2.0 * np.pi**2)
    h = lnk[1] - lnk[0]
    return h / 3.0 * (f[0] + f[-1] + 4.0 * f[1:-1:2].sum() + 2.0 * f[2:-1:2].sum())


def linear_matter_power(c, k, a=1.0):
    """Linear matter power spectrum at scale factor ``a``; ``k`` in h/Mpc,
    ``P`` in (Mpc/h)^3."""
    from . import growth
    k = np.asarray(k, dtype=np.float64)
    amp = c.sigma8**2 / _sigma8_sq_unit(c)
    return amp * k**c.n_s * _transfer_eh(c, k)**2 * growth.growth_factor(c, a)**2
