"""Growth factors and the FastPM growth functions (host-side scalars).

Mirrors ``jaxpm/growth.py``: ``E``, ``df_de``, ``dEa``, ``Gf``, ``Gf2``,
``dGfa``, ``dGf2a``, ``gp``, ``Dplusdada``, ``Dplus_to_a`` follow
``jaxpm/growth.py:31-334``; ``growth_factor``, ``growth_rate``,
``growth_factor_second``, ``growth_rate_second`` and
``compute_growth_tables`` are the quantities JaxPM imports from jax_cosmo
(``jaxpm/growth.py:6-9``).  They solve the first- and second-order growth
equations in the scale factor,

    D1'' + q D1' - r D1 = 0,   D2'' + q D2' - r D2 = -r D1^2,
    q = (2 - (Om(a) + (1 + 3w) Ode(a)) / 2) / a,   r = 1.5 Om(a) / a^2,

from matter domination at a = 1e-3 (D1 = a, D2 = -3/7 a^2) with a
fixed-step fourth-order Runge-Kutta in ln a (16 sub-steps per table
interval), tabulated on ``logspace(-3, 0, 128)`` and normalised to 1 at
a = 1.  The table tuple is ``(a, g, f, h, g2, f2, h2)`` with
``f = dlnD/dlna`` and ``h = a D''/D``.  Lookups interpolate linearly in a.
Everything here is float64 host arithmetic: these are per-step scalars.
"""
import math

import numpy as np

from .cosmology import Esqr, Omega_de_a, Omega_m_a, f_de, w

__all__ = [
    "growth_factor", "growth_rate", "growth_factor_second", "growth_rate_second",
    "E", "df_de", "dEa", "Gf", "Gf2", "dGfa", "dGf2a", "gp", "Dplusdada", "Dplus_to_a",
    "compute_growth_tables", "Esqr",
]

_CACHE = {}


def _rhs(c, a, y):
    d1, v1, d2, v2 = y
    om = Omega_m_a(c, a)
    q = (2.0 - 0.5 * (om + (1.0 + 3.0 * w(c, a)) * Omega_de_a(c, a))) / a
    r = 1.5 * om / (a * a)
    return np.array([v1, r * d1 - q * v1, v2, r * d2 - q * v2 - r * d1 * d1])


def _rhs_lna(c, lna, y):
    """``a * _rhs(c, a, y)`` at ``a = exp(lna)`` in plain float arithmetic
    (the same formulas as ``_rhs`` and the background functions; the RK4
    loop calls it 8192 times per table)."""
    a = math.exp(lna)
    d1, v1, d2, v2 = y
    fde = -3.0 * (1.0 + c.w0) + 3.0 * c.wa * ((a - 1.0) / math.log(a - 1e-5) - 1.0)
    esq = c.Omega_m / a**3 + c.Omega_k / a**2 + c.Omega_de * a**fde
    om = c.Omega_m / a**3 / esq
    ode = c.Omega_de * a**fde / esq
    q = (2.0 - 0.5 * (om + (1.0 + 3.0 * (c.w0 + (1.0 - a) * c.wa)) * ode)) / a
    r = 1.5 * om / (a * a)
    return (a * v1, a * (r * d1 - q * v1), a * v2, a * (r * d2 - q * v2 - r * d1 * d1))


def compute_growth_tables(c):
    """``(a, g, f, h, g2, f2, h2)`` on ``logspace(-3, 0, 128)`` (cached per
    cosmology)."""
    hit = _CACHE.get(c)
    if hit is not None:
        return hit
    atab = np.logspace(-3.0, 0.0, 128)
    sub = 16
    y = (float(atab[0]), 1.0, -3.0 / 7.0 * float(atab[0])**2, -6.0 / 7.0 * float(atab[0]))
    ys = [y]
    for i in range(len(atab) - 1):
        la, lb = math.log(atab[i]), math.log(atab[i + 1])
        hstep = (lb - la) / sub
        lna = la
        for _ in range(sub):
            k1 = _rhs_lna(c, lna, y)
            k2 = _rhs_lna(c, lna + hstep / 2, tuple(u + hstep / 2 * k for u, k in zip(y, k1)))
            k3 = _rhs_lna(c, lna + hstep / 2, tuple(u + hstep / 2 * k for u, k in zip(y, k2)))
            k4 = _rhs_lna(c, lna + hstep, tuple(u + hstep * k for u, k in zip(y, k3)))
            y = tuple(u + hstep / 6.0 * (p1 + 2 * p2 + 2 * p3 + p4)
                      for u, p1, p2, p3, p4 in zip(y, k1, k2, k3, k4))
            lna += hstep
        ys.append(y)
    ys = np.array(ys)
    dys = np.array([_rhs(c, a, yy) for a, yy in zip(atab, ys)])
    d1n, d2n = ys[-1, 0], ys[-1, 2]
    g = ys[:, 0] / d1n
    g2 = ys[:, 2] / d2n
    out = (atab, g, ys[:, 1] / d1n * atab / g, dys[:, 1] / d1n * atab / g,
           g2, ys[:, 3] / d2n * atab / g2, dys[:, 3] / d2n * atab / g2)
    _CACHE[c] = out
    return out


def growth_factor(c, a):
    t = compute_growth_tables(c)
    return np.clip(np.interp(a, t[0], t[1]), 0.0, 1.0)


def growth_rate(c, a):
    t = compute_growth_tables(c)
    return np.interp(a, t[0], t[2])


def growth_factor_second(c, a):
    t = compute_growth_tables(c)
    return np.interp(a, t[0], t[4])


def growth_rate_second(c, a):
    t = compute_growth_tables(c)
    return np.interp(a, t[0], t[5])


def E(c, a):
    """``E(a) = sqrt(E^2(a))`` (``jaxpm/growth.py:31-52``)."""
    return np.sqrt(Esqr(c, a))


def df_de(c, a, epsilon=1e-5):
    """``jaxpm/growth.py:55-85``."""
    a = np.asarray(a, dtype=np.float64)
    la = np.log(a - epsilon)
    return 3 * c.wa * (la - (a - 1) / (a - epsilon)) / (la * la)


def dEa(c, a):
    """``dE/da`` (``jaxpm/growth.py:88-121``)."""
    a = np.asarray(a, dtype=np.float64)
    num = (-3 * c.Omega_m / a**4 - 2 * c.Omega_k / a**3 +
           df_de(c, a) * c.Omega_de * np.exp(f_de(c, a)))
    return 0.5 * num / E(c, a)


def gp(c, a):
    """``dD1/da = f1 D1 / a`` (``jaxpm/growth.py:264-293``)."""
    a = np.asarray(a, dtype=np.float64)
    return growth_rate(c, a) * growth_factor(c, a) / a


def Gf(c, a):
    """``D1' a^3 E`` (``jaxpm/growth.py:124-154``)."""
    a = np.asarray(a, dtype=np.float64)
    return gp(c, a) * a**3 * E(c, a)


def Gf2(c, a):
    """``D2' a^3 E`` (``jaxpm/growth.py:157-187``)."""
    a = np.asarray(a, dtype=np.float64)
    return growth_rate_second(c, a) * growth_factor_second(c, a) / a * a**3 * E(c, a)


def _dG(c, a, second):
    a = np.asarray(a, dtype=np.float64)
    t = compute_growth_tables(c)
    if second:
        dfa = growth_rate_second(c, a) * growth_factor_second(c, a) / a
        dd = np.interp(np.log(a), np.log(t[0]), t[6] / t[0] * t[4])
    else:
        dfa = gp(c, a)
        dd = np.interp(np.log(a), np.log(t[0]), t[3] / t[0] * t[1])
    e = E(c, a)
    return dd * a**3 * e + dfa * a**3 * dEa(c, a) + 3 * a**2 * e * dfa


def dGfa(c, a):
    """``dGf/da`` (``jaxpm/growth.py:190-224``)."""
    return _dG(c, a, False)


def dGf2a(c, a):
    """``dGf2/da`` (``jaxpm/growth.py:227-261``)."""
    return _dG(c, a, True)


def Dplusdada(c, a):
    """``d^2 D1/da^2`` (``jaxpm/growth.py:296-314``)."""
    t = compute_growth_tables(c)
    return np.interp(np.log(np.atleast_1d(a)), np.log(t[0]), t[3] * t[1] / t[0])


def Dplus_to_a(c, D):
    """Inverse growth factor (``jaxpm/growth.py:317-334``)."""
    t = compute_growth_tables(c)
    return np.interp(np.atleast_1d(D), t[1], t[0])
