"""ODE right-hand sides and the FastPM leapfrog, with jaxpm's call surface
(``jaxpm/ode.py``).

``make_ode_fn`` (``:122-147``), ``make_diffrax_ode`` (``:150-176``),
``symplectic_ode`` (``:85-119``) and ``symplectic_fpm_ode`` (``:13-82``)
return functions with the reference's arguments and results, built on the
GPU ``pm_forces``.  ``fpm_coefficients`` folds the FastPM kick and drift
factors into one pair of scalars per step, for the fused step kernel
(``simulate.FastPM``): step ``i`` computes forces at ``pos_i``, kicks the
velocities (the first kick is the half kick of ``first_kick``, later ones
the full kicks of ``kick``) and drifts the positions from ``a_i`` to
``a_{i+1}``.
"""
import numpy as np
import torch

from . import growth as gr
from .painting import _single_device
from .pm import pm_forces


def _E(cosmo, a):
    return float(np.sqrt(gr.Esqr(cosmo, a)))


def make_ode_fn(mesh_shape, paint_absolute_pos=True, halo_size=0, sharding=None,
                paint_mode="atomic"):
    """``nbody_ode(state, a, cosmo) -> (dpos, dvel)`` with
    ``dpos = vel / (a^3 E)`` and ``dvel = 1.5 Omega_m F / (a^2 E)``."""
    _single_device(halo_size, sharding)

    def nbody_ode(state, a, cosmo):
        pos, vel = state
        forces = pm_forces(pos, mesh_shape=mesh_shape, paint_absolute_pos=paint_absolute_pos,
                           paint_mode=paint_mode) * (1.5 * cosmo.Omega_m)
        a = float(a)
        e = _E(cosmo, a)
        dpos = (1.0 / (a**3 * e)) * vel
        dvel = (1.0 / (a**2 * e)) * forces
        return dpos, dvel

    return nbody_ode


def make_diffrax_ode(mesh_shape, paint_absolute_pos=True, halo_size=0, sharding=None,
                     paint_mode="atomic"):
    """``nbody_ode(a, state, args) -> stack([dpos, dvel])`` (the stacked
    state layout of diffrax users)."""
    f = make_ode_fn(mesh_shape, paint_absolute_pos, halo_size, sharding, paint_mode)

    def nbody_ode(a, state, args):
        dpos, dvel = f((state[0], state[1]), a, args)
        return torch.stack([dpos, dvel])

    return nbody_ode


def symplectic_ode(mesh_shape, cosmo, paint_absolute_pos=True, halo_size=0, sharding=None,
                   paint_mode="atomic"):
    """``(drift, kick)`` rates of the plain symplectic scheme."""
    _single_device(halo_size, sharding)

    def drift(a, vel, args):
        return (1.0 / (float(a)**3 * _E(cosmo, float(a)))) * vel

    def kick(a, pos, args):
        forces = pm_forces(pos, mesh_shape=mesh_shape, paint_absolute_pos=paint_absolute_pos,
                           paint_mode=paint_mode) * (1.5 * cosmo.Omega_m)
        return (1.0 / (float(a)**2 * _E(cosmo, float(a)))) * forces

    return drift, kick


def symplectic_fpm_ode(mesh_shape, dt0, cosmo, paint_absolute_pos=True, halo_size=0,
                       sharding=None, paint_mode="atomic"):
    """``(drift, kick, first_kick)`` of the FastPM scheme: each returns a rate
    that a fixed-step stepper multiplies by ``dt0``."""
    _single_device(halo_size, sharding)

    def forces(pos):
        return pm_forces(pos, mesh_shape=mesh_shape, paint_absolute_pos=paint_absolute_pos,
                         paint_mode=paint_mode) * (1.5 * cosmo.Omega_m)

    def drift(a, vel, args):
        a = float(a)
        ai, af = a, a + dt0
        ac = (ai * af)**0.5
        contr = (gr.growth_factor(cosmo, af) - gr.growth_factor(cosmo, ai)) / gr.gp(cosmo, ac)
        return (float(contr) / dt0 / (ac**3 * _E(cosmo, ac))) * vel

    def kick(a, pos, args):
        t0 = float(a)
        t1, t2 = t0 + dt0, t0 + 2 * dt0
        t0t1, t1t2 = (t0 * t1)**0.5, (t1 * t2)**0.5
        k1 = (gr.Gf(cosmo, t1) - gr.Gf(cosmo, t0t1)) / gr.dGfa(cosmo, t1)
        k2 = (gr.Gf(cosmo, t1t2) - gr.Gf(cosmo, t1)) / gr.dGfa(cosmo, t1)
        return (float(k1 + k2) / dt0 / (t1**2 * _E(cosmo, t1))) * forces(pos)

    def first_kick(a, pos, args):
        t0 = float(a)
        t0t1 = (t0 * (t0 + dt0))**0.5
        kf = (gr.Gf(cosmo, t0t1) - gr.Gf(cosmo, t0)) / gr.dGfa(cosmo, t0)
        return (float(kf) / dt0 / (t0**2 * _E(cosmo, t0))) * forces(pos)

    return drift, kick, first_kick


def fpm_coefficients(cosmo, a0, a1, n_steps):
    """Per-step ``(kick, drift)`` scalars (float64 arrays of length
    ``n_steps``) of the fused FastPM step on ``a_i = a0 + i (a1-a0)/n``:
    ``kick`` includes ``1.5 Omega_m`` and the growth-factor kick factor of
    ``jaxpm/ode.py:35-80`` times ``dt``; ``drift`` the drift factor of
    ``jaxpm/ode.py:20-33`` times ``dt``."""
    dt = (a1 - a0) / n_steps
    ag = a0 + dt * np.arange(n_steps + 1)
    c = cosmo
    kick = np.empty(n_steps)
    drift = np.empty(n_steps)
    for i in range(n_steps):
        if i == 0:
            t0 = ag[0]
            t0t1 = np.sqrt(t0 * ag[1])
            kf = (gr.Gf(c, t0t1) - gr.Gf(c, t0)) / gr.dGfa(c, t0)
            kick[i] = 1.5 * c.Omega_m / (t0**2 * gr.E(c, t0)) * kf
        else:
            t0, t1, t2 = ag[i - 1], ag[i], ag[i + 1]
            t0t1, t1t2 = np.sqrt(t0 * t1), np.sqrt(t1 * t2)
            kf = ((gr.Gf(c, t1) - gr.Gf(c, t0t1)) + (gr.Gf(c, t1t2) - gr.Gf(c, t1))) / gr.dGfa(c, t1)
            kick[i] = 1.5 * c.Omega_m / (t1**2 * gr.E(c, t1)) * kf
        ai, af = ag[i], ag[i + 1]
        ac = np.sqrt(ai * af)
        drift[i] = ((gr.growth_factor(c, af) - gr.growth_factor(c, ai)) / gr.gp(c, ac) /
                    (ac**3 * gr.E(c, ac)))
    return kick, drift
