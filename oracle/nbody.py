"""Initial conditions, LPT and the FastPM leapfrog, restated in NumPy
(test infrastructure only).

Follows ``jaxpm/pm.py:61-144`` (``lpt``, ``linear_field``) and
``jaxpm/ode.py:13-82`` (``symplectic_fpm_ode``) and ``:122-147``
(``make_ode_fn``).
"""
import numpy as np

from . import cic, cosmology as cm, fourier as fo


def linear_field(noise, box_size, pk_k, pk_p, dtype=np.float32):
    """``linear_field`` (``jaxpm/pm.py:129-144``) with the white noise given
    as an input (so both sides use the same field) and ``pk`` the linear
    interpolation of the table ``(pk_k, pk_p)`` used by the reference tests
    (``tests/conftest.py:90-94``)."""
    shape = noise.shape
    field = fo.fft3d(np.asarray(noise, dtype))
    kvec = fo.fftk(shape, dtype)
    kmesh = sum((kk / box_size[i] * shape[i])**2 for i, kk in enumerate(kvec))**0.5
    pkmesh = (np.interp(kmesh, pk_k, pk_p).astype(dtype) *
              dtype(shape[0] * shape[1] * shape[2]) /
              dtype(box_size[0] * box_size[1] * box_size[2]))
    field = field * np.sqrt(pkmesh)
    return fo.ifft3d(field).astype(dtype)


def lpt(cosmo, initial_conditions, particles=None, a=0.1, order=1,
        dtype=np.float32):
    """``lpt`` (``jaxpm/pm.py:61-126``) on one device."""
    ic = np.asarray(initial_conditions, dtype)
    absolute = particles is not None
    if particles is None:
        particles = np.zeros((*ic.shape, 3), dtype)
    a = np.atleast_1d(a).astype(np.float64)
    E = np.sqrt(cm.Esqr(cosmo, a))
    delta_k = fo.fft3d(ic)
    f1 = fo.pm_forces(particles, delta=delta_k, paint_absolute_pos=absolute,
                      dtype=dtype)
    dx = (cm.growth_factor(cosmo, a) * f1).astype(dtype)
    p = (a**2 * cm.growth_rate(cosmo, a) * E * dx).astype(dtype)
    f = (a**2 * E * cm.dGfa(cosmo, a) * f1).astype(dtype)
    if order == 2:
        delta2 = source_2lpt(delta_k, dtype)
        f2 = fo.pm_forces(particles, delta=fo.fft3d(delta2),
                          paint_absolute_pos=absolute, dtype=dtype)
        dx2 = (3 / 7 * cm.growth_factor_second(cosmo, a) * f2).astype(dtype)
        p2 = (a**2 * cm.growth_rate_second(cosmo, a) * E * dx2).astype(dtype)
        ff2 = (a**2 * E * cm.dGf2a(cosmo, a) * f2).astype(dtype)
        dx = dx + dx2
        p = p + p2
        f = f + ff2
    return dx, p, f


def source_2lpt(delta_k, dtype=np.float32):
    """Second-order source ``sum_{i<j} (phi_ii phi_jj - phi_ij^2)``
    (``jaxpm/pm.py:88-109``)."""
    kvec = fo.fftk(delta_k.shape, dtype)
    pot_k = delta_k * fo.invlaplace_kernel(kvec)
    delta2 = 0
    shear_acc = 0
    for i in range(3):
        shear_ii = fo.ifft3d(fo.gradient_kernel(kvec, i)**2 * pot_k)
        delta2 = delta2 + shear_ii * shear_acc
        shear_acc = shear_acc + shear_ii
        for j in range(i + 1, 3):
            nij = fo.gradient_kernel(kvec, i) * fo.gradient_kernel(kvec, j)
            delta2 = delta2 - fo.ifft3d(nij * pot_k)**2
    return np.asarray(delta2, dtype)


def fpm_coefficients(cosmo, a0, a1, n_steps):
    """Kick and drift coefficients of the FastPM leapfrog, one pair per
    fused step ``force(pos_i) -> kick -> drift``.

    ``jaxpm/ode.py:60-80`` (first half kick), ``:35-58`` (full kicks between
    half-step times, forces times ``1.5 Omega_m``) and ``:20-33`` (drifts),
    on the grid ``a_i = a0 + i*dt``.  The reference's stepper multiplies
    each returned rate by ``dt0``; the coefficients here are those products.
    The last full kick (which would reach past ``a1``) is not part of a step.
    """
    dt = (a1 - a0) / n_steps
    ag = a0 + dt * np.arange(n_steps + 1)
    c = cosmo
    kick, drift = [], []
    for i in range(n_steps):
        if i == 0:
            t0 = ag[0]
            t0t1 = np.sqrt(t0 * ag[1])
            kf = (cm.Gf(c, t0t1) - cm.Gf(c, t0)) / cm.dGfa(c, t0)
            kc = 1.5 * c.Omega_m / (t0**2 * cm.E(c, t0)) * kf
        else:
            t0, t1, t2 = ag[i - 1], ag[i], ag[i + 1]
            t0t1, t1t2 = np.sqrt(t0 * t1), np.sqrt(t1 * t2)
            k1 = (cm.Gf(c, t1) - cm.Gf(c, t0t1)) / cm.dGfa(c, t1)
            k2 = (cm.Gf(c, t1t2) - cm.Gf(c, t1)) / cm.dGfa(c, t1)
            kc = 1.5 * c.Omega_m / (t1**2 * cm.E(c, t1)) * (k1 + k2)
        ai, af = ag[i], ag[i + 1]
        ac = np.sqrt(ai * af)
        dc = ((cm.growth_factor(c, af) - cm.growth_factor(c, ai)) /
              cm.gp(c, ac) / (ac**3 * cm.E(c, ac)))
        kick.append(float(kc))
        drift.append(float(dc))
    return np.array(kick), np.array(drift)


def fpm_step(pos, vel, mesh_shape, kick_c, drift_c, dtype=np.float32):
    """One fused FastPM step: forces at ``pos``, ``vel += kick_c * F``,
    ``pos += drift_c * vel``."""
    F = fo.pm_forces(pos, mesh_shape=mesh_shape, dtype=dtype)
    vel = (vel + dtype(kick_c) * F).astype(dtype)
    pos = (pos + dtype(drift_c) * vel).astype(dtype)
    return pos, vel


def fpm_run_vjp(pos, vel, mesh_shape, kicks, drifts, g_pos, g_vel, r_split=0.0):
    """Float64 forward run of FastPM steps (``fpm_step`` with the given
    per-step coefficients) and its reverse sweep, the transpose that
    ``jax.grad`` takes through ``jaxpm/ode.py:13-82``: per step, from the
    output cotangents, ``u = g_vel + drift g_pos``,
    ``g_pos += (dF/dx)^T (kick u)`` at the step's starting positions,
    ``g_vel = u``.  Returns ``((pos, vel), (g_pos0, g_vel0))``."""
    x = np.asarray(pos, dtype=np.float64)
    v = np.asarray(vel, dtype=np.float64)
    starts = []
    for k, d in zip(kicks, drifts):
        starts.append(x)
        F = fo.pm_forces(x, mesh_shape=mesh_shape, r_split=r_split, dtype=np.float64)
        v = v + k * F
        x = x + d * v
    gx = np.asarray(g_pos, dtype=np.float64)
    gv = np.asarray(g_vel, dtype=np.float64)
    for i in reversed(range(len(starts))):
        u = gv + drifts[i] * gx
        gx = gx + fo.pm_forces_vjp(starts[i], mesh_shape, kicks[i] * u, r_split=r_split)
        gv = u
    return (x, v), (gx, gv)


def nbody_ode(cosmo, mesh_shape, state, a, dtype=np.float32):
    """``make_ode_fn(...)(state, a, cosmo)`` (``jaxpm/ode.py:122-147``)."""
    pos, vel = state
    F = fo.pm_forces(pos, mesh_shape=mesh_shape, dtype=dtype) * dtype(1.5 * cosmo.Omega_m)
    Ea = np.sqrt(cm.Esqr(cosmo, a))
    dpos = (1.0 / (a**3 * Ea)) * vel
    dvel = (1.0 / (a**2 * Ea)) * F
    return dpos.astype(dtype), dvel.astype(dtype)
