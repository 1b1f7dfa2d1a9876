"""The ODE drop-ins (``jaxpm/ode.py:13-176``) on the GPU against the oracle:
``make_ode_fn`` (``:122-147``), ``make_diffrax_ode`` (``:150-176``),
``symplectic_ode`` (``:85-119``) and the three closures of
``symplectic_fpm_ode`` (``:13-82``), on a 32^3 mesh with particles displaced
from the lattice.  Rates are compared in relative L2 with the float64
oracle at 1e-5 (the force parity bar); a few steps integrated with the
FastPM closures must land where the fused engine's steps do."""
import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import cic, cosmology as oc, fourier as fo, nbody as onb

pytestmark = pytest.mark.gpu

N = 32
TOL = 1e-5


@pytest.fixture(scope="module")
def state(cuda):
    rng = np.random.default_rng(4)
    lat = cic.lattice((N,) * 3).reshape(-1, 3)
    pos = (lat + rng.normal(0, 1.2, lat.shape)).astype(np.float32)
    vel = rng.normal(0, 0.4, lat.shape).astype(np.float32)
    return pos, vel, torch.from_numpy(pos).to(cuda), torch.from_numpy(vel).to(cuda)


def oracle_forces(pos):
    return fo.pm_forces(pos.astype(np.float64), mesh_shape=(N,) * 3, dtype=np.float64)


def test_make_ode_fn_matches_oracle(state):
    from jaxpm_gb300 import cosmology, ode
    pos, vel, x, v = state
    cosmo = cosmology.Planck15()
    f = ode.make_ode_fn((N,) * 3)
    for a in (0.1, 0.5, 1.0):
        dpos, dvel = f((x, v), a, cosmo)
        rp, rv = onb.nbody_ode(oc.Cosmology(), (N,) * 3, (pos.astype(np.float64),
                                                          vel.astype(np.float64)), a,
                               dtype=np.float64)
        assert rel_l2(dpos.cpu(), rp) < TOL
        assert rel_l2(dvel.cpu(), rv) < TOL


def test_make_ode_fn_binned_paint_and_relative_mode(state):
    from jaxpm_gb300 import cosmology, ode
    pos, vel, x, v = state
    cosmo = cosmology.Planck15()
    a = 0.7
    d_atomic = ode.make_ode_fn((N,) * 3)((x, v), a, cosmo)[1]
    d_binned = ode.make_ode_fn((N,) * 3, paint_mode="binned")((x, v), a, cosmo)[1]
    assert rel_l2(d_binned.cpu(), d_atomic.cpu()) < TOL
    # relative mode: the state holds displacements from the lattice
    lat = cic.lattice((N,) * 3).astype(np.float32)
    disp = (pos.reshape(N, N, N, 3) - lat)
    dx = torch.from_numpy(disp).to(x.device)
    dv = torch.from_numpy(vel.reshape(N, N, N, 3)).to(x.device)
    d_rel = ode.make_ode_fn((N,) * 3, paint_absolute_pos=False)((dx, dv), a, cosmo)[1]
    ref = fo.pm_forces(disp.astype(np.float64), paint_absolute_pos=False,
                       mesh_shape=(N,) * 3, dtype=np.float64)
    Ea = np.sqrt(oc.Esqr(oc.Cosmology(), a))
    ref = ref * 1.5 * oc.Cosmology().Omega_m / (a**2 * Ea)
    assert rel_l2(d_rel.cpu(), ref) < TOL


def test_make_diffrax_ode_stacks_the_state(state):
    from jaxpm_gb300 import cosmology, ode
    _, _, x, v = state
    cosmo = cosmology.Planck15()
    # deterministic paint: the two calls' forces are then identical bit for bit
    f = ode.make_ode_fn((N,) * 3, paint_mode="deterministic")
    g = ode.make_diffrax_ode((N,) * 3, paint_mode="deterministic")
    y = torch.stack([x, v])
    out = g(0.4, y, cosmo)
    dpos, dvel = f((x, v), 0.4, cosmo)
    assert out.shape == (2,) + tuple(x.shape)
    assert torch.equal(out[0], dpos) and torch.equal(out[1], dvel)


def test_symplectic_ode_rates(state):
    from jaxpm_gb300 import cosmology, ode
    pos, vel, x, v = state
    cosmo = cosmology.Planck15()
    drift, kick = ode.symplectic_ode((N,) * 3, cosmo)
    c = oc.Cosmology()
    for a in (0.2, 0.9):
        Ea = np.sqrt(oc.Esqr(c, a))
        assert rel_l2(drift(a, v, None).cpu(), vel / (a**3 * Ea)) < TOL
        ref = oracle_forces(pos) * 1.5 * c.Omega_m / (a**2 * Ea)
        assert rel_l2(kick(a, x, None).cpu(), ref) < TOL


def test_symplectic_fpm_closures_match_the_oracle_coefficients(state):
    """drift(a_i) dt0 = drift_i vel, first_kick(a_0) dt0 = kick_0 F and
    kick(a_{i-1}) dt0 = kick_i F, with the oracle's FastPM coefficients
    (``jaxpm/ode.py:20-80`` restated) and its float64 forces."""
    from jaxpm_gb300 import cosmology, ode
    pos, vel, x, v = state
    cosmo = cosmology.Planck15()
    a0, a1, n = 0.1, 1.0, 6
    dt0 = (a1 - a0) / n
    drift, kick, first_kick = ode.symplectic_fpm_ode((N,) * 3, dt0, cosmo)
    kc, dc = onb.fpm_coefficients(oc.Cosmology(), a0, a1, n)
    F = oracle_forces(pos)
    ag = a0 + dt0 * np.arange(n + 1)
    assert rel_l2(first_kick(ag[0], x, None).cpu() * dt0, kc[0] * F) < TOL
    for i in (1, 3, 5):
        assert rel_l2(kick(ag[i - 1], x, None).cpu() * dt0, kc[i] * F) < TOL
        assert rel_l2(drift(ag[i], v, None).cpu() * dt0, dc[i] * vel) < TOL


def test_fpm_closures_integrate_like_the_fused_engine(state):
    """Three steps with the closures (force -> kick -> drift, as the fused
    step) against simulate.FastPM on the same state."""
    from jaxpm_gb300 import cosmology, ode, simulate
    _, _, x, v = state
    cosmo = cosmology.Planck15()
    a0, a1, n = 0.1, 1.0, 3
    dt0 = (a1 - a0) / n
    drift, kick, first_kick = ode.symplectic_fpm_ode((N,) * 3, dt0, cosmo)
    xc, vc = x.clone(), v.clone()
    for i in range(n):
        a = a0 + i * dt0
        vc = vc + dt0 * (first_kick(a, xc, None) if i == 0 else kick(a - dt0, xc, None))
        xc = xc + dt0 * drift(a, vc, None)
    eng = simulate.FastPM((N,) * 3, cosmo, a0, a1, n, device=x.device)
    xe, ve = x.clone(), v.clone()
    eng.run(xe, ve)
    torch.cuda.synchronize()
    assert rel_l2(xc.cpu() - x.cpu(), xe.cpu() - x.cpu()) < 1e-4
    assert rel_l2(vc.cpu(), ve.cpu()) < 1e-4
