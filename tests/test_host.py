"""Host-side logic of the product, checked against the oracle on the CPU:
growth scalars, FastPM coefficients, the jaxpm-compatible argument checks
and the power-spectrum bin edges."""
import numpy as np
import pytest
import torch

from oracle import cosmology as oc, nbody as onb
from jaxpm_gb300 import cosmology as pc, growth as pg, ode, utils
from jaxpm_gb300 import painting, pm


def test_growth_matches_oracle():
    c1, c2 = pc.Planck15(), oc.Cosmology()
    a = np.linspace(0.05, 1.0, 40)
    for name in ["growth_factor", "growth_rate", "growth_factor_second", "growth_rate_second",
                 "Gf", "Gf2", "dGfa", "dGf2a", "gp", "E", "dEa"]:
        x, y = getattr(pg, name)(c1, a), getattr(oc, name)(c2, a)
        assert np.allclose(x, y, rtol=1e-8, atol=1e-12), name


def test_growth_tables_match_fixture(golden):
    d = golden("growth.npz")
    t = pg.compute_growth_tables(pc.Planck15())
    for i, k in enumerate(["a", "g", "f", "h", "g2", "f2", "h2"]):
        assert np.allclose(t[i], d[k], rtol=1e-8), k


def test_dark_energy_parameters_change_growth():
    base = pc.Planck15()
    wcdm = pc.Planck15(w0=-0.9, wa=0.1)
    assert not np.isclose(pg.growth_factor(base, 0.5), pg.growth_factor(wcdm, 0.5))
    assert np.isclose(pg.growth_factor(wcdm, 0.5), oc.growth_factor(
        oc.Cosmology(w0=-0.9, wa=0.1), 0.5), rtol=1e-8)


def test_fpm_coefficients_match_oracle():
    k1, d1 = ode.fpm_coefficients(pc.Planck15(), 0.1, 1.0, 40)
    k2, d2 = onb.fpm_coefficients(oc.Cosmology(), 0.1, 1.0, 40)
    assert np.allclose(k1, k2, rtol=1e-9) and np.allclose(d1, d2, rtol=1e-9)


def test_linear_power_matches_oracle():
    k = np.logspace(-4, 1, 128)
    assert np.allclose(pc.linear_matter_power(pc.Planck15(), k),
                       oc.linear_matter_power(oc.Cosmology(), k), rtol=1e-10)


def test_sharding_and_halo_are_rejected():
    mesh = torch.zeros(4, 4, 4)
    pos = torch.zeros(64, 3)
    with pytest.raises(NotImplementedError):
        painting.cic_paint(mesh, pos, halo_size=2)
    with pytest.raises(NotImplementedError):
        painting.cic_read(mesh, pos, sharding=object())
    with pytest.raises(NotImplementedError):
        pm.pm_forces(pos, mesh_shape=(4, 4, 4), halo_size=(4, 4))


def test_particle_count_must_match_mesh_like_the_reference():
    with pytest.raises(TypeError, match="cannot reshape"):
        painting.cic_paint(torch.zeros(4, 4, 4), torch.zeros(10, 3))


def test_pm_forces_requires_mesh_shape_or_delta():
    with pytest.raises(AssertionError, match="delta should be provided"):
        pm.pm_forces(torch.zeros(8, 3))


def test_unknown_paint_mode():
    with pytest.raises(ValueError, match="unknown paint mode"):
        painting._mode("fancy")


def test_kedges_match_reference_rule():
    e = utils.kedges_for((32, 32, 32), (256.0,) * 3)
    dk = 2 * np.pi / 256 * 2
    assert np.isclose(e[0], 1.5 * dk) and np.allclose(np.diff(e), dk)
    assert e[-1] < np.pi * 32 / 256


def test_forward_model_host_scalar_derivatives():
    """The cosmology scalars' backward (central differences of host float64
    functions) agrees with an independent difference at a 10x larger step;
    sigma8 does not enter the LPT or step scalars."""
    import torch
    from jaxpm_gb300 import forward_model as fm
    th = torch.tensor([0.2589, 0.8159], dtype=torch.float64, requires_grad=True)

    def fn(t):
        return fm._scalars(t, None, 0.1, 1.0, 8, 2)
    out = fm._HostScalars.apply(th, fn, 1e-5)
    w = torch.linspace(0.5, 1.5, out.numel(), dtype=torch.float64)
    (out * w).sum().backward()
    h = 1e-4
    t0 = th.detach().numpy()
    fd = (fn(t0 + [h, 0]) - fn(t0 - [h, 0])) / (2 * h)
    ref = float(np.dot(w.numpy(), fd))
    assert abs(float(th.grad[0]) - ref) < 1e-5 * abs(ref)
    assert float(th.grad[1]) == 0.0
    # the scalars reproduce the step coefficients of the plain integrator
    from jaxpm_gb300 import ode
    k, d = ode.fpm_coefficients(fm.cosmology_of(t0), 0.1, 1.0, 8)
    assert np.allclose(out.detach().numpy()[4:12], k, rtol=1e-12)
    assert np.allclose(out.detach().numpy()[12:], d, rtol=1e-12)


def test_reference_arm_line_on_a_small_mesh(capsys):
    """bench.py --impl reference prints one JSON line with the contract's
    keys, the GPU arm's metric and the workload it ran (the oracle on the
    full workload at the given mesh; 16^3 here so it runs in seconds)."""
    import json
    import sys
    import bench
    argv = sys.argv
    sys.argv = ["bench.py", "--impl", "reference", "--mesh", "16", "--steps", "2",
                "--warmup", "1"]
    try:
        bench.main()
    finally:
        sys.argv = argv
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "higher_is_better",
                "impl", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["steps"] == 2 and line["value"] > 0
    assert line["config"]["particles"] == 16 ** 3 and line["config"]["mesh"] == [16] * 3
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
