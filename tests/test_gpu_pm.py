"""GPU parity of the force solver, LPT, the FastPM step and the power
spectrum against the oracle, through the C ABI.

Bars (float32 GPU vs oracle): forces within 1e-5 relative L2 of the float64
oracle; LPT fields and one-step states within 1e-5; final density power
spectrum within 1e-3 per k-bin after a full run."""
import numpy as np
import pytest
import torch

from oracle import cic, cosmology as oc, fourier as fo, nbody as onb, power as opw
from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5
PK_TOL = 1e-3


def T(x, cuda):
    return torch.as_tensor(np.ascontiguousarray(x)).to(cuda)


@pytest.mark.parametrize("mode", ["atomic", "binned", "deterministic"])
def test_pm_forces_golden(cuda, golden, mode):
    from jaxpm_gb300 import pm
    d = golden("pm_forces16.npz")
    f = pm.pm_forces(T(d["pos"], cuda), mesh_shape=(16,) * 3, paint_mode=mode)
    assert rel_l2(f.cpu(), d["forces64"]) < TOL
    f = pm.pm_forces(T(d["pos"], cuda), mesh_shape=(16,) * 3, r_split=1.5, paint_mode=mode)
    assert rel_l2(f.cpu(), d["forces64_rsplit"]) < TOL


@pytest.mark.parametrize("shape", [(32, 32, 32), (32, 32, 64), (24, 20, 18)])
def test_pm_forces_vs_oracle_shapes(cuda, shape):
    from jaxpm_gb300 import pm
    rng = np.random.default_rng(1)
    n = int(np.prod(shape))
    pos = (cic.lattice(shape).reshape(-1, 3) + rng.normal(0, 2.0, (n, 3))).astype(np.float32)
    ref = fo.pm_forces(pos.astype(np.float64), mesh_shape=shape, dtype=np.float64)
    f = pm.pm_forces(T(pos, cuda), mesh_shape=shape)
    assert rel_l2(f.cpu(), ref) < TOL


def test_force_meshes_from_delta(cuda):
    from jaxpm_gb300 import distributed, pm
    rng = np.random.default_rng(2)
    delta = rng.standard_normal((16, 16, 16))
    ref = fo.force_mesh(fo.fft3d(delta), dtype=np.float64)
    got = pm.force_meshes(T(delta.astype(np.float32), cuda))
    for i in range(3):
        assert rel_l2(got[i].cpu(), ref[i]) < TOL
    # complex (half-spectrum) delta gives the same forces at the particles
    pos = T(cic.lattice((16,) * 3).reshape(-1, 3).astype(np.float32), cuda)
    dk = distributed.fft3d(T(delta.astype(np.float32), cuda))
    f1 = pm.pm_forces(pos, delta=dk)
    f2 = pm.pm_forces(pos, delta=T(delta.astype(np.float32), cuda))
    assert torch.allclose(f1, f2, rtol=1e-5, atol=1e-6)


def test_fft_roundtrip_and_plain_kspace(cuda):
    from jaxpm_gb300 import distributed
    x = torch.randn((16, 12, 10), device=cuda)
    assert torch.allclose(distributed.ifft3d(distributed.fft3d(x), 10), x, atol=1e-5)


def test_pm_forces_vjp_matches_oracle(cuda):
    from jaxpm_gb300 import pm
    shape = (16, 16, 16)
    rng = np.random.default_rng(3)
    pos = (cic.lattice(shape).reshape(-1, 3) + rng.normal(0, 1.5, (4096, 3))).astype(np.float32)
    g = rng.standard_normal((4096, 3)).astype(np.float32)
    ref = fo.pm_forces_vjp(pos.astype(np.float64), shape, g.astype(np.float64))
    for mode in ["atomic", "binned", "deterministic"]:
        p = T(pos, cuda).requires_grad_(True)
        f = pm.pm_forces(p, mesh_shape=shape, paint_mode=mode)
        (f * T(g, cuda)).sum().backward()
        assert rel_l2(p.grad.cpu(), ref) < 1e-4, mode


def test_fused_step_plain_step_and_oracle_agree(cuda, golden):
    from jaxpm_gb300 import simulate, cosmology
    d = golden("sim16.npz")
    n = 16
    lat = cic.lattice((n,) * 3).reshape(-1, 3).astype(np.float32)
    x0, v0 = lat + d["dx2"], d["p2"]
    x_ref, v_ref = onb.fpm_step(x0, v0, (n,) * 3, d["kick"][0], d["drift"][0])
    for plain in [False, True]:
        sim = simulate.FastPM((n,) * 3, cosmology.Planck15(), 0.1, 1.0, 5, plain=plain)
        x, v = T(x0, cuda), T(v0, cuda)
        sim.step(x, v, 0)
        assert rel_l2(v.cpu() - T(v0, "cpu"), v_ref - v0) < TOL
        assert rel_l2(x.cpu() - T(x0, "cpu"), x_ref - x0) < TOL
        assert np.allclose(sim.kick, d["kick"], rtol=1e-9)


@pytest.mark.parametrize("order", [1, 2])
def test_lpt_golden(cuda, golden, order):
    from jaxpm_gb300 import pm, cosmology
    d = golden("sim16.npz")
    n = 16
    lat = T(cic.lattice((n,) * 3).reshape(-1, 3).astype(np.float32), cuda)
    dx, p, f = pm.lpt(cosmology.Planck15(), T(d["ic"], cuda), lat, a=0.1, order=order)
    assert rel_l2(dx.cpu(), d[f"dx{order}"]) < TOL
    assert rel_l2(p.cpu(), d[f"p{order}"]) < TOL
    assert rel_l2(f.cpu(), d[f"f{order}"]) < TOL
    # relative mode (particles=None) reads the same meshes at the lattice
    dxr, _, _ = pm.lpt(cosmology.Planck15(), T(d["ic"], cuda), None, a=0.1, order=order)
    assert rel_l2(dxr.reshape(-1, 3).cpu(), d[f"dx{order}"]) < TOL


def test_linear_field_golden(cuda, golden):
    from jaxpm_gb300 import pm
    d = golden("sim16.npz")
    ic = pm.linear_field((16,) * 3, [64.0] * 3, (d["pk_k"], d["pk_p"]), seed=None,
                         noise=T(d["noise"], cuda))
    assert rel_l2(ic.cpu(), d["ic"]) < TOL


def test_power_spectrum_matches_oracle(cuda):
    from jaxpm_gb300 import utils
    rng = np.random.default_rng(4)
    for shape, box in [((32, 32, 32), (256.0,) * 3), ((32, 32, 64), (256.0, 256.0, 512.0))]:
        m = (1 + 0.5 * rng.standard_normal(shape)).astype(np.float32)
        k_ref, p_ref = opw.power_spectrum(m, box_shape=box)
        k, p = utils.power_spectrum(T(m, cuda), box_shape=box)
        assert np.allclose(k, k_ref, rtol=1e-6)
        assert np.max(np.abs(p / p_ref - 1)) < 1e-5


def run_oracle_sim(noise, box, n_steps, order):
    cosmo = oc.Cosmology()
    k = np.logspace(-4, 1, 128)
    pk = oc.linear_matter_power(cosmo, k)
    shape = noise.shape
    ic = onb.linear_field(noise, box, k, pk)
    lat = cic.lattice(shape).reshape(-1, 3).astype(np.float32)
    dx, p, _ = onb.lpt(cosmo, ic, lat, a=0.1, order=order)
    kc, dc = onb.fpm_coefficients(cosmo, 0.1, 1.0, n_steps)
    x, v = lat + dx, p
    for i in range(n_steps):
        x, v = onb.fpm_step(x, v, shape, kc[i], dc[i])
    return cic.cic_paint(np.zeros(shape, np.float32), x), (k, pk)


@pytest.mark.parametrize("mode", ["atomic", "binned"])
def test_plain_pm_config_power_spectrum(cuda, mode):
    """32^3 particles on 32^3, box 200, 1LPT to a=0.1, 10 FastPM steps to
    a=1: final density P(k) within 1e-3 per bin of the oracle."""
    from jaxpm_gb300 import cosmology, distributed, painting, pm, simulate, utils
    n, box = 32, [200.0] * 3
    noise = np.random.default_rng(0).standard_normal((n,) * 3).astype(np.float32)
    rho_ref, table = run_oracle_sim(noise, box, 10, 1)
    cosmo = cosmology.Planck15()
    ic = pm.linear_field((n,) * 3, box, table, None, noise=T(noise, cuda))
    lat = distributed.uniform_particles((n,) * 3, device=cuda).reshape(-1, 3)
    dx, p, _ = pm.lpt(cosmo, ic, lat, a=0.1, order=1)
    x, v = (lat + dx).contiguous(), p.contiguous()
    simulate.FastPM((n,) * 3, cosmo, 0.1, 1.0, 10, paint_mode=mode).run(x, v)
    rho = painting.cic_paint(torch.zeros((n,) * 3, device=cuda), x)
    _, pk = utils.power_spectrum(rho, box_shape=box)
    _, pk_ref = opw.power_spectrum(rho_ref, box_shape=box)
    assert np.max(np.abs(pk / pk_ref - 1)) < PK_TOL
    # the field itself stays close as well
    assert rel_l2(rho.cpu(), rho_ref) < 1e-3


def test_2lpt_run_matches_golden_pk(cuda, golden):
    from jaxpm_gb300 import cosmology, painting, simulate, utils
    d = golden("sim16.npz")
    n = 16
    lat = cic.lattice((n,) * 3).reshape(-1, 3).astype(np.float32)
    x, v = T(lat + d["dx2"], cuda), T(d["p2"], cuda)
    simulate.FastPM((n,) * 3, cosmology.Planck15(), 0.1, 1.0, 5).run(x, v)
    assert rel_l2(x.cpu() - T(lat, "cpu"), d["final_pos"] - lat) < 1e-4
    rho = painting.cic_paint(torch.zeros((n,) * 3, device=cuda), x)
    _, pk = utils.power_spectrum(rho, box_shape=[64.0] * 3)
    _, pk_ref = opw.power_spectrum(d["final_rho"], box_shape=[64.0] * 3)
    assert np.max(np.abs(pk / pk_ref - 1)) < PK_TOL


def test_differentiable_nbody_gradient(cuda):
    """Gradient of a density loss through LPT and 3 steps w.r.t. the initial
    field, checked by a directional finite difference."""
    from jaxpm_gb300 import cosmology, distributed, painting, pm, simulate
    n = 16
    cosmo = cosmology.Planck15()
    ic0 = pm.linear_field((n,) * 3, [64.0] * 3, pm.pk_table(cosmo), seed=5, device=cuda)
    lat = distributed.uniform_particles((n,) * 3, device=cuda).reshape(-1, 3)
    target = torch.rand((n,) * 3, device=cuda, generator=torch.Generator(device=cuda).manual_seed(1))

    def loss(ic):
        dx, p, _ = pm.lpt(cosmo, ic, lat, a=0.1, order=1)
        x, v = simulate.nbody((lat + dx).contiguous(), p.contiguous(), cosmo, (n,) * 3, 0.1, 1.0,
                              3, checkpoint_every=2)
        rho = painting.cic_paint(torch.zeros((n,) * 3, device=cuda), x)
        return ((rho - target)**2).mean()

    ic = ic0.clone().requires_grad_(True)
    loss(ic).backward()
    g = ic.grad.double()
    direction = torch.randn((n,) * 3, device=cuda, generator=torch.Generator(device=cuda).manual_seed(2))
    eps = 1e-2
    with torch.no_grad():
        fd = (loss(ic0 + eps * direction) - loss(ic0 - eps * direction)).item() / (2 * eps)
    an = (g * direction.double()).sum().item()
    assert abs(an - fd) / abs(fd) < 2e-2
