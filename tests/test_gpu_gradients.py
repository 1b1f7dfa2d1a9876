"""GPU gradients of the differentiable forward model: the colouring and
2LPT-source adjoints (dot-product tests), and the gradient of a density
loss with respect to the white noise and to (Omega_c, sigma8) against
central finite differences of the float32 pipeline.

Bars: adjoint dot products within 1e-4 relative; end-to-end gradients
within 5e-2 of the finite differences (the CIC step has kinks at cell
faces, so float32 finite differences of a whole run carry percent-level
noise; the oracle-level check of the step adjoint is in the step tests)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_colouring_is_self_adjoint(cuda):
    from jaxpm_gb300 import cosmology, pm
    shape, box = (16, 24, 32), (40.0, 60.0, 80.0)
    table = pm.power_table(*pm.pk_table(cosmology.Planck15()), cuda)
    g = torch.Generator(device=cuda).manual_seed(0)
    x = torch.randn(shape, generator=g, device=cuda)
    y = torch.randn(shape, generator=g, device=cuda)
    lhs = float((pm.colour(x, table, box).double() * y.double()).sum())
    rhs = float((x.double() * pm.colour(y, table, box).double()).sum())
    assert abs(lhs - rhs) < 1e-4 * abs(lhs)
    # the autograd path of linear_field uses it
    noise = x.clone().requires_grad_(True)
    ic = pm.linear_field(shape, box, pm.pk_table(cosmology.Planck15()), 0, noise=noise)
    (ic * y).sum().backward()
    assert torch.allclose(noise.grad, pm.colour(y, table, box), rtol=1e-5, atol=1e-6)


def test_lpt2_source_adjoint_dot_product(cuda):
    """delta2 is quadratic in ic, so a central difference is exact up to
    rounding: <g, J h> against <J^T g, h>."""
    from jaxpm_gb300 import cosmology, pm
    shape = (32, 32, 32)
    ic = pm.linear_field(shape, [64.0] * 3, pm.pk_table(cosmology.Planck15()), seed=3,
                         device=cuda)
    gen = torch.Generator(device=cuda).manual_seed(1)
    h = torch.randn(shape, generator=gen, device=cuda) * ic.std()
    g = torch.randn(shape, generator=gen, device=cuda)
    icg = ic.clone().requires_grad_(True)
    d2 = pm._Source2LPT.apply(icg)
    (d2 * g).sum().backward()
    adj = float((icg.grad.double() * h.double()).sum())
    eps = 1e-2
    with torch.no_grad():
        jh = (pm._Source2LPT.apply(ic + eps * h).double() -
              pm._Source2LPT.apply(ic - eps * h).double()) / (2 * eps)
    fwd = float((g.double() * jh).sum())
    assert abs(adj - fwd) < 1e-4 * abs(fwd), (adj, fwd)


def _loss_setup(cuda, n=32, steps=6, order=2, engine="lattice"):
    from jaxpm_gb300 import distributed, forward_model as fm
    shape, box = (n,) * 3, (2.0 * n,) * 3
    theta0 = torch.tensor([0.2589, 0.8159], dtype=torch.float64)
    noise = distributed.normal_field(1, shape, device=cuda)
    with torch.no_grad():
        xt, _ = fm.lpt_nbody(distributed.normal_field(2, shape, device=cuda), theta0, shape,
                             box, n_steps=steps, order=order, checkpoint_every=0)
        target = torch.zeros(shape, device=cuda)
        from jaxpm_gb300 import painting
        target = painting.cic_paint(target, xt)

    def loss(nz, th):
        x, _ = fm.lpt_nbody(nz, th, shape, box, n_steps=steps, order=order, checkpoint_every=2,
                            engine=engine)
        return fm.density_mse(x, target)
    return noise, theta0, loss


@pytest.mark.parametrize("engine", ["lattice", "sorted"])
def test_gradient_wrt_cosmology_matches_finite_differences(cuda, engine):
    noise, theta0, loss = _loss_setup(cuda, engine=engine)
    th = theta0.clone().requires_grad_(True)
    loss(noise, th).backward()
    eps = 1e-3
    with torch.no_grad():
        for j in range(2):
            tp, tm = theta0.clone(), theta0.clone()
            tp[j] += eps
            tm[j] -= eps
            fd = (float(loss(noise, tp)) - float(loss(noise, tm))) / (2 * eps)
            an = float(th.grad[j])
            assert abs(an - fd) < 5e-2 * abs(fd), (j, an, fd)


@pytest.mark.parametrize("order,engine", [(1, "lattice"), (2, "lattice"), (2, "sorted")])
def test_gradient_wrt_noise_matches_finite_differences(cuda, order, engine):
    noise, theta0, loss = _loss_setup(cuda, order=order, engine=engine)
    nz = noise.clone().requires_grad_(True)
    loss(nz, theta0).backward()
    d = torch.randn(noise.shape, generator=torch.Generator(device=cuda).manual_seed(5),
                    device=cuda)
    eps = 1e-3
    with torch.no_grad():
        fd = (float(loss(noise + eps * d, theta0)) - float(loss(noise - eps * d, theta0))) / (
            2 * eps)
    an = float((nz.grad.double() * d.double()).sum())
    assert abs(an - fd) < 5e-2 * abs(fd), (an, fd)


def test_forward_model_matches_the_plain_pipeline(cuda):
    """Without gradients the forward model equals linear_field + lpt +
    nbody with host scalars."""
    from jaxpm_gb300 import cosmology, distributed, forward_model as fm, pm, simulate
    n, steps = 16, 3
    shape, box = (n,) * 3, (32.0,) * 3
    theta = torch.tensor([0.3, 0.7], dtype=torch.float64)
    noise = distributed.normal_field(4, shape, device=cuda)
    with torch.no_grad():
        x, v = fm.lpt_nbody(noise, theta, shape, box, n_steps=steps, checkpoint_every=0)
        c = fm.cosmology_of(theta)
        ic = pm.linear_field(shape, box, pm.pk_table(c), 0, noise=noise)
        lat = distributed.uniform_particles(shape, device=cuda).reshape(-1, 3)
        dx, p, _ = pm.lpt(c, ic, lat, a=0.1, order=2)
        xr, vr = simulate.nbody((lat + dx).contiguous(), p.contiguous(), c, shape, 0.1, 1.0,
                                steps)
    assert torch.allclose(x, xr, rtol=1e-5, atol=1e-4)
    assert torch.allclose(v, vr, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("shape,k", [((32, 32, 32), 3), ((24, 40, 16), 0)])
def test_sorted_engine_gradients_match_lattice_engine(cuda, shape, k):
    """simulate.nbody's two engines: the same final state and the same
    cotangents of the initial positions and velocities and of every step's
    kick and drift coefficients (the sorted engine's from its reverse sweep,
    the lattice engine's step by step), to float32 rounding of different
    force and paint orders."""
    from jaxpm_gb300 import cosmology, simulate
    from jaxpm_gb300.ode import fpm_coefficients
    steps = 6
    n = int(np.prod(shape))
    rng = np.random.default_rng(7)
    lat = np.stack(np.meshgrid(*[np.arange(s, dtype=np.float32) for s in shape], indexing="ij"),
                   -1).reshape(-1, 3)
    x0 = torch.from_numpy(lat + rng.normal(0, 0.7, (n, 3)).astype(np.float32)).to(cuda)
    v0 = torch.from_numpy(rng.normal(0, 0.3, (n, 3)).astype(np.float32)).to(cuda)
    gxo = torch.from_numpy(rng.normal(0, 1, (n, 3)).astype(np.float32)).to(cuda)
    gvo = torch.from_numpy(rng.normal(0, 1, (n, 3)).astype(np.float32)).to(cuda)
    kc, dc = fpm_coefficients(cosmology.Planck15(), 0.1, 1.0, steps)
    out = {}
    for engine in ("lattice", "sorted"):
        x = x0.clone().requires_grad_(True)
        v = v0.clone().requires_grad_(True)
        kick = torch.tensor(kc, dtype=torch.float64, requires_grad=True)
        drift = torch.tensor(dc, dtype=torch.float64, requires_grad=True)
        xf, vf = simulate.nbody(x, v, None, shape, 0.1, 1.0, steps, checkpoint_every=k,
                                coefficients=(kick, drift), engine=engine)
        ((xf * gxo).sum() + (vf * gvo).sum()).backward()
        out[engine] = (xf.detach(), vf.detach(), x.grad, v.grad, kick.grad.numpy(),
                       drift.grad.numpy())

    def rel(a, b):
        a, b = torch.as_tensor(a).double(), torch.as_tensor(b).double()
        return float((a - b).norm() / b.norm())
    L, S = out["lattice"], out["sorted"]
    assert rel(S[0].cpu() - x0.cpu(), L[0].cpu() - x0.cpu()) < 1e-4
    assert rel(S[1].cpu(), L[1].cpu()) < 1e-4
    assert rel(S[2].cpu(), L[2].cpu()) < 1e-3
    assert rel(S[3].cpu(), L[3].cpu()) < 1e-3
    assert rel(S[4], L[4]) < 1e-3 and rel(S[5], L[5]) < 1e-3
