"""GPU parity of the batched engine (one launch per phase over many
simulations of different mesh shapes and cosmologies) against the oracle
and against the single-simulation engine, through the C ABI.

Bars: forces within 1e-5 relative L2 of the float64 oracle per simulation;
batched steps within 1e-5 of the single-simulation step (both paint with
float32 atomics, so only the summation order differs); adjoints within
1e-4 of the single-simulation reverse sweep; a graph replay equal to the
eager run up to atomic summation order."""
import numpy as np
import pytest
import torch

from oracle import cic, cosmology as oc, fourier as fo, nbody as onb
from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5
SHAPES = [(16, 16, 16), (24, 24, 24), (16, 16, 16), (16, 24, 32), (32, 32, 32)]


def T(x, cuda):
    return torch.as_tensor(np.ascontiguousarray(x)).to(cuda)


def perturbed_lattice(shape, seed, sigma=1.5):
    rng = np.random.default_rng(seed)
    n = int(np.prod(shape))
    return (cic.lattice(shape).reshape(-1, 3) + rng.normal(0, sigma, (n, 3))).astype(np.float32)


def cosmos(n, seed=0):
    from jaxpm_gb300 import cosmology
    rng = np.random.default_rng(seed)
    return [cosmology.Planck15(Omega_c=float(rng.uniform(0.2, 0.35)),
                               sigma8=float(rng.uniform(0.6, 1.0))) for _ in range(n)]


def test_batched_forces_match_oracle_per_simulation(cuda):
    from jaxpm_gb300 import batched
    b = batched.BatchedFastPM(SHAPES, cosmos(len(SHAPES)), 0.1, 1.0, 2, device=cuda)
    parts = [perturbed_lattice(s, i) for i, s in enumerate(SHAPES)]
    f = b.forces(T(np.concatenate(parts), cuda))
    for s, (shape, p, fs) in enumerate(zip(SHAPES, parts, b.split(f))):
        ref = fo.pm_forces(p.astype(np.float64), mesh_shape=shape, dtype=np.float64)
        assert rel_l2(fs.cpu(), ref) < TOL, (s, shape)


def test_batched_forces_rsplit_and_empty_simulation(cuda):
    from jaxpm_gb300 import batched
    shapes = [(16, 16, 16), (8, 8, 8), (24, 16, 16)]
    counts = [4096, 0, 3000]
    b = batched.BatchedFastPM(shapes, cosmos(3), 0.1, 1.0, 2, n_particles=counts,
                              r_split=1.5, device=cuda)
    rng = np.random.default_rng(4)
    parts = [rng.uniform(-4, np.array(sh) + 4, (n, 3)).astype(np.float32)
             for sh, n in zip(shapes, counts)]
    f = b.forces(T(np.concatenate(parts), cuda))
    for shape, p, fs in zip(shapes, parts, b.split(f)):
        if len(p) == 0:
            assert fs.numel() == 0
            continue
        ref = fo.pm_forces(p.astype(np.float64), mesh_shape=shape, r_split=1.5,
                           dtype=np.float64)
        assert rel_l2(fs.cpu(), ref) < TOL


def test_batched_paint_matches_oracle(cuda):
    from jaxpm_gb300 import batched
    b = batched.BatchedFastPM(SHAPES, cosmos(len(SHAPES)), 0.1, 1.0, 2, device=cuda)
    parts = [perturbed_lattice(s, 10 + i, sigma=3.0) for i, s in enumerate(SHAPES)]
    meshes = b.paint(T(np.concatenate(parts), cuda))
    for shape, p, m in zip(SHAPES, parts, meshes):
        ref = cic.cic_paint(np.zeros(shape), p.astype(np.float64))
        assert m.shape == shape
        assert rel_l2(m.cpu(), ref) < TOL
        assert abs(float(m.double().sum()) - len(p)) < 1e-3 * len(p)


def test_batched_mixed_distributions(cuda):
    """One batch holding a slightly perturbed lattice, uniform random
    positions in lattice storage, a 12^3 lattice and a non-cubic mesh:
    paint, forces and one step of each against the oracle."""
    from jaxpm_gb300 import batched
    shapes = [(16, 16, 16), (16, 16, 16), (12, 12, 12), (16, 24, 32)]
    rng = np.random.default_rng(11)
    parts = [perturbed_lattice(shapes[0], 1, sigma=0.3),
             rng.uniform(0, 16, (16**3, 3)).astype(np.float32),
             perturbed_lattice(shapes[2], 2, sigma=0.5),
             perturbed_lattice(shapes[3], 3, sigma=1.2)]
    b = batched.BatchedFastPM(shapes, cosmos(len(shapes)), 0.1, 1.0, 2, device=cuda)
    x = T(np.concatenate(parts), cuda)
    for shape, p, m in zip(shapes, parts, b.paint(x)):
        ref = cic.cic_paint(np.zeros(shape), p.astype(np.float64))
        assert rel_l2(m.cpu(), ref) < TOL
    f = b.forces(x)
    for shape, p, fs in zip(shapes, parts, b.split(f)):
        ref = fo.pm_forces(p.astype(np.float64), mesh_shape=shape, dtype=np.float64)
        assert rel_l2(fs.cpu(), ref) < TOL
    v = torch.zeros_like(x)
    xs = x.clone()
    b.step(xs, v, 0)
    kick = b.kick[0].cpu().numpy()
    for s, (shape, p) in enumerate(zip(shapes, parts)):
        ref = fo.pm_forces(p.astype(np.float64), mesh_shape=shape, dtype=np.float64)
        assert rel_l2(b.split(v)[s].cpu(), kick[s] * ref) < TOL


def test_batched_step_matches_single_simulation_steps(cuda):
    from jaxpm_gb300 import batched, simulate
    cs = cosmos(len(SHAPES), seed=1)
    n_steps = 3
    b = batched.BatchedFastPM(SHAPES, cs, 0.1, 1.0, n_steps, device=cuda)
    xs = [perturbed_lattice(s, 20 + i, sigma=1.0) for i, s in enumerate(SHAPES)]
    vs = [np.random.default_rng(30 + i).normal(0, 0.3, x.shape).astype(np.float32)
          for i, x in enumerate(xs)]
    x, v = T(np.concatenate(xs), cuda), T(np.concatenate(vs), cuda)
    b.run(x, v)
    for s, shape in enumerate(SHAPES):
        sim = simulate.FastPM(shape, cs[s], 0.1, 1.0, n_steps, device=cuda)
        xr, vr = T(xs[s], cuda), T(vs[s], cuda)
        sim.run(xr, vr)
        assert np.allclose(sim.kick, b.kick[:, s].cpu().numpy(), rtol=1e-6)
        assert rel_l2(b.split(x)[s].cpu().numpy() - xs[s], (xr.cpu().numpy() - xs[s])) < TOL, s
        assert rel_l2(b.split(v)[s].cpu().numpy() - vs[s], (vr.cpu().numpy() - vs[s])) < TOL, s


def test_batched_step_matches_oracle_step(cuda):
    """One step of each simulation against the oracle's FastPM step with
    that simulation's own kick and drift."""
    from jaxpm_gb300 import batched
    shapes = [(16, 16, 16), (24, 24, 24)]
    cs = cosmos(2, seed=2)
    b = batched.BatchedFastPM(shapes, cs, 0.1, 1.0, 4, device=cuda)
    xs = [perturbed_lattice(s, 40 + i, sigma=1.0) for i, s in enumerate(shapes)]
    vs = [np.random.default_rng(50 + i).normal(0, 0.3, x.shape).astype(np.float32)
          for i, x in enumerate(xs)]
    x, v = T(np.concatenate(xs), cuda), T(np.concatenate(vs), cuda)
    b.step(x, v, 1)
    for s, shape in enumerate(shapes):
        oc_s = oc.Cosmology(Omega_c=cs[s].Omega_c, Omega_b=cs[s].Omega_b, h=cs[s].h,
                            n_s=cs[s].n_s, sigma8=cs[s].sigma8)
        kick, drift = onb.fpm_coefficients(oc_s, 0.1, 1.0, 4)
        assert np.allclose(b.kick[1, s].item(), kick[1], rtol=1e-6)
        xr, vr = onb.fpm_step(xs[s], vs[s], shape, kick[1], drift[1])
        assert rel_l2(b.split(v)[s].cpu().numpy() - vs[s], vr - vs[s]) < TOL
        assert rel_l2(b.split(x)[s].cpu().numpy() - xs[s], xr - xs[s]) < TOL


def test_batched_pos_before_record(cuda):
    from jaxpm_gb300 import batched
    b = batched.BatchedFastPM(SHAPES[:2], cosmos(2), 0.1, 1.0, 2, device=cuda)
    x0 = T(np.concatenate([perturbed_lattice(s, i) for i, s in enumerate(SHAPES[:2])]), cuda)
    x, v = x0.clone(), torch.zeros_like(x0)
    rec = torch.full_like(x0, float("nan"))
    b.step(x, v, 0, pos_before=rec)
    assert torch.equal(rec, x0)
    assert not torch.equal(x, x0)


def test_batched_vjp_matches_single_simulation_vjp(cuda):
    from jaxpm_gb300 import batched, simulate
    shapes = [(16, 16, 16), (24, 24, 24), (16, 16, 16)]
    cs = cosmos(3, seed=3)
    n_steps = 3
    b = batched.BatchedFastPM(shapes, cs, 0.1, 1.0, n_steps, device=cuda)
    xs = [perturbed_lattice(s, 60 + i, sigma=1.0) for i, s in enumerate(shapes)]
    vs = [np.random.default_rng(70 + i).normal(0, 0.3, x.shape).astype(np.float32)
          for i, x in enumerate(xs)]
    rng = np.random.default_rng(80)
    gxs = [rng.standard_normal(x.shape).astype(np.float32) for x in xs]
    gvs = [rng.standard_normal(x.shape).astype(np.float32) for x in xs]
    (xf, vf), (gx, gv) = b.vjp(T(np.concatenate(xs), cuda), T(np.concatenate(vs), cuda),
                               T(np.concatenate(gxs), cuda), T(np.concatenate(gvs), cuda))
    for s, shape in enumerate(shapes):
        sim = simulate.FastPM(shape, cs[s], 0.1, 1.0, n_steps, device=cuda)
        (xr, vr), (gxr, gvr) = sim.vjp(T(xs[s], cuda), T(vs[s], cuda), T(gxs[s], cuda),
                                       T(gvs[s], cuda))
        assert rel_l2(b.split(xf)[s].cpu().numpy() - xs[s], xr.cpu().numpy() - xs[s]) < TOL
        assert rel_l2(b.split(gx)[s].cpu(), gxr.cpu()) < 1e-4, s
        assert rel_l2(b.split(gv)[s].cpu(), gvr.cpu()) < 1e-4, s


def test_batched_vjp_matches_oracle_reverse_sweep(cuda):
    """Input cotangents of a two-step batched run against the float64
    oracle's reverse sweep with each simulation's own coefficients (the
    oracle sweep itself is pinned to float64 finite differences on the
    CPU).  Finite differences of the float32 GPU run cannot reach this bar:
    the CIC step has kinks at cell faces, so a difference step large enough
    to rise above float32 rounding crosses faces for ~1% of particles."""
    from jaxpm_gb300 import batched
    shapes = [(16, 16, 16), (8, 8, 16)]
    cs = cosmos(2, seed=5)
    b = batched.BatchedFastPM(shapes, cs, 0.1, 1.0, 2, device=cuda)
    rng = np.random.default_rng(95)
    xs = [perturbed_lattice(s, 90 + i, 0.8) for i, s in enumerate(shapes)]
    vs = [rng.normal(0, 0.2, x.shape).astype(np.float32) for x in xs]
    gxs = [rng.standard_normal(x.shape).astype(np.float32) for x in xs]
    gvs = [rng.standard_normal(x.shape).astype(np.float32) for x in xs]
    _, (gx, gv) = b.vjp(T(np.concatenate(xs), cuda), T(np.concatenate(vs), cuda),
                        T(np.concatenate(gxs), cuda), T(np.concatenate(gvs), cuda))
    kick, drift = b.kick.double().cpu().numpy(), b.drift.double().cpu().numpy()
    for s, shape in enumerate(shapes):
        _, (gxr, gvr) = onb.fpm_run_vjp(xs[s], vs[s], shape, kick[:, s], drift[:, s], gxs[s],
                                        gvs[s])
        assert rel_l2(b.split(gx)[s].cpu(), gxr) < 1e-4, s
        assert rel_l2(b.split(gv)[s].cpu(), gvr) < 1e-4, s


def test_batched_graph_replay_matches_eager(cuda):
    from jaxpm_gb300 import batched
    shapes = [(16, 16, 16), (24, 24, 24), (32, 32, 32)]
    b = batched.BatchedFastPM(shapes, cosmos(3), 0.1, 1.0, 4, device=cuda)
    x0 = T(np.concatenate([perturbed_lattice(s, i, 1.0) for i, s in enumerate(shapes)]), cuda)
    v0 = torch.zeros_like(x0)
    xe, ve = x0.clone(), v0.clone()
    b.run(xe, ve)
    xg, vg = x0.clone(), v0.clone()
    g = b.capture(xg, vg)
    assert torch.equal(xg, x0)
    g.replay()
    torch.cuda.synchronize()
    assert rel_l2((xg - x0).cpu(), (xe - x0).cpu()) < TOL
    assert rel_l2(vg.cpu(), ve.cpu()) < TOL


def test_batched_workspace_must_be_initialised(cuda):
    from jaxpm_gb300 import _lib
    lib = _lib.load()
    t = _lib.sim_table([(16, 16, 16)], [10])
    nbytes = lib.pmgb_batch_workspace_size(t, 1)
    ws = torch.empty(nbytes, dtype=torch.uint8, device=cuda)
    pos = torch.zeros((10, 3), device=cuda)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_pm_forces_batched_f32", t, 1, _lib.ptr(pos), _lib.ptr(pos), 0.0,
                  _lib.ptr(ws), nbytes, _lib.stream())
    assert "pmgb_batch_init" in str(e.value)
    _lib.call("pmgb_batch_init", t, 1, _lib.ptr(ws), nbytes, _lib.stream())
    # a different table on the same workspace is refused
    t2 = _lib.sim_table([(16, 16, 16)], [11])
    with pytest.raises(_lib.PmgbError):
        _lib.call("pmgb_pm_forces_batched_f32", t2, 1, _lib.ptr(pos), _lib.ptr(pos), 0.0,
                  _lib.ptr(ws), nbytes, _lib.stream())
    lib.pmgb_batch_release(_lib.ptr(ws))


def test_batched_initial_conditions_match_single(cuda):
    from jaxpm_gb300 import batched, cosmology, distributed, pm
    shapes = [(16, 16, 16), (24, 24, 24)]
    cs = cosmos(2, seed=7)
    boxes = [[2.0 * s[0]] * 3 for s in shapes]
    x, v = batched.initial_conditions(shapes, boxes, cs, [3, 4], device=cuda)
    assert x.shape == (16**3 + 24**3, 3)
    ic = pm.linear_field(shapes[1], boxes[1], pm.pk_table(cs[1]), seed=4, device=cuda)
    lat = distributed.uniform_particles(shapes[1], device=cuda).reshape(-1, 3)
    dx, p, _ = pm.lpt(cs[1], ic, lat, a=0.1, order=2)
    assert torch.allclose(x[16**3:], lat + dx)
    assert torch.allclose(v[16**3:], p)


def test_batched_groups_at_unaligned_offsets(cuda):
    """A 5^3 group ahead of 16^3 simulations puts their pool meshes at float
    offsets that are not multiples of 4: the painters must fall back to
    scalar reductions there (and stay exact against the oracle)."""
    from jaxpm_gb300 import batched
    shapes = [(5, 5, 5), (16, 16, 16), (16, 16, 16)]
    parts = [perturbed_lattice(s, 200 + i, sigma=1.0) for i, s in enumerate(shapes)]
    b = batched.BatchedFastPM(shapes, cosmos(3), 0.1, 1.0, 2, device=cuda)
    x = T(np.concatenate(parts), cuda)
    for shape, p, m in zip(shapes, parts, b.paint(x)):
        ref = cic.cic_paint(np.zeros(shape), p.astype(np.float64))
        assert rel_l2(m.cpu(), ref) < TOL
    for shape, p, fs in zip(shapes, parts, b.split(b.forces(x))):
        ref = fo.pm_forces(p.astype(np.float64), mesh_shape=shape, dtype=np.float64)
        assert rel_l2(fs.cpu(), ref) < TOL
    rng = np.random.default_rng(7)
    gx = T(rng.standard_normal(x.shape).astype(np.float32), cuda)
    gv = T(rng.standard_normal(x.shape).astype(np.float32), cuda)
    _, (gxb, gvb) = b.vjp(x, torch.zeros_like(x), gx, gv)
    kick, drift = b.kick.double().cpu().numpy(), b.drift.double().cpu().numpy()
    for s, shape in enumerate(shapes):
        _, (gxr, gvr) = onb.fpm_run_vjp(parts[s], np.zeros_like(parts[s]), shape, kick[:, s],
                                        drift[:, s], b.split(gx)[s].cpu().numpy(),
                                        b.split(gv)[s].cpu().numpy())
        assert rel_l2(b.split(gxb)[s].cpu(), gxr) < 1e-4, s


@pytest.mark.parametrize("groups", [1, 3, 8])
def test_batched_run_host_matches_device_run(cuda, groups):
    """BatchedFastPM.run_host (state in pinned host memory, the simulations
    streamed through the host link in groups that overlap) equals the device
    run from the same state; two calls over the halves of the run equal one
    call; a range past the engine's steps raises before any copy."""
    from jaxpm_gb300 import batched
    K = 4
    b = batched.BatchedFastPM(SHAPES, cosmos(len(SHAPES), 3), 0.1, 1.0, K, device=cuda)
    parts = [perturbed_lattice(s, 10 + i) for i, s in enumerate(SHAPES)]
    x0 = np.concatenate(parts)
    rng = np.random.default_rng(5)
    v0 = rng.normal(0, 0.3, x0.shape).astype(np.float32)
    x, v = T(x0, cuda), T(v0, cuda)
    b.run(x, v)
    hx = torch.from_numpy(x0.copy()).pin_memory()
    hv = torch.from_numpy(v0.copy()).pin_memory()
    b.run_host(hx, hv, groups=groups)
    torch.cuda.synchronize(cuda)
    assert rel_l2(hx.numpy() - x0, x.cpu().numpy() - x0) < TOL
    assert rel_l2(hv.numpy() - v0, v.cpu().numpy() - v0) < 1e-4
    hx2 = torch.from_numpy(x0.copy()).pin_memory()
    hv2 = torch.from_numpy(v0.copy()).pin_memory()
    b.run_host(hx2, hv2, steps=2, groups=groups)
    b.run_host(hx2, hv2, steps=2, start=2, groups=groups)
    torch.cuda.synchronize(cuda)
    assert rel_l2(hx2.numpy() - x0, hx.numpy() - x0) < TOL
    with pytest.raises(ValueError):
        b.run_host(hx2, hv2, steps=3, start=2)
    with pytest.raises(ValueError):
        b.run_host(torch.from_numpy(x0.copy()), torch.from_numpy(v0.copy()))
