"""The tile-sorted FastPM loop: the counting sort is a permutation that
orders particles by Morton tile key, the box-staged gather equals the plain
gather, and sorted runs reproduce the lattice-order runs and the oracle."""
import numpy as np
import pytest
import torch

from oracle import cic, cosmology as oc, fourier as fo, nbody as onb, power as opw
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def T(x, cuda):
    return torch.as_tensor(np.ascontiguousarray(x)).to(cuda)


def morton_keys(pos, shape, tile=8):
    cells = np.mod(np.floor(pos).astype(np.int64), np.array(shape))
    t = cells // tile

    def spread(v):
        out = np.zeros_like(v)
        for b in range(10):
            out |= ((v >> b) & 1) << (3 * b)
        return out
    return (spread(t[:, 0]) << 2) | (spread(t[:, 1]) << 1) | spread(t[:, 2])


@pytest.mark.parametrize("shape", [(64, 64, 64), (48, 40, 72)])
def test_tile_sort_is_a_sorting_permutation(cuda, lib, shape):
    from jaxpm_gb300 import _lib
    n = int(np.prod(shape))
    rng = np.random.default_rng(0)
    pos = rng.uniform(-shape[0], 2 * shape[0], (n, 3)).astype(np.float32)
    vel = rng.standard_normal((n, 3)).astype(np.float32)
    p, v = T(pos, cuda), T(vel, cuda)
    p2, v2 = torch.empty_like(p), torch.empty_like(v)
    ids = torch.empty(n, dtype=torch.int32, device=cuda)
    wsb = lib.pmgb_tile_sort_workspace_size(*shape, n)
    ws = torch.empty(wsb, dtype=torch.uint8, device=cuda)
    _lib.call("pmgb_tile_sort_f32", _lib.ptr(p), _lib.ptr(v), None, n, *shape, _lib.ptr(p2),
              _lib.ptr(v2), _lib.ptr(ids), _lib.ptr(ws), wsb, _lib.stream())
    i = ids.cpu().numpy()
    assert np.array_equal(np.sort(i), np.arange(n))
    assert np.array_equal(p2.cpu().numpy(), pos[i]) and np.array_equal(v2.cpu().numpy(), vel[i])
    keys = morton_keys(pos[i], shape)
    assert np.all(np.diff(keys) >= 0)
    back = torch.empty_like(p)
    _lib.call("pmgb_unpermute3_f32", _lib.ptr(p2), _lib.ptr(ids), n, _lib.ptr(back), _lib.stream())
    assert torch.equal(back, p)
    fwd = torch.empty_like(p)
    _lib.call("pmgb_permute3_f32", _lib.ptr(p), _lib.ptr(ids), n, _lib.ptr(fwd), _lib.stream())
    assert torch.equal(fwd, p2)


@pytest.mark.parametrize("shape", [(64, 64, 64), (48, 40, 72)])
def test_tile_sort_dest_and_gather3_pieces(cuda, lib, shape):
    """dest is the inverse of the sort's ids, and gather3 over the pieces of
    dest returns the sorted arrays to the caller's order bit for bit; index
    entries at or past n_in leave their rows untouched."""
    from jaxpm_gb300 import _lib
    n = int(np.prod(shape))
    rng = np.random.default_rng(3)
    pos = rng.uniform(0, shape[0], (n, 3)).astype(np.float32)
    vel = rng.standard_normal((n, 3)).astype(np.float32)
    p, v = T(pos, cuda), T(vel, cuda)
    p2, v2 = torch.empty_like(p), torch.empty_like(v)
    ids = torch.empty(n, dtype=torch.int32, device=cuda)
    dest = torch.empty(n, dtype=torch.int32, device=cuda)
    wsb = lib.pmgb_tile_sort_workspace_size(*shape, n)
    ws = torch.empty(wsb, dtype=torch.uint8, device=cuda)
    _lib.call("pmgb_tile_sort_dest_f32", _lib.ptr(p), _lib.ptr(v), None, n, *shape, _lib.ptr(p2),
              _lib.ptr(v2), _lib.ptr(ids), _lib.ptr(dest), _lib.ptr(ws), wsb, _lib.stream())
    i, d = ids.cpu().numpy(), dest.cpu().numpy()
    assert np.array_equal(i[d], np.arange(n)) and np.array_equal(d[i], np.arange(n))
    bounds = np.linspace(0, n, 8).astype(np.int64)
    back_p, back_v = torch.full_like(p, -1.0), torch.full_like(v, -1.0)
    for a, b in zip(bounds[:-1], bounds[1:]):
        a, b = int(a), int(b)
        _lib.call("pmgb_gather3_f32", _lib.ptr(p2), n, _lib.ptr(dest[a:b]), b - a,
                  _lib.ptr(back_p[a:b]), _lib.stream())
        _lib.call("pmgb_gather3_f32", _lib.ptr(v2), n, _lib.ptr(dest[a:b]), b - a,
                  _lib.ptr(back_v[a:b]), _lib.stream())
    assert torch.equal(back_p, p) and torch.equal(back_v, v)
    # rows whose index is past the source are skipped
    idx = torch.tensor([0, n, 1, 2 * n], dtype=torch.int32, device=cuda)
    out = torch.full((4, 3), 7.0, device=cuda)
    _lib.call("pmgb_gather3_f32", _lib.ptr(p2), n, _lib.ptr(idx), 4, _lib.ptr(out), _lib.stream())
    o = out.cpu().numpy()
    assert np.array_equal(o[0], pos[i[0]]) and np.array_equal(o[2], pos[i[1]])
    assert np.all(o[1] == 7.0) and np.all(o[3] == 7.0)
    with pytest.raises(Exception):
        _lib.call("pmgb_gather3_f32", _lib.ptr(p2), n, _lib.ptr(dest), n, _lib.ptr(p2),
                  _lib.stream())


def sorted_state(cuda, lib, pos, vel, shape):
    """Tile-sorts (pos, vel); returns sorted tensors, ids and the sort
    workspace holding the ranges."""
    from jaxpm_gb300 import _lib
    n = len(pos)
    p, v = T(pos, cuda), T(vel, cuda)
    ps, vs = torch.empty_like(p), torch.empty_like(v)
    ids = torch.empty(n, dtype=torch.int32, device=cuda)
    wsb = lib.pmgb_tile_sort_workspace_size(*shape, n)
    ws = torch.empty(wsb, dtype=torch.uint8, device=cuda)
    _lib.call("pmgb_tile_sort_f32", _lib.ptr(p), _lib.ptr(v), None, n, *shape, _lib.ptr(ps),
              _lib.ptr(vs), _lib.ptr(ids), _lib.ptr(ws), wsb, _lib.stream())
    return ps, vs, ids, ws, wsb


@pytest.mark.parametrize("shape,spread", [((64, 64, 64), 1.0), ((64, 64, 64), 6.0),
                                          ((40, 36, 44), 2.0)])
def test_tile_gather_and_paint_match_plain(cuda, lib, shape, spread):
    from jaxpm_gb300 import _lib
    n = int(np.prod(shape))
    rng = np.random.default_rng(1)
    pos = (cic.lattice(shape).reshape(-1, 3) + rng.normal(0, spread, (n, 3))).astype(np.float32)
    vel = rng.standard_normal((n, 3)).astype(np.float32)
    pb, vb, _, ws, wsb = sorted_state(cuda, lib, pos, vel, shape)
    stats = torch.zeros(3, dtype=torch.int32, device=cuda)
    s = _lib.stream()
    # paint of the sorted particles vs the oracle
    mesh = torch.empty(shape, device=cuda)
    _lib.call("pmgb_cic_paint_sorted_f32", _lib.ptr(mesh), *shape, _lib.ptr(pb), n, _lib.ptr(ws),
              wsb, _lib.ptr(stats), s)
    ref = cic.cic_paint(np.zeros(shape), pos.astype(np.float64), dtype=np.float64)
    assert rel_l2(mesh.cpu(), ref) < 1e-5
    # tile-staged gather + kick + drift vs the plain kernel on the same order
    f3 = T(rng.standard_normal((3, *shape)).astype(np.float32), cuda)
    pa, va = pb.clone(), vb.clone()
    _lib.call("pmgb_read3_kick_drift_f32", _lib.ptr(f3), n, *shape, _lib.ptr(pa), _lib.ptr(va), n,
              0.3, 0.7, None, s)
    _lib.call("pmgb_read3_kick_drift_binned_f32", _lib.ptr(f3), n, *shape, _lib.ptr(pb),
              _lib.ptr(vb), n, 0.3, 0.7, _lib.ptr(ws), wsb, _lib.ptr(stats), s)
    assert torch.allclose(va, vb, rtol=1e-6, atol=1e-6)
    assert torch.allclose(pa, pb, rtol=1e-6, atol=1e-5)
    assert stats.tolist() == [0, 0, 0]  # every particle inside its tile; no TMA timeout


def test_sorted_run_matches_lattice_run_and_oracle(cuda, golden):
    from jaxpm_gb300 import cosmology, painting, simulate, utils
    d = golden("sim16.npz")
    n = 16
    lat = cic.lattice((n,) * 3).reshape(-1, 3).astype(np.float32)
    x0, v0 = T(lat + d["dx2"], cuda), T(d["p2"], cuda)
    eng = simulate.SortedFastPM((n,) * 3, cosmology.Planck15(), 0.1, 1.0, 5, device=cuda)
    eng.load(x0, v0)
    eng.run()
    x, v = eng.state()
    assert rel_l2(x.cpu() - T(lat, "cpu"), d["final_pos"] - lat) < 1e-4
    assert rel_l2(v.cpu(), d["final_vel"]) < 1e-4
    rho = painting.cic_paint(torch.zeros((n,) * 3, device=cuda), x)
    _, pk = utils.power_spectrum(rho, box_shape=[64.0] * 3)
    _, pk_ref = opw.power_spectrum(d["final_rho"], box_shape=[64.0] * 3)
    assert np.max(np.abs(pk / pk_ref - 1)) < 1e-3


def test_sorted_c1_config_power_spectrum(cuda):
    """32^3, box 200, 1LPT to a=0.1, 10 steps: the sorted loop's final P(k)
    within 1e-3 per bin of the oracle run."""
    from jaxpm_gb300 import cosmology, distributed, painting, pm, simulate, utils
    n, box = 32, [200.0] * 3
    noise = np.random.default_rng(0).standard_normal((n,) * 3).astype(np.float32)
    cosmo_o = oc.Cosmology()
    k = np.logspace(-4, 1, 128)
    pkt = oc.linear_matter_power(cosmo_o, k)
    ic_o = onb.linear_field(noise, box, k, pkt)
    lat_o = cic.lattice((n,) * 3).reshape(-1, 3).astype(np.float32)
    dx_o, p_o, _ = onb.lpt(cosmo_o, ic_o, lat_o, a=0.1, order=1)
    kc, dc = onb.fpm_coefficients(cosmo_o, 0.1, 1.0, 10)
    xo, vo = lat_o + dx_o, p_o
    for i in range(10):
        xo, vo = onb.fpm_step(xo, vo, (n,) * 3, kc[i], dc[i])
    rho_ref = cic.cic_paint(np.zeros((n,) * 3, np.float32), xo)

    cosmo = cosmology.Planck15()
    ic = pm.linear_field((n,) * 3, box, (k, pkt), None, noise=T(noise, cuda))
    lat = distributed.uniform_particles((n,) * 3, device=cuda).reshape(-1, 3)
    dx, p, _ = pm.lpt(cosmo, ic, lat, a=0.1, order=1)
    eng = simulate.SortedFastPM((n,) * 3, cosmo, 0.1, 1.0, 10, device=cuda)
    eng.load(lat + dx, p)
    eng.run()
    rho = painting.paint(torch.zeros((n,) * 3, device=cuda), eng.positions, mode="binned")
    _, pk = utils.power_spectrum(rho, box_shape=box)
    _, pk_ref = opw.power_spectrum(rho_ref, box_shape=box)
    assert np.max(np.abs(pk / pk_ref - 1)) < 1e-3
    x, _ = eng.state()
    assert rel_l2(x.cpu(), xo) < 1e-4


def test_sorted_adjoint_matches_lattice_adjoint(cuda, golden):
    from jaxpm_gb300 import cosmology, simulate
    d = golden("sim16.npz")
    n = 16
    lat = cic.lattice((n,) * 3).reshape(-1, 3).astype(np.float32)
    x0, v0 = T(lat + d["dx2"], cuda), T(d["p2"], cuda)
    g = torch.Generator(device=cuda).manual_seed(3)
    gx = torch.randn(x0.shape, device=cuda, generator=g)
    gv = torch.randn(x0.shape, device=cuda, generator=g)
    ref = simulate.FastPM((n,) * 3, cosmology.Planck15(), 0.1, 1.0, 4, device=cuda)
    (_, _), (ax, av) = ref.vjp(x0, v0, gx, gv)
    eng = simulate.SortedFastPM((n,) * 3, cosmology.Planck15(), 0.1, 1.0, 4, device=cuda)
    (_, _), (bx, bv) = eng.vjp(x0, v0, gx, gv)
    assert rel_l2(bx.cpu(), ax.cpu()) < 1e-4
    assert rel_l2(bv.cpu(), av.cpu()) < 1e-4


@pytest.mark.parametrize("shape", [(32, 32, 32), (24, 40, 16)])
def test_sorted_adjoint_clustered(cuda, shape):
    """Reverse sweep of the sorted loop on a clustered distribution: one tile
    holds more than the shared-memory box limit (global-atomic path), others
    sit on the periodic edges (wrapped boxes), the rest is a perturbed
    lattice.  Reference: the lattice-order adjoint (pm_forces_vjp)."""
    from jaxpm_gb300 import cosmology, simulate
    n = int(np.prod(shape))
    rng = np.random.default_rng(11)
    lat = cic.lattice(shape).reshape(-1, 3).astype(np.float64)
    pos = lat + rng.normal(0, 0.3, lat.shape)
    k = 9000
    pos[:k] = rng.uniform(8.0, 15.99, (k, 3))           # one 8^3 tile, > 8192 particles
    pos[k:k + 2000] = rng.uniform(-0.5, 0.5, (2000, 3))  # straddles the periodic corner
    vel = rng.normal(0, 0.2, lat.shape)
    x0, v0 = T(pos.astype(np.float32), cuda), T(vel.astype(np.float32), cuda)
    g = torch.Generator(device=cuda).manual_seed(5)
    gx = torch.randn(x0.shape, device=cuda, generator=g)
    gv = torch.randn(x0.shape, device=cuda, generator=g)
    cosmo = cosmology.Planck15()
    ref = simulate.FastPM(shape, cosmo, 0.5, 1.0, 2, n_particles=n, device=cuda)
    (ax_f, av_f), (ax, av) = ref.vjp(x0, v0, gx, gv)
    eng = simulate.SortedFastPM(shape, cosmo, 0.5, 1.0, 2, n_particles=n, device=cuda)
    (bx_f, bv_f), (bx, bv) = eng.vjp(x0, v0, gx, gv)
    assert rel_l2(bx_f.cpu(), ax_f.cpu()) < 1e-5
    assert rel_l2(bx.cpu(), ax.cpu()) < 1e-4
    assert rel_l2(bv.cpu(), av.cpu()) < 1e-4
    assert eng.stats["tma_wait_timeout"] == 0


def test_sorted_reverse_step_identity_dest(cuda, lib):
    """pmgb_fpm_step_sorted_vjp_f32 with dest = NULL (no re-sort) on the
    quantities recorded by one sorted step equals the generic adjoint
    u = gv + drift gx, gx += (dF/dx)^T (kick u), gv = u."""
    from jaxpm_gb300 import _lib, cosmology, simulate
    n = 16
    shape = (n,) * 3
    np_ = n ** 3
    rng = np.random.default_rng(2)
    lat = cic.lattice(shape).reshape(-1, 3)
    x = T((lat + rng.normal(0, 0.4, lat.shape)).astype(np.float32), cuda)
    v = T(rng.normal(0, 0.1, lat.shape).astype(np.float32), cuda)
    eng = simulate.SortedFastPM(shape, cosmology.Planck15(), 0.3, 1.0, 1, device=cuda)
    eng.load(x, v)
    xs = eng.pos[eng.cur].clone()
    f3, dest, offs = [t[0] for t in eng.alloc_store(potential=False)[1:]]
    eng.step(0, record=(f3, dest, offs))
    gx = torch.randn((np_, 3), device=cuda)
    gv = torch.randn((np_, 3), device=cuda)
    gxo, gvo = torch.empty_like(gx), torch.empty_like(gv)
    kick, drift = float(eng.kick[0]), float(eng.drift[0])
    s = _lib.stream()
    _lib.call("pmgb_fpm_step_sorted_vjp_f32", _lib.ptr(xs), _lib.ptr(f3), None, _lib.ptr(offs),
              _lib.ptr(gx), _lib.ptr(gv), _lib.ptr(gxo), _lib.ptr(gvo), np_, n, n, n, kick,
              drift, 0.0, _lib.ptr(eng.ws), eng.ws_bytes, None, s)
    ref = simulate.FastPM(shape, cosmology.Planck15(), 0.3, 1.0, 1, device=cuda)
    rx, rv = gx.clone(), gv.clone()
    ref.step_vjp(xs, rx, rv, 0)
    assert rel_l2(gvo.cpu(), rv.cpu()) < 1e-6
    assert rel_l2(gxo.cpu(), rx.cpu()) < 1e-4


@pytest.mark.parametrize("shape", [(64, 64, 64), (48, 40, 72)])
def test_gather_paint_matches_gather_then_paint(cuda, lib, shape):
    """The fused gather + kick + drift + paint of the new positions equals the
    plain sorted gather followed by a separate paint (same new state bit for
    bit, same density to float rounding), on a clustered distribution with
    tiles on the periodic edges and one tile above the single-word limit."""
    from jaxpm_gb300 import _lib, cosmology, simulate
    n = int(np.prod(shape))
    rng = np.random.default_rng(21)
    lat = cic.lattice(shape).reshape(-1, 3).astype(np.float64)
    pos = lat + rng.normal(0, 0.4, lat.shape)
    pos[:5000] = rng.uniform(16.0, 23.99, (5000, 3))   # one tile > 4096 particles
    pos[5000:7000] = rng.uniform(-0.6, 0.6, (2000, 3))  # the periodic corner
    vel = rng.normal(0, 1.0, lat.shape)
    vel[:100] *= 20.0                                  # a few leave the paint box
    x0, v0 = T(pos.astype(np.float32), cuda), T(vel.astype(np.float32), cuda)
    eng = simulate.SortedFastPM(shape, cosmology.Planck15(), 0.5, 1.0, 1, device=cuda)
    eng.load(x0, v0)
    px, pv = eng.pos[eng.cur], eng.vel[eng.cur]
    nx, ny, nz = shape
    g = torch.Generator(device=cuda).manual_seed(8)
    f3 = torch.randn((3, *shape), device=cuda, generator=g) * 0.05
    s = _lib.stream()
    kick, drift = 0.7, 0.9
    a_x, a_v = px.clone(), pv.clone()
    _lib.call("pmgb_read3_kick_drift_binned_f32", _lib.ptr(f3), n, nx, ny, nz, _lib.ptr(a_x),
              _lib.ptr(a_v), n, kick, drift, _lib.ptr(eng.sort_ws), eng.sort_bytes, None, s)
    b_x, b_v = px.clone(), pv.clone()
    mesh = torch.full(shape, 7.0, device=cuda)  # overwritten
    stats = torch.zeros(3, dtype=torch.int32, device=cuda)
    _lib.call("pmgb_read3_kick_drift_paint_binned_f32", _lib.ptr(f3), n, nx, ny, nz,
              _lib.ptr(b_x), _lib.ptr(b_v), n, kick, drift, _lib.ptr(mesh),
              _lib.ptr(eng.sort_ws), eng.sort_bytes, _lib.ptr(stats), s)
    assert torch.equal(a_x, b_x) and torch.equal(a_v, b_v)
    ref = torch.zeros(shape, device=cuda)
    _lib.call("pmgb_cic_paint_f32", _lib.ptr(ref), nx, ny, nz, _lib.ptr(b_x), n, None, 1.0,
              _lib.PAINT_ATOMIC, 0, None, 0, s)
    assert rel_l2(mesh.cpu(), ref.cpu()) < 1e-6
    assert abs(mesh.double().sum().item() - n) / n < 1e-6
    st = stats.cpu().tolist()
    assert st[2] == 0


@pytest.mark.parametrize("shape", [(64, 64, 64), (32, 32, 32)])
def test_fused_run_matches_step_by_step(cuda, shape):
    """pmgb_fpm_run_sorted_f32 (density painted by the previous gather) equals
    the same steps made one composite call at a time."""
    from jaxpm_gb300 import cosmology, simulate
    rng = np.random.default_rng(22)
    lat = cic.lattice(shape).reshape(-1, 3)
    x0 = T((lat + rng.normal(0, 0.5, lat.shape)).astype(np.float32), cuda)
    v0 = T(rng.normal(0, 0.3, lat.shape).astype(np.float32), cuda)
    cosmo = cosmology.Planck15()
    a = simulate.SortedFastPM(shape, cosmo, 0.1, 1.0, 7, device=cuda)
    a.load(x0, v0)
    a.run()
    b = simulate.SortedFastPM(shape, cosmo, 0.1, 1.0, 7, device=cuda)
    b.load(x0, v0)
    for i in range(7):
        b.step(i)
    (ax, av), (bx, bv) = a.state(), b.state()
    assert rel_l2(ax.cpu(), bx.cpu()) < 1e-5
    assert rel_l2(av.cpu(), bv.cpu()) < 1e-4
    assert torch.equal(a.ids_current.sort().values, b.ids_current.sort().values)
    assert a.stats["tma_wait_timeout"] == 0


@pytest.mark.parametrize("split", [(1, 1), (2, 3), (3, 4)])
def test_permuted_run_leaves_tile_order_and_chains(cuda, lib, split):
    """The run loop moves only a permutation between steps and sorts the
    particles once at the end: after run() they are in tile order (a sorted
    paint finds no particle outside its tile), and runs of odd and even step
    counts chained one after the other equal one run over all the steps."""
    from jaxpm_gb300 import _lib, cosmology, simulate
    shape = (32, 32, 32)
    n1, n2 = split
    rng = np.random.default_rng(5)
    lat = cic.lattice(shape).reshape(-1, 3)
    x0 = T((lat + rng.normal(0, 0.8, lat.shape)).astype(np.float32), cuda)
    v0 = T(rng.normal(0, 0.5, lat.shape).astype(np.float32), cuda)
    cosmo = cosmology.Planck15()
    a = simulate.SortedFastPM(shape, cosmo, 0.1, 1.0, n1 + n2, device=cuda)
    a.load(x0, v0)
    a.run(steps=n1)
    mesh = torch.empty(shape, device=cuda)
    stats = torch.zeros(3, dtype=torch.int32, device=cuda)
    _lib.call("pmgb_cic_paint_sorted_f32", _lib.ptr(mesh), *shape, _lib.ptr(a.positions),
              a.n, _lib.ptr(a.sort_ws), a.sort_bytes, _lib.ptr(stats), _lib.stream())
    torch.cuda.synchronize()
    assert stats.tolist() == [0, 0, 0]
    a.run(steps=n2, start=n1)
    b = simulate.SortedFastPM(shape, cosmo, 0.1, 1.0, n1 + n2, device=cuda)
    b.load(x0, v0)
    b.run()
    (ax, av), (bx, bv) = a.state(), b.state()
    assert rel_l2(ax.cpu() - x0.cpu(), bx.cpu() - x0.cpu()) < 1e-5
    assert rel_l2(av.cpu(), bv.cpu()) < 1e-5
    assert torch.equal(a.ids_current.sort().values, torch.arange(a.n, device=cuda,
                                                                  dtype=torch.int32))


@pytest.mark.parametrize("shape", [(64, 64, 64), (32, 128, 64)])
@pytest.mark.parametrize("r_split", [0.0, 1.5])
def test_run_loop_potential_path_matches_oracle(cuda, shape, r_split):
    """On the potential pipeline's shapes (cubic and not) the run loop takes
    the forces from the potential (one inverse transform; the order-1
    gradient as its real-space stencil in the gather).  Three steps against
    the oracle's FastPM steps (float64)."""
    from jaxpm_gb300 import cosmology, simulate
    rng = np.random.default_rng(31)
    lat = cic.lattice(shape).reshape(-1, 3)
    x0 = (lat + rng.normal(0, 1.0, lat.shape)).astype(np.float32)
    v0 = rng.normal(0, 0.3, lat.shape).astype(np.float32)
    eng = simulate.SortedFastPM(shape, cosmology.Planck15(), 0.1, 1.0, 3, r_split=r_split,
                                device=cuda)
    eng.load(T(x0, cuda), T(v0, cuda))
    eng.run()
    x, v = eng.state()
    xr, vr = x0.astype(np.float64), v0.astype(np.float64)
    for i in range(3):
        F = fo.pm_forces(xr, mesh_shape=shape, r_split=r_split, dtype=np.float64)
        vr = vr + eng.kick[i] * F
        xr = xr + eng.drift[i] * vr
    assert rel_l2(v.cpu().numpy() - v0, vr - v0) < 1e-5
    assert rel_l2(x.cpu().numpy() - x0, xr - x0) < 1e-5
    assert eng.stats["gather"] == 0 and eng.stats["tma_wait_timeout"] == 0


@pytest.mark.parametrize("r_split", [0.0, 1.5])
def test_sorted_adjoint_potential_recording(cuda, r_split):
    """The reverse sweep recorded with each step's potential (the gather and
    its reverse step derive the forces with the order-1 stencil) against the
    same sweep recorded with three force meshes per step, and against the
    lattice-order adjoint, on a 64^3 perturbed lattice over 3 steps."""
    from jaxpm_gb300 import cosmology, simulate
    n = 64
    shape = (n,) * 3
    rng = np.random.default_rng(21)
    lat = cic.lattice(shape).reshape(-1, 3)
    x0 = T((lat + rng.normal(0, 0.6, lat.shape)).astype(np.float32), cuda)
    v0 = T(rng.normal(0, 0.3, lat.shape).astype(np.float32), cuda)
    g = torch.Generator(device=cuda).manual_seed(8)
    gx = torch.randn(x0.shape, device=cuda, generator=g)
    gv = torch.randn(x0.shape, device=cuda, generator=g)
    cosmo = cosmology.Planck15()
    eng = simulate.SortedFastPM(shape, cosmo, 0.3, 1.0, 3, r_split=r_split, device=cuda)
    store_p = eng.alloc_store(potential=True)
    assert store_p[1].dim() == 4  # [n, nx, ny, nz]: one potential per step
    (px, pv), (pgx, pgv) = eng.vjp(x0, v0, gx, gv, store=store_p)
    (fx, fv), (fgx, fgv) = eng.vjp(x0, v0, gx, gv, store=eng.alloc_store(potential=False))
    assert rel_l2(px.cpu(), fx.cpu()) < 1e-6
    assert rel_l2(pgx.cpu(), fgx.cpu()) < 1e-5
    assert rel_l2(pgv.cpu(), fgv.cpu()) < 1e-5
    ref = simulate.FastPM(shape, cosmo, 0.3, 1.0, 3, r_split=r_split, device=cuda)
    (_, _), (ax, av) = ref.vjp(x0, v0, gx, gv)
    assert rel_l2(pgx.cpu(), ax.cpu()) < 1e-4
    assert rel_l2(pgv.cpu(), av.cpu()) < 1e-4
    assert eng.stats["tma_wait_timeout"] == 0


def test_tile_schedule_dynamic_tails_128(cuda):
    """At 128^3 (4096 tiles) both gathers reach the dynamic part of their
    tile schedule: the forward gather takes three quarters of the keys
    statically and the rest from its counter, the reverse gather only its
    first two tiles per CTA.  Two run-loop steps against the oracle's FastPM
    steps (float64), and the reverse sweep against the lattice-order
    adjoint."""
    from jaxpm_gb300 import cosmology, simulate
    shape = (128, 128, 128)
    rng = np.random.default_rng(41)
    lat = cic.lattice(shape).reshape(-1, 3)
    x0 = (lat + rng.normal(0, 1.0, lat.shape)).astype(np.float32)
    v0 = rng.normal(0, 0.3, lat.shape).astype(np.float32)
    cosmo = cosmology.Planck15()
    eng = simulate.SortedFastPM(shape, cosmo, 0.1, 1.0, 2, device=cuda)
    eng.load(T(x0, cuda), T(v0, cuda))
    eng.run()
    x, v = eng.state()
    xr, vr = x0.astype(np.float64), v0.astype(np.float64)
    for i in range(2):
        F = fo.pm_forces(xr, mesh_shape=shape, dtype=np.float64)
        vr = vr + eng.kick[i] * F
        xr = xr + eng.drift[i] * vr
    assert rel_l2(v.cpu().numpy() - v0, vr - v0) < 1e-5
    assert rel_l2(x.cpu().numpy() - x0, xr - x0) < 1e-5
    assert eng.stats["gather"] == 0 and eng.stats["tma_wait_timeout"] == 0
    g = torch.Generator(device=cuda).manual_seed(9)
    gx = torch.randn(x.shape, device=cuda, generator=g)
    gv = torch.randn(x.shape, device=cuda, generator=g)
    (_, _), (bx, bv) = eng.vjp(T(x0, cuda), T(v0, cuda), gx, gv)
    ref = simulate.FastPM(shape, cosmo, 0.1, 1.0, 2, device=cuda)
    (_, _), (ax, av) = ref.vjp(T(x0, cuda), T(v0, cuda), gx, gv)
    assert rel_l2(bx.cpu(), ax.cpu()) < 1e-4
    assert rel_l2(bv.cpu(), av.cpu()) < 1e-4
    assert eng.stats["tma_wait_timeout"] == 0


@pytest.mark.parametrize("shape,paint_mode", [((64, 64, 64), "binned"),
                                              ((64, 64, 64), "atomic"),
                                              ((64, 64, 64), "deterministic"),
                                              ((48, 40, 72), "binned")])
def test_run_host_matches_device_run(cuda, shape, paint_mode):
    """SortedFastPM.run_host (state in pinned host memory, copies chunked and
    overlapped across steps) equals the device run loop from the same
    state: the streamed schedule (pieces painted as they land, gathered and
    sent back as they are done) on the potential pipeline's shapes, the
    sorted composite step on the others."""
    from jaxpm_gb300 import cosmology, simulate
    rng = np.random.default_rng(51)
    lat = cic.lattice(shape).reshape(-1, 3)
    x0 = (lat + rng.normal(0, 0.8, lat.shape)).astype(np.float32)
    v0 = rng.normal(0, 0.3, lat.shape).astype(np.float32)
    eng = simulate.SortedFastPM(shape, cosmology.Planck15(), 0.1, 1.0, 4, device=cuda)
    eng.load(T(x0, cuda), T(v0, cuda))
    eng.run()
    x, v = eng.state()
    hx = torch.from_numpy(x0.copy()).pin_memory()
    hv = torch.from_numpy(v0.copy()).pin_memory()
    eng.run_host(hx, hv, chunks=5, paint_mode=paint_mode)
    torch.cuda.synchronize(cuda)
    assert rel_l2(hx.numpy() - x0, x.cpu().numpy() - x0) < 1e-5
    assert rel_l2(hv.numpy() - v0, v.cpu().numpy() - v0) < 1e-4
    # the engine holds the same final state, in tile order again
    ex, ev = eng.state()
    assert torch.equal(ex.cpu(), hx) and torch.equal(ev.cpu(), hv)
    # two calls over the halves of the run (start=) equal one call
    hx2 = torch.from_numpy(x0.copy()).pin_memory()
    hv2 = torch.from_numpy(v0.copy()).pin_memory()
    eng.run_host(hx2, hv2, steps=2, paint_mode=paint_mode)
    eng.run_host(hx2, hv2, steps=2, start=2, paint_mode=paint_mode)
    torch.cuda.synchronize(cuda)
    assert rel_l2(hx2.numpy() - x0, hx.numpy() - x0) < 1e-5
    with pytest.raises(ValueError):
        eng.run_host(hx2, hv2, steps=3, start=2)
    with pytest.raises(ValueError):
        eng.run_host(torch.from_numpy(x0.copy()), torch.from_numpy(v0.copy()))
    with pytest.raises(ValueError):
        eng.run_host(hx2, hv2, steps=1, paint_mode="nearest")


def test_permuted_gather_abi_pieces_compose_to_the_run(cuda, lib):
    """The run loop's pieces through the C ABI (pmgb_mesh_potential_f32,
    pmgb_read_potential_kick_drift_paint_perm_f32, pmgb_tile_resort_index,
    pmgb_gather_u32, pmgb_tile_scatter_f32), issued one by one as a caller
    would, give the state of pmgb_fpm_run_sorted_f32 (64^3: the potential
    pipeline's shapes)."""
    from jaxpm_gb300 import _lib, cosmology, simulate
    shape = (64, 64, 64)
    nx, ny, nz = shape
    K = 4
    rng = np.random.default_rng(9)
    lat = cic.lattice(shape).reshape(-1, 3)
    x0 = T((lat + rng.normal(0, 0.8, lat.shape)).astype(np.float32), cuda)
    v0 = T(rng.normal(0, 0.5, lat.shape).astype(np.float32), cuda)
    cosmo = cosmology.Planck15()
    ref = simulate.SortedFastPM(shape, cosmo, 0.1, 1.0, K, device=cuda)
    ref.load(x0, v0)
    ref.run()
    e = simulate.SortedFastPM(shape, cosmo, 0.1, 1.0, K, device=cuda)
    e.load(x0, v0)
    n = e.n
    s = _lib.stream()
    mesh = torch.empty(shape, device=cuda)
    pot = torch.empty(shape, device=cuda)
    wsb = lib.pmgb_mesh_forces_workspace_size(nx, ny, nz)
    ws = torch.empty(wsb, dtype=torch.uint8, device=cuda)
    perms = torch.empty((2, n), dtype=torch.int32, device=cuda)
    P = _lib.ptr
    _lib.call("pmgb_cic_paint_sorted_f32", P(mesh), nx, ny, nz, P(e.pos[0]), n, P(e.sort_ws),
              e.sort_bytes, P(e.stats_buf), s)
    cur, pc, permuted = 0, 0, False
    for i in range(K):
        _lib.call("pmgb_mesh_potential_f32", P(mesh), P(pot), nx, ny, nz, 0.0, P(ws), wsb, s)
        last = i + 1 == K
        out = cur if not permuted else 1 - cur
        _lib.call("pmgb_read_potential_kick_drift_paint_perm_f32", P(pot), nx, ny, nz,
                  P(e.pos[cur]), P(e.vel[cur]), P(perms[pc]) if permuted else None,
                  P(e.pos[out]), P(e.vel[out]), n, float(e.kick[i]), float(e.drift[i]),
                  None if last else P(mesh), P(e.sort_ws), e.sort_bytes, P(e.stats_buf), s)
        if last:
            if permuted:
                _lib.call("pmgb_gather_u32", P(e.ids[cur]), P(perms[pc]), n, P(e.ids[out]), s)
            _lib.call("pmgb_tile_scatter_f32", P(e.pos[out]), P(e.vel[out]), P(e.ids[out]), n,
                      nx, ny, nz, P(e.pos[1 - out]), P(e.vel[1 - out]), P(e.ids[1 - out]),
                      None, P(e.sort_ws), e.sort_bytes, s)
            cur = 1 - out
        else:
            _lib.call("pmgb_tile_resort_index", n, nx, ny, nz,
                      P(perms[pc]) if permuted else None, P(perms[1 - pc]), P(e.ids[cur]),
                      P(e.ids[out]), P(e.sort_ws), e.sort_bytes, s)
            pc, cur, permuted = 1 - pc, out, True
    e.cur = cur
    (ax, av), (bx, bv) = ref.state(), e.state()
    assert rel_l2(bx.cpu() - x0.cpu(), ax.cpu() - x0.cpu()) < 1e-5
    assert rel_l2(bv.cpu(), av.cpu()) < 1e-5
    assert torch.equal(e.ids_current.sort().values, torch.arange(n, device=cuda,
                                                                  dtype=torch.int32))
    assert e.stats == {"paint": 0, "gather": 0, "tma_wait_timeout": 0}


def test_coef_cotangents_match_a_torch_statement(cuda, lib):
    """pmgb_fpm_coef_cotangents_f32 adds <g_vel, F(pos)> and
    <g_pos_next[dest], pos_next[dest] - pos> to two device doubles: the
    same sums computed with pmgb_cic_read3_f32 and torch gathers."""
    from jaxpm_gb300 import _lib
    shape = (32, 24, 16)
    nx, ny, nz = shape
    n = 20000
    rng = np.random.default_rng(12)
    pos = T(rng.uniform(-3, 40, (n, 3)).astype(np.float32), cuda)
    pos_next = T(rng.uniform(-3, 40, (n, 3)).astype(np.float32), cuda)
    dest = T(rng.permutation(n).astype(np.int32), cuda)
    f3 = T(rng.standard_normal((3, nx, ny, nz)).astype(np.float32), cuda)
    gpn = T(rng.standard_normal((n, 3)).astype(np.float32), cuda)
    gv = T(rng.standard_normal((n, 3)).astype(np.float32), cuda)
    out = torch.tensor([0.5, -0.25], dtype=torch.float64, device=cuda)  # added to
    _lib.call("pmgb_fpm_coef_cotangents_f32", _lib.ptr(pos), _lib.ptr(pos_next), _lib.ptr(dest),
              _lib.ptr(f3), nx * ny * nz, nx, ny, nz, _lib.ptr(gpn), _lib.ptr(gv), n,
              _lib.ptr(out), _lib.stream())
    F = torch.empty_like(pos)
    _lib.call("pmgb_cic_read3_f32", _lib.ptr(f3), nx * ny * nz, nx, ny, nz, _lib.ptr(pos), n,
              _lib.ptr(F), _lib.stream())
    d = dest.long()
    ref_k = float((gv.double() * F.double()).sum()) + 0.5
    ref_d = float((gpn[d].double() * (pos_next[d].double() - pos.double())).sum()) - 0.25
    got = out.cpu().numpy()
    assert abs(got[0] - ref_k) < 1e-5 * (1 + abs(ref_k))
    assert abs(got[1] - ref_d) < 1e-4 * (1 + abs(ref_d))
    with pytest.raises(_lib.PmgbError):
        _lib.call("pmgb_fpm_coef_cotangents_f32", _lib.ptr(pos), _lib.ptr(pos_next), None,
                  _lib.ptr(f3), 10, nx, ny, nz, _lib.ptr(gpn), _lib.ptr(gv), n, _lib.ptr(out),
                  _lib.stream())


def test_run_timing_reads_the_runs_phases_and_changes_nothing(cuda):
    """With launch timing on, a run records its gathers, force evaluations
    and re-sorts: each phase's mean is positive and their sum fits in the
    run's own time; the state equals that of an untimed run (up to the
    order of the float atomics of the particles that leave their tiles)."""
    from jaxpm_gb300 import _lib, cosmology, simulate
    shape, K = (64, 64, 64), 5
    rng = np.random.default_rng(23)
    lat = cic.lattice(shape).reshape(-1, 3)
    x0 = T((lat + rng.normal(0, 0.5, lat.shape)).astype(np.float32), cuda)
    v0 = T(rng.normal(0, 0.3, lat.shape).astype(np.float32), cuda)
    eng = simulate.SortedFastPM(shape, cosmology.Planck15(), 0.1, 1.0, K, device=cuda)
    eng.load(x0, v0)
    eng.run()
    ref = [t.clone() for t in eng.state()]
    _lib.set_run_timing(True)
    try:
        eng.load(x0, v0)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        eng.run()
        b.record()
        torch.cuda.synchronize()
        t = _lib.run_timing()
    finally:
        _lib.set_run_timing(False)
    total = a.elapsed_time(b)
    assert t["steps"] == K
    assert t["read_kick_drift"] > 0 and t["forces"] > 0 and t["sort"] > 0
    assert K * t["read_kick_drift"] + K * t["forces"] < total
    got = eng.state()
    assert rel_l2(got[0].cpu(), ref[0].cpu()) < 1e-6
    assert rel_l2(got[1].cpu(), ref[1].cpu()) < 1e-5
