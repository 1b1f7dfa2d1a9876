"""The CPU oracle against analytic known answers and its frozen fixtures.

The reference cannot run here and ships no golden vectors, so the oracle is
held by closed-form cases (single particles, lattices, plane waves,
Einstein-de Sitter growth) and by the fixtures in ``tests/golden``.
"""
import numpy as np
import pytest

from oracle import cic, cosmology as cm, fourier as fo, nbody as nb, power as pw
from conftest import rel_l2


# --- CIC known answers -------------------------------------------------------

def test_particle_at_cell_corner_paints_one_cell():
    m = cic.cic_paint(np.zeros((4, 4, 4)), np.array([[1.0, 2.0, 3.0]]), dtype=np.float64)
    assert m[1, 2, 3] == 1.0 and m.sum() == 1.0


def test_particle_at_cell_centre_splits_evenly():
    m = cic.cic_paint(np.zeros((4, 4, 4)), np.array([[1.5, 1.5, 1.5]]), dtype=np.float64)
    assert np.allclose(m[1:3, 1:3, 1:3], 1 / 8) and np.isclose(m.sum(), 1.0)


def test_face_and_wrap():
    # on a face: half in each of two cells along z
    m = cic.cic_paint(np.zeros((4, 4, 4)), np.array([[0.0, 0.0, 3.5]]), dtype=np.float64)
    assert m[0, 0, 3] == 0.5 and m[0, 0, 0] == 0.5
    # just below zero wraps to the last cell
    m = cic.cic_paint(np.zeros((4, 4, 4)), np.array([[-0.25, 0.0, 0.0]]), dtype=np.float64)
    assert np.isclose(m[3, 0, 0], 0.25) and np.isclose(m[0, 0, 0], 0.75)


def test_uniform_lattice_paints_constant_mesh():
    for shape in [(8, 8, 8), (4, 6, 10)]:
        pos = cic.lattice(shape).reshape(-1, 3) + 0.25
        m = cic.cic_paint(np.zeros(shape), pos, dtype=np.float64)
        assert np.allclose(m, 1.0)


def test_read_of_linear_field_is_exact_inside():
    n = 16
    x = np.arange(n, dtype=np.float64)
    mesh = np.broadcast_to(x[:, None, None], (n, n, n)).copy()
    pos = np.array([[3.3, 7.1, 2.9], [10.75, 0.5, 15.0]])
    out = cic.cic_read(mesh, pos, np.float64)
    assert np.allclose(out, pos[:, 0])


def test_paint_read_adjointness():
    rng = np.random.default_rng(0)
    pos = rng.uniform(-3, 11, size=(300, 3))
    g = rng.standard_normal((8, 8, 8))
    w = rng.uniform(0.5, 2, 300)
    lhs = (cic.cic_paint(np.zeros((8, 8, 8)), pos, weight=w, dtype=np.float64) * g).sum()
    rhs = (w * cic.cic_read(g, pos, np.float64)).sum()
    assert np.isclose(lhs, rhs, rtol=1e-12)


def test_paint_vjp_matches_finite_differences():
    rng = np.random.default_rng(1)
    pos = rng.uniform(0.1, 7.9, size=(20, 3))
    g = rng.standard_normal((8, 8, 8))
    gpos, _ = cic.cic_paint_vjp(pos, (8, 8, 8), g)
    eps = 1e-6
    for p in range(5):
        for d in range(3):
            dp = np.zeros_like(pos)
            dp[p, d] = eps
            f = lambda x: (cic.cic_paint(np.zeros((8, 8, 8)), x, dtype=np.float64) * g).sum()
            fd = (f(pos + dp) - f(pos - dp)) / (2 * eps)
            assert np.isclose(gpos[p, d], fd, rtol=1e-5, atol=1e-8)


def test_relative_mode_matches_absolute_away_from_wrap():
    rng = np.random.default_rng(2)
    shape = (8, 8, 8)
    disp = rng.uniform(-0.4, 0.4, size=(*shape, 3))
    pos = cic.lattice(shape) + disp
    a = cic.cic_paint(np.zeros(shape), pos.reshape(-1, 3), dtype=np.float64)
    r = cic.cic_paint_dx(disp, dtype=np.float64)
    assert np.allclose(a, r, atol=1e-12)
    mesh = rng.standard_normal(shape)
    assert np.allclose(cic.cic_read(mesh, pos.reshape(-1, 3), np.float64),
                       cic.cic_read_dx(mesh, disp, np.float64).reshape(-1), atol=1e-12)


# --- Fourier / forces --------------------------------------------------------

def test_plane_wave_force_is_analytic():
    # delta = cos(w x), w = 2 pi m / n: the potential is -cos(w x)/w^2 and,
    # with the order-1 gradient g = (8 sin w - sin 2w)/6, the force is
    # F_x = -g/w^2 sin(w x) (pointing towards the overdensity at x = 0)
    n, m = 32, 3
    w = 2 * np.pi * m / n
    x = np.arange(n)
    delta = np.broadcast_to(np.cos(w * x)[:, None, None], (n, n, n)).astype(np.float64)
    f = fo.force_mesh(fo.fft3d(delta), dtype=np.float64)
    g = (8 * np.sin(w) - np.sin(2 * w)) / 6
    expect = -g / w**2 * np.sin(w * x)
    assert np.allclose(f[0][:, 0, 0], expect, atol=1e-12)
    assert np.allclose(f[1], 0, atol=1e-12) and np.allclose(f[2], 0, atol=1e-12)


def test_kspace_operator_is_antisymmetric():
    # K_i(-k) = conj(K_i(k)) and conj(K_i) = -K_i: the real-space operator
    # A_i satisfies <A_i a, b> = -<a, A_i b>
    rng = np.random.default_rng(3)
    a, b = rng.standard_normal((2, 8, 8, 8))
    for i in range(3):
        K = fo.kspace_multiplier((8, 8, 8), i)
        Aa = fo.ifft3d(K * fo.fft3d(a))
        Ab = fo.ifft3d(K * fo.fft3d(b))
        assert np.isclose((Aa * b).sum(), -(a * Ab).sum(), rtol=1e-10, atol=1e-12)


def test_pm_forces_vjp_matches_finite_differences():
    rng = np.random.default_rng(5)
    shape = (8, 8, 8)
    pos = (cic.lattice(shape).reshape(-1, 3) + rng.uniform(-0.3, 0.3, (512, 3)) + 0.5)
    g = rng.standard_normal((512, 3))
    gp = fo.pm_forces_vjp(pos, shape, g)
    v = rng.standard_normal((512, 3))
    eps = 1e-6
    f = lambda x: (fo.pm_forces(x, mesh_shape=shape, dtype=np.float64) * g).sum()
    fd = (f(pos + eps * v) - f(pos - eps * v)) / (2 * eps)
    assert np.isclose((gp * v).sum(), fd, rtol=1e-6)


def test_lattice_particles_feel_no_force():
    pos = cic.lattice((8, 8, 8)).reshape(-1, 3).astype(np.float64)
    f = fo.pm_forces(pos, mesh_shape=(8, 8, 8), dtype=np.float64)
    assert np.abs(f).max() < 1e-12


# --- cosmology ----------------------------------------------------------------

def test_einstein_de_sitter_growth():
    eds = cm.Cosmology(Omega_c=1.0 - 0.05, Omega_b=0.05)
    a = np.array([0.2, 0.5, 0.9])
    assert np.allclose(cm.growth_factor(eds, a), a, rtol=1e-6)
    assert np.allclose(cm.growth_rate(eds, a), 1.0, rtol=1e-6)
    assert np.allclose(cm.growth_rate_second(eds, a), 2.0, rtol=1e-4)
    assert np.allclose(cm.growth_factor_second(eds, a), a**2, rtol=2e-3)


def test_power_spectrum_of_white_noise_is_flat():
    rng = np.random.default_rng(4)
    m = rng.standard_normal((32, 32, 32))
    k, p = pw.power_spectrum(m, box_shape=[32.0] * 3)
    assert np.allclose(p, 1.0, rtol=0.15)


def test_fpm_coefficients_positive_and_finite():
    kc, dc = nb.fpm_coefficients(cm.Cosmology(), 0.1, 1.0, 10)
    assert np.all(np.isfinite(kc)) and np.all(kc > 0) and np.all(dc > 0)


# --- frozen fixtures ----------------------------------------------------------

@pytest.mark.parametrize("tag,shape", [("cube", (8, 8, 8)), ("rect", (8, 6, 10))])
def test_oracle_cic_fixtures(golden, tag, shape):
    d = golden("cic.npz")
    idx, w = cic.cic_weights(d[f"{tag}_pos"], shape, np.float32)
    assert np.array_equal(idx, d[f"{tag}_idx"])
    assert np.array_equal(w.view(np.int32), d[f"{tag}_w"].view(np.int32))
    ridx, rw = cic.enmesh(cic.lattice(shape), d[f"{tag}_disp"], shape, np.float32)
    assert np.array_equal(ridx, d[f"{tag}_rel_idx"])
    assert np.array_equal(rw.view(np.int32), d[f"{tag}_rel_w"].view(np.int32))
    assert np.array_equal(cic.cic_read(d[f"{tag}_mesh"], d[f"{tag}_pos"], np.float32),
                          d[f"{tag}_read32"])


def test_oracle_forces_fixture(golden):
    d = golden("pm_forces16.npz")
    f = fo.pm_forces(d["pos"].astype(np.float64), mesh_shape=(16,) * 3, dtype=np.float64)
    assert rel_l2(f, d["forces64"]) < 1e-12
    f32 = fo.pm_forces(d["pos"], mesh_shape=(16,) * 3, dtype=np.float32)
    # float32 restatement vs float64: the error the float32 GPU path is held to
    assert rel_l2(f32, d["forces64"]) < 1e-5


def test_oracle_growth_fixture(golden):
    d = golden("growth.npz")
    t = cm.growth_tables(cm.Cosmology())
    for i, k in enumerate(["a", "g", "f", "h", "g2", "f2", "h2"]):
        assert np.allclose(t[i], d[k], rtol=1e-9)


def test_oracle_step_adjoint_matches_float64_finite_difference():
    """The oracle's reverse sweep of two FastPM steps against central
    differences in float64 (eps 1e-6 cells: no particle crosses a cell face,
    where the CIC step has kinks)."""
    shape = (8, 8, 16)
    n = int(np.prod(shape))
    rng = np.random.default_rng(0)
    x0 = cic.lattice(shape).reshape(-1, 3) + rng.normal(0, 0.8, (n, 3))
    v0 = rng.normal(0, 0.2, (n, 3))
    ks, ds = [0.9, 1.3], [0.7, 0.5]
    gxo, gvo = rng.standard_normal((n, 3)), rng.standard_normal((n, 3))
    _, (gx, gv) = nb.fpm_run_vjp(x0, v0, shape, ks, ds, gxo, gvo)

    def loss(x, v):
        (xf, vf), _ = nb.fpm_run_vjp(x, v, shape, ks, ds, gxo, gvo)
        return (xf * gxo).sum() + (vf * gvo).sum()

    d = rng.standard_normal((n, 3))
    eps = 1e-6
    fd_x = (loss(x0 + eps * d, v0) - loss(x0 - eps * d, v0)) / (2 * eps)
    fd_v = (loss(x0, v0 + eps * d) - loss(x0, v0 - eps * d)) / (2 * eps)
    assert abs(fd_x - (gx * d).sum()) < 1e-6 * abs(fd_x)
    assert abs(fd_v - (gv * d).sum()) < 1e-6 * abs(fd_v)


# --- the C statement of paint/read against the NumPy statement --------------

@pytest.mark.parametrize("shape", [(8, 8, 8), (8, 6, 10), (32, 32, 32)])
def test_c_oracle_matches_numpy_oracle(shape):
    from oracle import native
    if native.lib() is None:
        pytest.skip("no C compiler for the C oracle")
    rng = np.random.default_rng(5)
    n = np.array(shape)
    for dtype in (np.float32, np.float64):
        pos = (rng.uniform(-2, 3, (20000, 3)) * n).astype(dtype)
        pos[:5] = [[0, 0, 0], [n[0], 0, n[2]], [-1e-4, -1e-4, -1e-4], [n[0] - 1e-4, 1, 2],
                   [0.5, 0.5, 0.5]]
        mesh = rng.standard_normal(shape).astype(dtype)
        wts = rng.uniform(0.5, 1.5, len(pos)).astype(dtype)
        out = {}
        for use_c in (True, False):
            cic.NATIVE = use_c
            try:
                out[use_c] = (cic.cic_read(mesh, pos, dtype),
                              cic.cic_paint(np.zeros(shape), pos, weight=wts, dtype=dtype),
                              cic.cic_paint(np.zeros(shape), pos, weight=0.7, dtype=dtype))
            finally:
                cic.NATIVE = True
        # the position gradients of the VJPs (float64 sums in another order)
        g = rng.standard_normal(len(pos))
        vjp = {}
        for use_c in (True, False):
            cic.NATIVE = use_c
            try:
                vjp[use_c] = (cic.cic_read_vjp(mesh, pos, g, np.float64)[1],
                              cic.cic_paint_vjp(pos, shape, mesh, weight=g)[0])
            finally:
                cic.NATIVE = True
        for a, b in zip(vjp[True], vjp[False]):
            assert np.allclose(a, b, rtol=1e-12, atol=1e-12)
        # reads: the same float operations in the same order, bit for bit
        assert np.array_equal(out[True][0], out[False][0])
        for a, b in zip(out[True][1:], out[False][1:]):
            if dtype == np.float32:  # float64 sums cast to float32: identical
                assert np.array_equal(a, b)
            else:  # float64: only the order of the float64 additions differs
                assert np.allclose(a, b, rtol=1e-13, atol=1e-13)


def test_large_fixtures_are_self_consistent(golden):
    """The full-size oracle fixtures: float32 and float64 runs of the same
    initial conditions agree (P(k) to 1e-5 per bin at a = 0.1 and a = 1), and
    the sample's lattice points sit where the particles started."""
    import os
    from conftest import GOLDEN
    import glob
    paths = sorted(glob.glob(os.path.join(GOLDEN, "large_*_*.npz")))
    assert paths, "no full-size oracle fixture"
    for path in paths:
        n, steps = (int(v) for v in os.path.basename(path)[6:-4].split("_"))
        d = golden(os.path.basename(path))
        assert int(d["n"]) == n and int(d["steps"]) == steps
        for key in ("pk0", "pk1"):
            assert np.max(np.abs(d[f"{key}_32"] / d[f"{key}_64"] - 1)) < 1e-5
        i = d["sample"].astype(np.int64)
        lat = np.stack([i // (n * n), (i // n) % n, i % n], -1)
        assert np.max(np.abs(d["x0_64"] - lat)) < 0.1 * n  # 2LPT displacements are small
        kc, dc = nb.fpm_coefficients(cm.Cosmology(), 0.1, 1.0, steps)
        np.testing.assert_allclose(d["kick"], kc, rtol=1e-12)
        np.testing.assert_allclose(d["drift"], dc, rtol=1e-12)
