"""Golden vectors from the reference itself, for a machine where JAX imports.

The reference (JaxPM) needs ``jax``, ``jaxlib``, ``jax_cosmo`` and
``jaxdecomp``; none of them can be installed where this project is built,
so the oracle is checked against analytic known answers and its own frozen
fixtures only.  This script closes that gap wherever the reference does
import: it runs the reference's own functions on the inputs of the oracle's
fixtures (``cic.npz``, ``pm_forces16.npz``, ``sim16.npz``, ``growth.npz``
in this folder) and writes their outputs to ``reference_jaxpm.npz``;
``tests/test_reference_pin.py`` then compares the oracle with them
(skipped while the file does not exist).

What it calls, per fixture:

* ``jaxpm.painting._cic_paint_impl`` / ``_cic_read_impl`` on the edge-case
  particles (``painting.py:15-45``, ``:78-106``) and ``cic_paint_dx`` /
  ``cic_read_dx`` on the relative-mode displacements (``:161-260``);
* ``jaxpm.pm.pm_forces`` on the 16^3 positions, with and without
  ``r_split`` (``pm.py:12-58``), in float64 (x64 enabled) and float32;
* ``jaxpm.pm.lpt`` orders 1 and 2 at a = 0.1 on the 16^3 initial field
  (``pm.py:61-126``), and five FastPM steps driven with the closures of
  ``jaxpm.ode.symplectic_fpm_ode`` (``ode.py:13-82``): first_kick at a0,
  then drift / kick on the grid a_i = a0 + i dt;
* jax_cosmo's growth factors and ``jaxpm.growth.Gf``/``dGfa``/``gp`` on a
  grid of scale factors.

Usage: ``python tests/golden/make_reference_golden.py <path to JaxPM>``.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    sys.path.insert(0, ref_root)
    import jax
    jax.config.update("jax_enable_x64", True)
    import jax.numpy as jnp
    import jax_cosmo as jc
    from jaxpm import growth, painting, pm
    from jaxpm.ode import symplectic_fpm_ode

    out = {}
    cic = np.load(os.path.join(HERE, "cic.npz"))
    for tag in ("cube", "rect"):
        pos = jnp.asarray(cic[f"{tag}_pos"], dtype=jnp.float32)
        mesh = jnp.asarray(cic[f"{tag}_mesh"], dtype=jnp.float32)
        wts = jnp.asarray(cic[f"{tag}_weights"], dtype=jnp.float64)
        shape = mesh.shape
        out[f"{tag}_paint64"] = np.asarray(painting._cic_paint_impl(
            jnp.zeros(shape, jnp.float64), pos.astype(jnp.float64), wts))
        out[f"{tag}_read32"] = np.asarray(painting._cic_read_impl(mesh, pos))
        disp = jnp.asarray(cic[f"{tag}_disp"], dtype=jnp.float32)
        out[f"{tag}_rel_paint32"] = np.asarray(painting.cic_paint_dx(disp))
        out[f"{tag}_rel_read32"] = np.asarray(painting.cic_read_dx(mesh, disp))

    f16 = np.load(os.path.join(HERE, "pm_forces16.npz"))
    pos = jnp.asarray(f16["pos"], dtype=jnp.float32)
    shape = (16, 16, 16)
    out["forces32"] = np.asarray(pm.pm_forces(pos, mesh_shape=shape))
    out["forces64"] = np.asarray(pm.pm_forces(pos.astype(jnp.float64), mesh_shape=shape))
    out["forces64_rsplit"] = np.asarray(pm.pm_forces(pos.astype(jnp.float64),
                                                     mesh_shape=shape, r_split=1.5))

    sim = np.load(os.path.join(HERE, "sim16.npz"))
    cosmo = jc.Planck15(Omega_c=0.2589, Omega_b=0.0486, h=0.6774, n_s=0.9667, sigma8=0.8159)
    ic = jnp.asarray(sim["ic"], dtype=jnp.float32)
    lat = jnp.stack(jnp.meshgrid(*[jnp.arange(16.0)] * 3, indexing="ij"),
                    axis=-1).reshape(-1, 3).astype(jnp.float32)
    for order in (1, 2):
        dx, p, f = pm.lpt(cosmo, ic, particles=lat, a=0.1, order=order)
        out[f"dx{order}"], out[f"p{order}"], out[f"f{order}"] = (np.asarray(dx), np.asarray(p),
                                                                 np.asarray(f))
    a0, a1, n = 0.1, 1.0, 5
    dt = (a1 - a0) / n
    drift, kick, first_kick = symplectic_fpm_ode(shape, dt, cosmo, paint_absolute_pos=True)
    x, v = lat + jnp.asarray(out["dx2"]), jnp.asarray(out["p2"])
    ac = a0
    v = v + dt * first_kick(ac, x, cosmo)
    for i in range(n):
        x = x + dt * drift(ac, v, cosmo)
        if i + 1 < n:
            v = v + dt * kick(ac, x, cosmo)
        ac = ac + dt
    out["final_pos"], out["final_vel"] = np.asarray(x), np.asarray(v)

    grid = np.linspace(0.05, 1.1, 23)
    a = jnp.asarray(grid)
    out["a"] = grid
    out["growth_factor"] = np.asarray(jc.background.growth_factor(cosmo, a))
    out["growth_rate"] = np.asarray(jc.background.growth_rate(cosmo, a))
    out["Gf"] = np.asarray(growth.Gf(cosmo, a))
    out["dGfa"] = np.asarray(growth.dGfa(cosmo, a))
    out["gp"] = np.asarray(growth.gp(cosmo, a))
    np.savez_compressed(os.path.join(HERE, "reference_jaxpm.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_jaxpm.npz"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    main(sys.argv[1])
