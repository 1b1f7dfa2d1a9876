"""Regenerates the golden fixtures in this folder from the NumPy oracle.

The reference (JAX) cannot run where this project is built, and it ships
no golden vectors, so these fixtures freeze the oracle's outputs on fixed
inputs: they pin the oracle against accidental change and give the GPU
tests exact expected values.  Run from the repository root:
``python tests/golden/make_golden.py``.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import cic, cosmology as cm, fourier as fo, nbody as nb  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def edge_positions(shape):
    """Particles at cell centres, on faces, on corners, at the periodic wrap
    (N - eps, -eps, exactly N, negative cells) and random ones."""
    n = np.array(shape, dtype=np.float32)
    eps = np.float32(1e-4)
    pts = [
        [0.5, 0.5, 0.5], [0.0, 0.0, 0.0], [1.0, 2.0, 3.0], [2.5, 0.0, 1.25],
        [n[0] - eps, n[1] - eps, n[2] - eps], [-eps, -eps, -eps], [n[0], 0.0, n[2]],
        [-1.5, -2.25, 3.75], [n[0] + 0.5, n[1] + 1.75, -0.5], [0.999999, 1.0000001, 7.9999995],
        [3 * n[0] + 0.3, -2 * n[1] - 0.7, 0.1],
    ]
    rng = np.random.default_rng(1234)
    rnd = rng.uniform(-2, 1, size=(53, 3)) * n + rng.uniform(0, 1, size=(53, 3))
    return np.concatenate([np.array(pts, np.float32), rnd.astype(np.float32)])


def main():
    cosmo = cm.Cosmology()
    out = {}
    for tag, shape in [("cube", (8, 8, 8)), ("rect", (8, 6, 10))]:
        pos = edge_positions(shape)
        idx, w = cic.cic_weights(pos, shape, np.float32)
        rng = np.random.default_rng(7)
        mesh = rng.standard_normal(shape).astype(np.float32)
        wts = rng.uniform(0.5, 1.5, size=len(pos)).astype(np.float32)
        out[f"{tag}_pos"] = pos
        out[f"{tag}_idx"] = idx
        out[f"{tag}_w"] = w
        out[f"{tag}_mesh"] = mesh
        out[f"{tag}_weights"] = wts
        out[f"{tag}_paint64"] = cic.cic_paint(np.zeros(shape), pos.astype(np.float64), weight=wts,
                                              dtype=np.float64)
        out[f"{tag}_read32"] = cic.cic_read(mesh, pos, np.float32)
        disp = rng.uniform(-3, 3, size=(*shape, 3)).astype(np.float32)
        disp.reshape(-1, 3)[:4] = [[-1e-7, 0, 0], [0, -1e-9, 0], [0.9999999, 0, 0], [0, 0, -2.5]]
        ridx, rw = cic.enmesh(cic.lattice(shape), disp, shape, np.float32)
        out[f"{tag}_disp"] = disp
        out[f"{tag}_rel_idx"] = ridx
        out[f"{tag}_rel_w"] = rw
        # float32 enmesh arithmetic (the reference's dtype: its wrap rounds
        # -1e-9 up to L and drops that neighbour), float64 accumulation
        out[f"{tag}_rel_paint32"] = cic.cic_paint_dx(disp, dtype=np.float32)
    np.savez_compressed(os.path.join(OUT, "cic.npz"), **out)

    # pm_forces on a 16^3 mesh, float64 oracle (C2C as the reference)
    n = 16
    rng = np.random.default_rng(11)
    pos = (cic.lattice((n,) * 3).reshape(-1, 3) +
           rng.normal(0, 1.5, size=(n**3, 3))).astype(np.float32)
    f64 = fo.pm_forces(pos.astype(np.float64), mesh_shape=(n,) * 3, dtype=np.float64)
    f64_rs = fo.pm_forces(pos.astype(np.float64), mesh_shape=(n,) * 3, r_split=1.5,
                          dtype=np.float64)
    f32 = fo.pm_forces(pos, mesh_shape=(n,) * 3, dtype=np.float32)
    np.savez_compressed(os.path.join(OUT, "pm_forces16.npz"), pos=pos, forces64=f64,
                        forces64_rsplit=f64_rs, forces32=f32)

    # LPT and a short FastPM run on 16^3 (box 64), float32 oracle
    k = np.logspace(-4, 1, 128)
    pk = cm.linear_matter_power(cosmo, k)
    noise = np.random.default_rng(3).standard_normal((n,) * 3).astype(np.float32)
    ic = nb.linear_field(noise, [64.0] * 3, k, pk)
    lat = cic.lattice((n,) * 3).reshape(-1, 3).astype(np.float32)
    dx1, p1, f1 = nb.lpt(cosmo, ic, lat, a=0.1, order=1)
    dx2, p2, f2 = nb.lpt(cosmo, ic, lat, a=0.1, order=2)
    kc, dc = nb.fpm_coefficients(cosmo, 0.1, 1.0, 5)
    x, v = lat + dx2, p2
    for i in range(5):
        x, v = nb.fpm_step(x, v, (n,) * 3, kc[i], dc[i])
    rho = cic.cic_paint(np.zeros((n,) * 3, np.float32), x)
    np.savez_compressed(os.path.join(OUT, "sim16.npz"), noise=noise, pk_k=k, pk_p=pk, ic=ic,
                        dx1=dx1, p1=p1, f1=f1, dx2=dx2, p2=p2, f2=f2, kick=kc, drift=dc,
                        final_pos=x, final_vel=v, final_rho=rho)

    t = cm.growth_tables(cosmo)
    np.savez_compressed(os.path.join(OUT, "growth.npz"), a=t[0], g=t[1], f=t[2], h=t[3],
                        g2=t[4], f2=t[5], h2=t[6])
    print("wrote fixtures to", OUT)


if __name__ == "__main__":
    main()
