"""Regenerates the full-size oracle fixtures ``large_<n>_<steps>.npz`` in this
folder.

Two workloads, both Planck15 cosmology, particles = cells, white noise from
NumPy PCG64 seed 0 coloured by the Eisenstein-Hu P(k) on
``logspace(-4, 1, 128)``, 2LPT to a = 0.1, then 20 (or the given number of) FastPM
steps linear in a up to a = 1 (``jaxpm/pm.py:61-144``, ``jaxpm/ode.py:13-82``):

* 256^3 particles on a 256^3 mesh, box 256 Mpc/h (the single-simulation
  throughput configuration);
* 512^3 particles on a 512^3 mesh, box 512 Mpc/h (the benchmark's
  default workload at 20 steps).

Each is run twice by the NumPy oracle, in float32 (the reference's dtype)
and in float64 (the accuracy reference), and the fixture keeps, per run:
the binned P(k) of the a = 0.1 and a = 1 CIC densities
(``jaxpm/utils.py:14-128``), and the positions and velocities of 4096
particles drawn once (PCG64 seed 123) at a = 0.1 and a = 1, in the
caller's (lattice) order.  The GPU tests and ``bench.py`` rebuild the same
initial conditions from the same seed and compare against these arrays.

Run from the repository root (about 3 minutes for 256^3 and 25 for 512^3
on 8 cores): ``python tests/golden/make_large_golden.py [256] [512] [512:40]``
(``n:steps`` picks another step count).
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import cic, cosmology as cm, nbody as nb, power  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
A0, A1 = 0.1, 1.0
SEED = 0
N_SAMPLE = 4096


def sample_indices(n):
    return np.sort(np.random.Generator(np.random.PCG64(123)).choice(n**3, N_SAMPLE,
                                                                  replace=False))


def run(n, steps, dtype, log):
    cosmo = cm.Cosmology()
    box = [float(n)] * 3
    k = np.logspace(-4, 1, 128)
    pk = cm.linear_matter_power(cosmo, k)
    noise = np.random.Generator(np.random.PCG64(SEED)).standard_normal((n,) * 3,
                                                                        dtype=np.float32)
    t = time.time()
    ic = nb.linear_field(noise.astype(dtype), box, k, pk, dtype)
    lat = cic.lattice((n,) * 3).reshape(-1, 3).astype(dtype)
    dx, p, _ = nb.lpt(cosmo, ic, lat, a=A0, order=2, dtype=dtype)
    del ic
    x = (lat + dx).astype(dtype)
    v = p.astype(dtype)
    del lat, dx, p
    idx = sample_indices(n)
    out = {"x0": x[idx].copy(), "v0": v[idx].copy()}
    rho = cic.cic_paint(np.zeros((n,) * 3, dtype), x, dtype=dtype)
    out["k"], out["pk0"] = power.power_spectrum(rho, box_shape=box)
    del rho
    log(f"{n}^3 {np.dtype(dtype).name}: initial state in {time.time() - t:.0f} s")
    kc, dc = nb.fpm_coefficients(cosmo, A0, A1, steps)
    for i in range(steps):
        x, v = nb.fpm_step(x, v, (n,) * 3, kc[i], dc[i], dtype=dtype)
    rho = cic.cic_paint(np.zeros((n,) * 3, dtype), x, dtype=dtype)
    _, out["pk1"] = power.power_spectrum(rho, box_shape=box)
    out["x1"], out["v1"] = x[idx].copy(), v[idx].copy()
    log(f"{n}^3 {np.dtype(dtype).name}: {steps} steps done at {time.time() - t:.0f} s")
    return out, kc, dc, idx


def main(cases):
    for n, steps in cases:
        res = {}
        for dtype in (np.float32, np.float64):
            out, kc, dc, idx = run(n, steps, dtype, lambda m: print(m, flush=True))
            tag = "32" if dtype == np.float32 else "64"
            for key, val in out.items():
                res[key if key == "k" else f"{key}_{tag}"] = val
        res.update(n=n, box=float(n), steps=steps, a0=A0, a1=A1, seed=SEED, kick=kc,
                   drift=dc, sample=idx)
        path = os.path.join(OUT, f"large_{n}_{steps}.npz")
        np.savez_compressed(path, **res)
        rel = np.abs(res["pk1_32"] / res["pk1_64"] - 1)
        print(f"wrote {path}; float32 vs float64 final P(k): max rel dev {rel.max():.2e}",
              flush=True)


if __name__ == "__main__":
    args = sys.argv[1:] or ["256", "512"]
    main([(int(a.split(":")[0]), int(a.split(":")[1]) if ":" in a else 20) for a in args])
