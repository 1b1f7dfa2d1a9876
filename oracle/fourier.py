"""Fourier-space force solver, restated in NumPy (test infrastructure only).

Follows ``jaxpm/kernels.py:10-115``, ``jaxpm/distributed.py:37-42`` and
``jaxpm/pm.py:12-58``.  The transforms are complex-to-complex, as in the
reference (``fft3d`` is unnormalised, ``ifft3d`` normalised and its real
part taken), so the GPU's R2C/C2R path is checked against the reference's
own C2C formulation.
"""
import numpy as np
import scipy.fft as sfft

from . import cic

WORKERS = -1  # scipy.fft worker threads (-1: all host cores)


def fft3d(x):
    """``jaxdecomp.pfft3d`` (``jaxpm/distributed.py:37-38``): forward C2C."""
    return sfft.fftn(x, workers=WORKERS)


def ifft3d(x):
    """``jaxdecomp.pifft3d(x).real`` (``jaxpm/distributed.py:41-42``)."""
    return sfft.ifftn(x, workers=WORKERS).real


def fftk(shape, dtype=np.float32):
    """``fftk`` / ``fftfreq3d`` (``jaxpm/kernels.py:10-23``): per-axis wave
    numbers ``2*pi*fftfreq(n)`` in radians per cell, broadcast shapes
    ``[n,1,1]``, ``[1,n,1]``, ``[1,1,n]``."""
    out = []
    for d, n in enumerate(shape):
        k = (2 * np.pi * np.fft.fftfreq(n)).astype(dtype)
        s = [1, 1, 1]
        s[d] = n
        out.append(k.reshape(s))
    return out


def gradient_kernel(kvec, direction, order=1):
    """``jaxpm/kernels.py:41-66``: ``i*(8 sin w - sin 2w)/6`` (order 1) or
    ``i*k`` with the Nyquist entry zeroed (order 0)."""
    w = kvec[direction]
    if order == 0:
        wts = 1j * w
        flat = np.squeeze(wts).copy()
        flat[len(flat) // 2] = 0
        return flat.reshape(w.shape)
    dt = w.dtype.type
    a = dt(1 / 6.0) * (dt(8) * np.sin(w) - np.sin(dt(2) * w))
    return a * 1j


def invlaplace_kernel(kvec, fd=False):
    """``jaxpm/kernels.py:69-92``: ``-1/sum(k^2)`` with the k=0 mode zeroed;
    ``fd=True`` uses ``(k sinc(k/2pi))^2`` per axis."""
    if fd:
        kk = sum((ki * np.sinc(ki / (2 * np.pi)))**2 for ki in kvec)
    else:
        kk = sum(ki**2 for ki in kvec)
    kk_nozeros = np.where(kk == 0, 1, kk)
    return -np.where(kk == 0, 0, 1 / kk_nozeros)


def longrange_kernel(kvec, r_split):
    """``jaxpm/kernels.py:95-115``: ``exp(-k^2 r_split^2)``, or 1 when
    ``r_split == 0``."""
    if r_split != 0:
        kk = sum(ki**2 for ki in kvec)
        return np.exp(-kk * r_split**2)
    return 1.0


def force_mesh(delta_k, r_split=0.0, dtype=np.float32):
    """The three real-space force meshes of ``pm_forces``
    (``jaxpm/pm.py:49-56`` before the read): ``ifft3d(-grad_i * pot_k)``."""
    kvec = fftk(delta_k.shape, dtype)
    pot_k = delta_k * invlaplace_kernel(kvec) * longrange_kernel(kvec, r_split)
    cdt = np.complex64 if dtype == np.float32 else np.complex128
    return [ifft3d((-gradient_kernel(kvec, i) * pot_k).astype(cdt)).astype(dtype)
            for i in range(3)]


def pm_forces(positions, mesh_shape=None, delta=None, r_split=0.0,
              paint_absolute_pos=True, dtype=np.float32):
    """``pm_forces`` (``jaxpm/pm.py:12-58``) on one device.

    Paint (absolute or relative), forward FFT, potential
    ``delta_k * invlaplace * longrange``, three gradient multiplies, inverse
    FFTs, read at the particles; forces stacked on the last axis.
    """
    if mesh_shape is None:
        assert delta is not None
        mesh_shape = delta.shape
    if delta is None:
        if paint_absolute_pos:
            field = cic.cic_paint(np.zeros(mesh_shape, dtype), positions,
                                  dtype=dtype)
        else:
            field = cic.cic_paint_dx(positions, dtype=dtype)
        delta_k = fft3d(field)
    elif np.isrealobj(delta):
        delta_k = fft3d(np.asarray(delta, dtype))
    else:
        delta_k = delta
    meshes = force_mesh(delta_k, r_split, dtype)
    if paint_absolute_pos:
        return np.stack([cic.cic_read(m, positions, dtype) for m in meshes], -1)
    return np.stack([cic.cic_read_dx(m, positions, dtype) for m in meshes], -1)


def pm_forces_vjp(positions, mesh_shape, g, r_split=0.0, dtype=np.float64):
    """Vector-Jacobian product of ``pm_forces`` (absolute positions) w.r.t.
    positions: ``sum_i g_i . d F_i / d x``.

    Two terms: the read's (the gradient of the three force meshes at each
    particle) and the paint's (the gradient at each particle of
    ``rho_bar = sum_i A_i^T paint(g_i)``, with ``A_i^T`` the real-space
    operator of the conjugate multiplier ``conj(K_i)``)."""
    pos = np.asarray(positions, dtype=dtype).reshape(-1, 3)
    g = np.asarray(g, dtype=dtype).reshape(-1, 3)
    rho = cic.cic_paint(np.zeros(mesh_shape, dtype), pos, dtype=dtype)
    meshes = force_mesh(fft3d(rho), r_split, dtype)
    gpos = np.zeros_like(pos)
    rho_bar = np.zeros(mesh_shape, dtype)
    for i in range(3):
        gmesh, gp = cic.cic_read_vjp(meshes[i], pos, g[:, i], dtype)
        gpos += gp
        K = kspace_multiplier(mesh_shape, i, r_split, dtype)
        rho_bar += ifft3d(np.conj(K) * fft3d(gmesh))
    gpos += cic.cic_paint_vjp(pos, mesh_shape, rho_bar, dtype=dtype)[0]
    return gpos


def kspace_multiplier(shape, direction, r_split=0.0, dtype=np.float64):
    """The complex multiplier ``K_i(k) = -grad_i(k) * invlaplace(k) *
    longrange(k)`` on the full C2C grid (used by the adjoint checks)."""
    kvec = fftk(shape, dtype)
    return (-gradient_kernel(kvec, direction) * invlaplace_kernel(kvec) *
            longrange_kernel(kvec, r_split))
