"""Binned power spectrum, restated in NumPy (test infrastructure only).

Follows ``jaxpm/utils.py:14-128`` (``_initialize_pk`` and
``power_spectrum``) for auto spectra of the monopole.
"""
import numpy as np
import scipy.fft as sfft


def power_spectrum(mesh, box_shape=None, kedges=None):
    """Returns ``(kavg, pk)`` as ``power_spectrum(mesh, box_shape=...,
    kedges=...)`` with ``multipoles=0``."""
    mesh = np.asarray(mesh)
    mesh_shape = np.array(mesh.shape)
    box_shape = mesh_shape if box_shape is None else np.asarray(box_shape, dtype=np.float64)
    kmax = np.pi * np.min(mesh_shape / box_shape)
    if kedges is None or isinstance(kedges, (int, float)):
        if kedges is None:
            dk = 2 * np.pi / np.min(box_shape) * 2
        elif isinstance(kedges, int):
            dk = kmax / (kedges + 1)
        else:
            dk = kedges
        kedges = np.arange(dk, kmax, dk) + dk / 2
    kshapes = np.eye(3, dtype=np.int32) * -2 + 1
    kvec = [(2 * np.pi * m / l) * np.fft.fftfreq(m).reshape(ks)
            for m, l, ks in zip(mesh_shape, box_shape, kshapes)]
    # jnp.sqrt of the float64 sum runs in float32 (x64 disabled by default)
    kmesh = np.sqrt(sum(ki**2 for ki in kvec).astype(np.float32)).astype(np.float64)
    dig = np.digitize(kmesh.reshape(-1), kedges)
    kcount = np.bincount(dig, minlength=len(kedges) + 1)
    kavg = np.bincount(dig, weights=kmesh.reshape(-1), minlength=len(kedges) + 1) / kcount
    kavg = kavg[1:-1]
    meshk = sfft.fftn(mesh, norm='ortho', workers=-1)
    mmk = meshk.real**2 + meshk.imag**2
    n_bins = len(kavg) + 2
    psum = np.bincount(dig, weights=mmk.reshape(-1), minlength=n_bins)[:n_bins]
    pk = (psum / kcount)[1:-1] * (box_shape / mesh_shape).prod()
    return kavg, pk
