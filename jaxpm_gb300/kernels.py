"""Fourier-space multipliers with jaxpm's call surface
(``jaxpm/kernels.py:10-115``), evaluated as CUDA tensors.

These exist so that code written against ``jaxpm.kernels`` keeps working;
the force path itself applies them inside the fused k-space kernel
(``pmgb_kspace_forces_f32``) without materialising them.  ``fftk`` returns
the wave numbers of the half spectrum layout ``[nx, ny, nz//2+1]`` used by
``distributed.fft3d``: ``2*pi*fftfreq(n)`` in radians per cell on the first
two axes and the first ``nz//2+1`` entries of it on the last.
"""
import math

import numpy as np
import torch


def fftk(mesh_shape, device="cuda"):
    """``[kx [nx,1,1], ky [1,ny,1], kz [1,1,nz//2+1]]`` (float32)."""
    out = []
    for d, n in enumerate(mesh_shape):
        k = (2 * np.pi * np.fft.fftfreq(n)).astype(np.float32)
        if d == 2:
            k = k[:n // 2 + 1]
        shape = [1, 1, 1]
        shape[d] = len(k)
        out.append(torch.tensor(k, device=device).reshape(shape))
    return out


def gradient_kernel(kvec, direction, order=1):
    """``i (8 sin w - sin 2w)/6`` (order 1) or ``i k`` with the Nyquist
    entry zeroed (order 0) (``jaxpm/kernels.py:41-66``)."""
    w = kvec[direction]
    if order == 0:
        flat = w.reshape(-1).clone()
        n = flat.numel() if direction < 2 else 2 * (flat.numel() - 1)
        if n // 2 < flat.numel():
            flat[n // 2] = 0
        return (1j * flat).reshape(w.shape)
    return (1.0 / 6.0 * (8 * torch.sin(w) - torch.sin(2 * w))) * 1j


def invlaplace_kernel(kvec, fd=False):
    """``-1/k^2`` with k=0 -> 0 (``jaxpm/kernels.py:69-92``)."""
    if fd:
        kk = sum((ki * torch.sinc(ki / (2 * math.pi)))**2 for ki in kvec)
    else:
        kk = sum(ki**2 for ki in kvec)
    kk_nozeros = torch.where(kk == 0, torch.ones_like(kk), kk)
    return -torch.where(kk == 0, torch.zeros_like(kk), 1 / kk_nozeros)


def longrange_kernel(kvec, r_split):
    """``exp(-k^2 r_split^2)`` or 1 (``jaxpm/kernels.py:95-115``)."""
    if r_split != 0:
        kk = sum(ki**2 for ki in kvec)
        return torch.exp(-kk * r_split**2)
    return 1.0
