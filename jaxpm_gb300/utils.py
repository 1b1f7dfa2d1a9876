"""Power-spectrum metrics on the GPU (``jaxpm/utils.py:14-151``).

``power_spectrum`` bins the R2C half spectrum of the mesh with the
``pmgb_power_spectrum_f32`` kernel (float64 histograms); the bin edges,
normalisation and returned ``(kavg, pk)`` follow ``_initialize_pk`` and
``power_spectrum`` of the reference for the monopole of an auto spectrum.
``transfer`` follows ``:131-135``.
"""
import numpy as np
import torch

from . import _lib


def kedges_for(mesh_shape, box_shape, kedges=None):
    """Bin edges of ``_initialize_pk`` (``jaxpm/utils.py:41-50``)."""
    mesh_shape = np.asarray(mesh_shape)
    box_shape = np.asarray(box_shape, dtype=np.float64)
    kmax = np.pi * np.min(mesh_shape / box_shape)
    if kedges is None or isinstance(kedges, (int, float)):
        if kedges is None:
            dk = 2 * np.pi / np.min(box_shape) * 2
        elif isinstance(kedges, int):
            dk = kmax / (kedges + 1)
        else:
            dk = kedges
        kedges = np.arange(dk, kmax, dk) + dk / 2
    return np.asarray(kedges, dtype=np.float64)


def power_spectrum(mesh, mesh2=None, box_shape=None, kedges=None, multipoles=0,
                   los=(0., 0., 1.)):
    """Auto power spectrum ``(kavg, pk)`` of a float32 CUDA mesh."""
    if mesh2 is not None or np.ndim(multipoles) != 0 or multipoles != 0:
        raise NotImplementedError("only the monopole of an auto spectrum is computed on the GPU")
    mesh = mesh.to(torch.float32).contiguous()
    _lib.require_cuda(mesh)
    nx, ny, nz = mesh.shape
    box = np.array(mesh.shape, dtype=np.float64) if box_shape is None else \
        np.asarray(box_shape, dtype=np.float64)
    edges = kedges_for(mesh.shape, box, kedges)
    dev = mesh.device
    spec = torch.empty((nx, ny, nz // 2 + 1), dtype=torch.complex64, device=dev)
    s = _lib.stream()
    _lib.call("pmgb_fft_r2c_f32", _lib.ptr(mesh), _lib.ptr(spec), nx, ny, nz, 1, s)
    e_d = torch.tensor(edges, dtype=torch.float64, device=dev)
    nb = len(edges) + 1
    acc = torch.empty((3, nb), dtype=torch.float64, device=dev)
    _lib.call("pmgb_power_spectrum_f32", _lib.ptr(spec), nx, ny, nz, float(box[0]),
              float(box[1]), float(box[2]), _lib.ptr(e_d), len(edges), _lib.ptr(acc[0]),
              _lib.ptr(acc[1]), _lib.ptr(acc[2]), s)
    psum, cnt, ksum = acc.cpu().numpy()
    with np.errstate(invalid="ignore", divide="ignore"):
        kavg = (ksum / cnt)[1:-1]
        pk = (psum / cnt)[1:-1] * np.prod(box / np.array(mesh.shape))
    return kavg, pk


def transfer(mesh0, mesh1, box_shape, kedges=None):
    """``sqrt(P1/P0)`` per bin (``jaxpm/utils.py:131-135``)."""
    ks, pk0 = power_spectrum(mesh0, box_shape=box_shape, kedges=kedges)
    ks, pk1 = power_spectrum(mesh1, box_shape=box_shape, kedges=kedges)
    return ks, (pk1 / pk0)**.5
