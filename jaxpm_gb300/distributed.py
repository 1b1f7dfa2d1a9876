"""Single-GPU counterparts of ``jaxpm/distributed.py``: FFTs, particle
lattices and white noise.

``fft3d``/``ifft3d`` (``jaxpm/distributed.py:37-42``) are cuFFT R2C/C2R
here: ``fft3d`` of a real mesh returns its half spectrum
``[nx, ny, nz//2+1]`` (complex64) and ``ifft3d`` maps a half spectrum back
to the real mesh, normalised, i.e. ``jaxpm``'s ``pifft3d(x).real``.  Both
are differentiable.  ``uniform_particles`` and ``normal_field`` follow
``:168-223`` on one device; white noise comes from NumPy's PCG64 generator
seeded with an integer (the same field can then be fed to any other
implementation), not from ``jax.random``.
"""
import numpy as np
import torch

from . import _lib
from .painting import _single_device


def _half_weights(nz, device):
    """Multiplicity of each kz plane of a half spectrum in the full one."""
    w = torch.full((nz // 2 + 1,), 2.0, dtype=torch.float32, device=device)
    w[0] = 1.0
    if nz % 2 == 0:
        w[-1] = 1.0
    return w


class _R2C(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x):
        nx, ny, nz = x.shape
        out = torch.empty((nx, ny, nz // 2 + 1), dtype=torch.complex64, device=x.device)
        _lib.call("pmgb_fft_r2c_f32", _lib.ptr(x), _lib.ptr(out), nx, ny, nz, 1, _lib.stream())
        ctx.nz = nz
        return out

    @staticmethod
    def backward(ctx, g):
        # adjoint of R2C: real part of the inverse sum over the half
        # spectrum, i.e. an unnormalised C2R of g divided by the multiplicity
        nx, ny, _ = g.shape
        spec = (g.resolve_conj() / _half_weights(ctx.nz, g.device)).contiguous()
        out = torch.empty((nx, ny, ctx.nz), dtype=torch.float32, device=g.device)
        _lib.call("pmgb_fft_c2r_f32", _lib.ptr(spec), _lib.ptr(out), nx, ny, ctx.nz, 1, 0,
                  _lib.stream())
        return out


class _C2R(torch.autograd.Function):
    @staticmethod
    def forward(ctx, spec, nz):
        nx, ny, _ = spec.shape
        tmp = spec.clone()  # cuFFT C2R overwrites its input
        out = torch.empty((nx, ny, nz), dtype=torch.float32, device=spec.device)
        _lib.call("pmgb_fft_c2r_f32", _lib.ptr(tmp), _lib.ptr(out), nx, ny, nz, 1, 1,
                  _lib.stream())
        ctx.nz = nz
        return out

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous()
        nx, ny, nz = g.shape
        spec = torch.empty((nx, ny, nz // 2 + 1), dtype=torch.complex64, device=g.device)
        _lib.call("pmgb_fft_r2c_f32", _lib.ptr(g), _lib.ptr(spec), nx, ny, nz, 1, _lib.stream())
        spec = spec * (_half_weights(nz, g.device) / float(nx * ny * nz))
        return spec, None


def fft3d(x):
    """Forward 3-D FFT of a real float32 mesh: the half spectrum
    ``[nx, ny, nz//2+1]`` (unnormalised)."""
    if x.dtype != torch.float32:
        raise TypeError("fft3d takes a real float32 mesh")
    x = x.contiguous()
    _lib.require_cuda(x)
    return _R2C.apply(x)


def ifft3d(x, nz=None):
    """Normalised inverse of ``fft3d``: half spectrum to real mesh.  The
    last mesh dimension defaults to ``2*(x.shape[-1]-1)`` (even sizes)."""
    if x.dtype != torch.complex64:
        raise TypeError("ifft3d takes a complex64 half spectrum")
    x = x.contiguous()
    _lib.require_cuda(x)
    nz = 2 * (x.shape[-1] - 1) if nz is None else int(nz)
    if nz // 2 + 1 != x.shape[-1]:
        raise ValueError(f"half spectrum of last size {x.shape[-1]} does not match nz={nz}")
    return _C2R.apply(x, nz)


FFT_PATHS = {"cufft": 0, "fused": 1, "own": 2}


def fft_path():
    """FFT path of the composite force calls: ``"cufft"`` (cuFFT 3-D
    transforms around the k-space kernel), ``"fused"`` (default: cuFFT's 2-D
    plane transforms around the library's x-direction kernel, which fuses
    the forward x transform, the force multiplies and the inverse x
    transforms) or ``"own"`` (the library's plane kernels as well).  The
    last two apply to the mesh shapes ``fft3_supported`` accepts."""
    return {v: k for k, v in FFT_PATHS.items()}[_lib.load().pmgb_fft_path()]


def set_fft_path(path):
    """Selects the FFT path of the composite force calls (process-wide);
    returns the previous one."""
    prev = fft_path()
    _lib.call("pmgb_set_fft_path", FFT_PATHS[path])
    return prev


def fft3_supported(mesh_shape):
    """Whether the library's own FFT pipeline handles this mesh shape."""
    return bool(_lib.load().pmgb_fft3_supported(*(int(s) for s in mesh_shape)))


def uniform_particles(mesh_shape, sharding=None, device="cuda"):
    """Lattice positions ``[*mesh_shape, 3]`` (``jaxpm/distributed.py:168-190``)."""
    _single_device(0, sharding)
    axes = [torch.arange(s, dtype=torch.float32, device=device) for s in mesh_shape]
    return torch.stack(torch.meshgrid(*axes, indexing="ij"), dim=-1).contiguous()


def normal_field(seed, shape, sharding=None, device="cuda"):
    """Standard-normal white noise of ``shape`` from NumPy's PCG64 generator
    seeded with ``seed`` (``jaxpm/distributed.py:193-223`` draws it with
    ``jax.random.normal``), as a float32 CUDA tensor."""
    _single_device(0, sharding)
    rng = np.random.Generator(np.random.PCG64(int(seed)))
    noise = rng.standard_normal(tuple(shape), dtype=np.float32)
    return torch.from_numpy(noise).to(device)
