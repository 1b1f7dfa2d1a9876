"""Particle-mesh forces, LPT and linear initial conditions on the GPU, with
jaxpm's call surface (``jaxpm/pm.py``).

``pm_forces`` (``jaxpm/pm.py:12-58``) runs, for absolute positions, as one
library call: paint -> R2C -> fused k-space kernel (Laplace inverse,
long-range filter and the three gradients in one pass) -> batched C2R ->
one gather of all three components.  Its gradient is the hand-written
``pmgb_pm_forces_vjp_f32``.  ``lpt`` (``:61-126``) and ``linear_field``
(``:129-144``) are built from the same kernels plus the 2LPT source and
white-noise colouring kernels.  Arrays are float32 CUDA tensors; a complex
``delta`` is a half spectrum as returned by ``distributed.fft3d``.
"""
import numpy as np
import torch

from . import _lib
from . import growth as gr
from .distributed import fft3d, ifft3d, normal_field
from .painting import MODES, _mode, _single_device, cic_read_dx


def _ws(nbytes, device):
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)


class _PMForces(torch.autograd.Function):
    """Forces at absolute positions; backward = pmgb_pm_forces_vjp_f32."""

    @staticmethod
    def forward(ctx, pos, mesh_shape, r_split, mode):
        nx, ny, nz = mesh_shape
        p = pos.reshape(-1, 3)
        _lib.require_cuda(p)
        n = p.shape[0]
        wsb = _lib.load().pmgb_pm_workspace_size(nx, ny, nz, n, mode)
        ws = _ws(wsb, p.device)
        out = torch.empty_like(p)
        _lib.call("pmgb_pm_forces_f32", _lib.ptr(p), n, nx, ny, nz, float(r_split), mode,
                  _lib.ptr(out), _lib.ptr(ws), wsb, _lib.stream())
        ctx.save_for_backward(p)
        ctx.args = (mesh_shape, float(r_split), mode, pos.shape)
        return out.reshape(pos.shape)

    @staticmethod
    def backward(ctx, g):
        (p,) = ctx.saved_tensors
        (nx, ny, nz), r_split, mode, shape = ctx.args
        g = g.contiguous().reshape(-1, 3)
        n = p.shape[0]
        wsb = _lib.load().pmgb_pm_workspace_size(nx, ny, nz, n, mode)
        ws = _ws(wsb, p.device)
        gpos = torch.empty_like(p)
        _lib.call("pmgb_pm_forces_vjp_f32", _lib.ptr(p), n, nx, ny, nz, r_split, mode,
                  _lib.ptr(g), _lib.ptr(gpos), _lib.ptr(ws), wsb, _lib.stream())
        return gpos.reshape(shape), None, None, None


class _ForceMeshes(torch.autograd.Function):
    """Real density mesh -> three real force meshes [3, nx, ny, nz]
    (``pmgb_mesh_forces_f32``: the library's fused FFT pipeline, or R2C +
    fused k-space kernel + batched C2R).  Linear; the adjoint is
    ``pmgb_mesh_forces_vjp_f32``."""

    @staticmethod
    def forward(ctx, rho, r_split):
        nx, ny, nz = rho.shape
        nb = _lib.load().pmgb_mesh_forces_workspace_size(nx, ny, nz)
        ws = torch.empty(nb, dtype=torch.uint8, device=rho.device)
        out = torch.empty((3, nx, ny, nz), dtype=torch.float32, device=rho.device)
        _lib.call("pmgb_mesh_forces_f32", _lib.ptr(rho), _lib.ptr(out), nx, ny, nz,
                  float(r_split), _lib.ptr(ws), nb, _lib.stream())
        ctx.r_split = float(r_split)
        return out

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous()
        _, nx, ny, nz = g.shape
        nb = _lib.load().pmgb_mesh_forces_workspace_size(nx, ny, nz)
        ws = torch.empty(nb, dtype=torch.uint8, device=g.device)
        out = torch.empty((nx, ny, nz), dtype=torch.float32, device=g.device)
        _lib.call("pmgb_mesh_forces_vjp_f32", _lib.ptr(g), _lib.ptr(out), nx, ny, nz,
                  ctx.r_split, _lib.ptr(ws), nb, _lib.stream())
        return out, None


class _Read3(torch.autograd.Function):
    """Gather of three meshes [3, nx, ny, nz] at positions -> [Np, 3]."""

    @staticmethod
    def forward(ctx, f3, pos):
        _, nx, ny, nz = f3.shape
        p = pos.reshape(-1, 3)
        out = torch.empty_like(p)
        _lib.call("pmgb_cic_read3_f32", _lib.ptr(f3), nx * ny * nz, nx, ny, nz, _lib.ptr(p),
                  p.shape[0], _lib.ptr(out), _lib.stream())
        ctx.save_for_backward(f3, p)
        ctx.shape = pos.shape
        return out.reshape(pos.shape)

    @staticmethod
    def backward(ctx, g):
        f3, p = ctx.saved_tensors
        g = g.contiguous().reshape(-1, 3)
        _, nx, ny, nz = f3.shape
        gf = torch.zeros_like(f3) if ctx.needs_input_grad[0] else None
        gp = torch.zeros_like(p) if ctx.needs_input_grad[1] else None
        s = _lib.stream()
        for c in range(3):
            gc = g[:, c].contiguous()
            tmp = torch.empty_like(p) if gp is not None else None
            _lib.call("pmgb_cic_read_vjp_f32", _lib.ptr(f3[c]), nx, ny, nz, _lib.ptr(p),
                      p.shape[0], _lib.ptr(gc), _lib.ptr(gf[c] if gf is not None else None),
                      _lib.ptr(tmp), s)
            if gp is not None:
                gp += tmp
        return gf, (gp.reshape(ctx.shape) if gp is not None else None)


def force_meshes(rho, r_split=0.0):
    """The three real-space force meshes ``ifft3d(-grad_i * invlaplace *
    longrange * fft3d(rho))`` (``jaxpm/pm.py:49-56`` before the read)."""
    rho = rho.contiguous()
    _lib.require_cuda(rho)
    return _ForceMeshes.apply(rho, r_split)


def pm_forces(positions, mesh_shape=None, delta=None, r_split=0, paint_absolute_pos=True,
              halo_size=0, sharding=None, paint_mode="atomic"):
    """``jaxpm.pm.pm_forces``: gravitational forces at the particles, in mesh
    units, stacked on the last axis.  ``paint_mode`` picks the painter
    (``"atomic"``, ``"binned"``, ``"deterministic"``)."""
    _single_device(halo_size, sharding)
    if mesh_shape is None:
        assert (delta is not None), "If mesh_shape is not provided, delta should be provided"
        if delta.is_complex():
            mesh_shape = (delta.shape[0], delta.shape[1], 2 * (delta.shape[2] - 1))
        else:
            mesh_shape = tuple(delta.shape)
    mesh_shape = tuple(int(s) for s in mesh_shape)
    mode = _mode(paint_mode)
    if delta is None and paint_absolute_pos:
        if positions.dtype != torch.float32:
            raise TypeError("positions must be float32")
        return _PMForces.apply(positions.contiguous(), mesh_shape, r_split, mode)
    if delta is None:
        from .painting import cic_paint_dx
        rho = cic_paint_dx(positions)
    elif delta.is_complex():
        rho = ifft3d(delta, mesh_shape[2])
    else:
        rho = delta
    f3 = force_meshes(rho.to(torch.float32), r_split)
    if paint_absolute_pos:
        return _Read3.apply(f3, positions.contiguous())
    return torch.stack([cic_read_dx(f3[i], positions) for i in range(3)], dim=-1)


def _lpt_scalars(cosmo, a):
    a = float(np.asarray(a).reshape(-1)[0])
    E = float(gr.E(cosmo, a))
    D1 = float(gr.growth_factor(cosmo, a))
    f1 = float(gr.growth_rate(cosmo, a))
    return a, E, D1, f1


def _combine(x, y, cx, cy):
    out = torch.empty_like(x)
    _lib.call("pmgb_lpt_combine_f32", _lib.ptr(x), _lib.ptr(y), x.numel(), float(cx),
              float(cy), _lib.ptr(out), _lib.stream())
    return out


class _Source2LPT(torch.autograd.Function):
    """Real linear field -> 2LPT source delta2 (``jaxpm/pm.py:88-109``)."""

    @staticmethod
    def forward(ctx, ic):
        nx, ny, nz = ic.shape
        dk = torch.empty((nx, ny, nz // 2 + 1), dtype=torch.complex64, device=ic.device)
        s = _lib.stream()
        _lib.call("pmgb_fft_r2c_f32", _lib.ptr(ic), _lib.ptr(dk), nx, ny, nz, 1, s)
        wsb = _lib.load().pmgb_lpt2_source_workspace_size(nx, ny, nz)
        ws = _ws(wsb, ic.device)
        out = torch.empty_like(ic)
        _lib.call("pmgb_lpt2_source_f32", _lib.ptr(dk), _lib.ptr(out), nx, ny, nz, _lib.ptr(ws),
                  wsb, s)
        ctx.save_for_backward(ic)
        return out

    @staticmethod
    def backward(ctx, g):
        """pmgb_lpt2_source_vjp_f32 (recomputes the six shear meshes)."""
        (ic,) = ctx.saved_tensors
        nx, ny, nz = ic.shape
        g = g.to(torch.float32).contiguous()
        wsb = _lib.load().pmgb_lpt2_source_workspace_size(nx, ny, nz)
        ws = _ws(wsb, ic.device)
        out = torch.empty_like(ic)
        _lib.call("pmgb_lpt2_source_vjp_f32", _lib.ptr(ic), _lib.ptr(g), _lib.ptr(out), nx, ny,
                  nz, _lib.ptr(ws), wsb, _lib.stream())
        return out


def lpt(cosmo, initial_conditions, particles=None, a=0.1, halo_size=0, sharding=None, order=1):
    """``jaxpm.pm.lpt``: first- (and second-) order LPT displacement ``dx``,
    momentum ``p`` and force term ``f`` of the particles."""
    _single_device(halo_size, sharding)
    ic = initial_conditions.to(torch.float32).contiguous()
    _lib.require_cuda(ic)
    absolute = particles is not None
    if particles is None:
        particles = torch.zeros((*ic.shape, 3), dtype=torch.float32, device=ic.device)
    a, E, D1, f1 = _lpt_scalars(cosmo, a)
    F1 = pm_forces(particles, delta=ic, paint_absolute_pos=absolute)
    dGfa = float(gr.dGfa(cosmo, a))
    dx = D1 * F1
    p = (a**2 * f1 * E) * dx
    f = (a**2 * E * dGfa) * F1
    if order == 2:
        delta2 = _Source2LPT.apply(ic)
        F2 = pm_forces(particles, delta=delta2, paint_absolute_pos=absolute)
        D2 = 3.0 / 7.0 * float(gr.growth_factor_second(cosmo, a))
        f2 = float(gr.growth_rate_second(cosmo, a))
        dGf2a = float(gr.dGf2a(cosmo, a))
        dx2 = D2 * F2
        dx = dx + dx2
        p = p + (a**2 * f2 * E) * dx2
        f = f + (a**2 * E * dGf2a) * F2
    return dx, p, f


def pk_table(cosmo, kmin=1e-4, kmax=10.0, n=128):
    """The (k, P) table the reference's tests interpolate
    (``tests/conftest.py:90-94``): ``logspace(-4, 1, 128)`` and the linear
    matter power at a = 1."""
    from .cosmology import linear_matter_power
    k = np.logspace(np.log10(kmin), np.log10(kmax), n)
    return k, linear_matter_power(cosmo, k)


def linear_field(mesh_shape, box_size, pk, seed, sharding=None, noise=None, device="cuda"):
    """``jaxpm.pm.linear_field``: a Gaussian field with power spectrum ``pk``.

    ``pk`` is either a ``(k, P)`` table (linearly interpolated on the GPU,
    clamped at the ends, as ``jnp.interp``) or a callable evaluated on the
    host over a fine log-spaced grid spanning the mesh's wave numbers.
    ``noise`` (optional) replaces the seeded white noise."""
    _single_device(0, sharding)
    mesh_shape = tuple(int(s) for s in mesh_shape)
    box = [float(b) for b in box_size]
    if noise is None:
        noise = normal_field(seed, mesh_shape, device=device)
    noise = noise.to(torch.float32).contiguous()
    if callable(pk):
        kmax = float(np.sqrt(sum((np.pi * n / b)**2 for n, b in zip(mesh_shape, box)))) * 1.01
        tk = np.concatenate([[0.0], np.logspace(-5, np.log10(kmax), 4096)])
        tp = np.asarray(pk(tk), dtype=np.float64)
    else:
        tk, tp = (np.asarray(v, dtype=np.float64) for v in pk)
    return _Colour.apply(noise, power_table(tk, tp, noise.device), tuple(box))


def power_table(tk, tp, device):
    """A (k, P) table as the two float32 device arrays of the colouring
    kernel."""
    return (torch.tensor(np.asarray(tk, dtype=np.float64), dtype=torch.float32, device=device),
            torch.tensor(np.asarray(tp, dtype=np.float64), dtype=torch.float32, device=device))


def colour(noise, table, box):
    """White noise -> the Gaussian field of power spectrum ``table``:
    R2C, ``pmgb_linear_field_colour_f32``, C2R (``jaxpm/pm.py:134-143``)."""
    nx, ny, nz = noise.shape
    tk_d, tp_d = table
    spec = torch.empty((nx, ny, nz // 2 + 1), dtype=torch.complex64, device=noise.device)
    s = _lib.stream()
    _lib.call("pmgb_fft_r2c_f32", _lib.ptr(noise), _lib.ptr(spec), nx, ny, nz, 1, s)
    _lib.call("pmgb_linear_field_colour_f32", _lib.ptr(spec), nx, ny, nz, *box, _lib.ptr(tk_d),
              _lib.ptr(tp_d), tk_d.numel(), 1.0 / (nx * ny * nz), s)
    out = torch.empty(noise.shape, dtype=torch.float32, device=noise.device)
    _lib.call("pmgb_fft_c2r_f32", _lib.ptr(spec), _lib.ptr(out), nx, ny, nz, 1, 0, s)
    return out


class _Colour(torch.autograd.Function):
    """noise -> linear field.  The map is a real circular convolution whose
    kernel (the inverse transform of sqrt(P(|k|) N/V), real and even in k)
    is symmetric, so the backward applies the same colouring to the
    cotangent."""

    @staticmethod
    def forward(ctx, noise, table, box):
        ctx.table, ctx.box = table, box
        return colour(noise.to(torch.float32).contiguous(), table, box)

    @staticmethod
    def backward(ctx, g):
        return colour(g.to(torch.float32).contiguous(), ctx.table, ctx.box), None, None


__all__ = ["pm_forces", "lpt", "linear_field", "force_meshes", "pk_table", "power_table",
           "colour", "fft3d", "ifft3d", "MODES"]
