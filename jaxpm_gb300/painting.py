"""CIC painting and reading on the GPU, with jaxpm's call surface.

Mirrors ``jaxpm/painting.py``: ``cic_paint`` (``:48-75``), ``cic_read``
(``:109-128``), ``cic_paint_dx`` (``:192-215``) and ``cic_read_dx``
(``:239-260``).  Arrays are torch CUDA tensors (float32); results are new
tensors, inputs are not modified.  ``halo_size`` and ``sharding`` exist for
signature compatibility: this engine runs on one GPU, so anything but
``0``/``None`` raises ``NotImplementedError``.

Absolute-position painting and reading are differentiable through
``torch.autograd`` with hand-written adjoints (``pmgb_cic_paint_vjp_f32``,
``pmgb_cic_read_vjp_f32``).
"""
import math

import torch

from . import _lib

MODES = {"atomic": _lib.PAINT_ATOMIC, "binned": _lib.PAINT_BINNED,
         "deterministic": _lib.PAINT_DETERMINISTIC}


def _single_device(halo_size, sharding):
    if sharding is not None or (halo_size not in (0, None) and any(
            h != 0 for h in (halo_size if isinstance(halo_size, (tuple, list)) else [halo_size]))):
        raise NotImplementedError(
            "jaxpm_gb300 runs one simulation per GPU: halo_size must be 0 and sharding None")


def _mode(mode):
    if isinstance(mode, int):
        return mode
    try:
        return MODES[mode]
    except KeyError:
        raise ValueError(f"unknown paint mode {mode!r}; expected one of {sorted(MODES)}")


def _reshape_like_jax(x, shape):
    n = math.prod(shape)
    if x.numel() != n:
        raise TypeError(f"cannot reshape array of shape {tuple(x.shape)} (size {x.numel()}) "
                        f"into shape {tuple(shape)} (size {n})")
    return x.reshape(shape)


def _f32(x):
    if x.dtype != torch.float32:
        raise TypeError(f"jaxpm_gb300 computes in float32; got {x.dtype}")
    return x.contiguous()


class _Paint(torch.autograd.Function):
    @staticmethod
    def forward(ctx, grid_mesh, positions, weight, wscale, mode):
        nx, ny, nz = grid_mesh.shape
        pos = positions.reshape(-1, 3)
        np_ = pos.shape[0]
        w = None if weight is None else weight.reshape(-1)
        _lib.require_cuda(grid_mesh, pos, w)
        out = grid_mesh.clone()
        wsb = _lib.load().pmgb_cic_paint_workspace_size(nx, ny, nz, np_, mode)
        ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device=grid_mesh.device)
        _lib.call("pmgb_cic_paint_f32", _lib.ptr(out), nx, ny, nz, _lib.ptr(pos), np_,
                  _lib.ptr(w), float(wscale), mode, 1, _lib.ptr(ws), wsb, _lib.stream())
        ctx.save_for_backward(pos, w)
        ctx.wscale = float(wscale)
        ctx.pshape = positions.shape
        return out

    @staticmethod
    def backward(ctx, g):
        pos, w = ctx.saved_tensors
        g = g.contiguous()
        nx, ny, nz = g.shape
        gpos = gw = None
        need_pos, need_w = ctx.needs_input_grad[1], ctx.needs_input_grad[2]
        if need_pos:
            gpos = torch.empty_like(pos)
        if need_w:
            gw = torch.empty(pos.shape[0], dtype=torch.float32, device=g.device)
        if need_pos or need_w:
            _lib.call("pmgb_cic_paint_vjp_f32", _lib.ptr(g), nx, ny, nz, _lib.ptr(pos),
                      pos.shape[0], _lib.ptr(w), ctx.wscale, _lib.ptr(gpos), _lib.ptr(gw),
                      _lib.stream())
        if gpos is not None:
            gpos = gpos.reshape(ctx.pshape)
        if gw is not None:
            gw = gw * ctx.wscale
            gw = gw.reshape(w.shape) if w is not None else None
        return g, gpos, gw, None, None


class _Read(torch.autograd.Function):
    @staticmethod
    def forward(ctx, grid_mesh, positions):
        nx, ny, nz = grid_mesh.shape
        pos = positions.reshape(-1, 3)
        _lib.require_cuda(grid_mesh, pos)
        out = torch.empty(pos.shape[0], dtype=torch.float32, device=grid_mesh.device)
        _lib.call("pmgb_cic_read_f32", _lib.ptr(grid_mesh), nx, ny, nz, _lib.ptr(pos),
                  pos.shape[0], _lib.ptr(out), _lib.stream())
        ctx.save_for_backward(grid_mesh, pos)
        ctx.pshape = positions.shape
        return out.reshape(positions.shape[:-1])

    @staticmethod
    def backward(ctx, g):
        mesh, pos = ctx.saved_tensors
        g = g.contiguous().reshape(-1)
        nx, ny, nz = mesh.shape
        gmesh = torch.zeros_like(mesh) if ctx.needs_input_grad[0] else None
        gpos = torch.empty_like(pos) if ctx.needs_input_grad[1] else None
        if gmesh is not None or gpos is not None:
            _lib.call("pmgb_cic_read_vjp_f32", _lib.ptr(mesh), nx, ny, nz, _lib.ptr(pos),
                      pos.shape[0], _lib.ptr(g), _lib.ptr(gmesh), _lib.ptr(gpos), _lib.stream())
        return gmesh, (gpos.reshape(ctx.pshape) if gpos is not None else None)


def paint(grid_mesh, positions, weight=1.0, mode="atomic"):
    """``_cic_paint_impl`` (``jaxpm/painting.py:15-45``) for any number of
    particles: returns ``grid_mesh`` plus the CIC deposit of ``positions``
    ([..., 3], cell units), each particle weighted by ``weight`` (scalar or
    one value per particle)."""
    grid_mesh = _f32(grid_mesh)
    positions = _f32(positions)
    if isinstance(weight, torch.Tensor) and weight.numel() > 1:
        w, ws = _f32(weight), 1.0
        if w.numel() * 3 != positions.numel():
            raise ValueError("Weight shape must match particle shape")
    else:
        w, ws = None, float(weight)
    return _Paint.apply(grid_mesh, positions, w, ws, _mode(mode))


def read(grid_mesh, positions):
    """``_cic_read_impl`` (``jaxpm/painting.py:78-106``) for any number of
    particles: CIC interpolation of ``grid_mesh`` at ``positions``."""
    return _Read.apply(_f32(grid_mesh), _f32(positions))


def cic_paint(grid_mesh, positions, weight=1.0, halo_size=0, sharding=None, mode="atomic"):
    """``jaxpm.painting.cic_paint``: positions must hold one particle per
    mesh cell (the reference reshapes them to ``(*grid_mesh.shape, 3)``).
    ``mode`` selects the painter: ``"atomic"`` (default), ``"binned"`` or
    ``"deterministic"`` (bit-identical run to run)."""
    _single_device(halo_size, sharding)
    positions = _reshape_like_jax(positions, (*grid_mesh.shape, 3))
    return paint(grid_mesh, positions, weight, mode)


def cic_read(grid_mesh, positions, halo_size=0, sharding=None):
    """``jaxpm.painting.cic_read``: interpolates ``grid_mesh`` at one particle
    per mesh cell; the output has shape ``positions.shape[:-1]``."""
    _single_device(halo_size, sharding)
    original = positions.shape
    positions = _reshape_like_jax(positions, (*grid_mesh.shape, 3))
    return read(grid_mesh, positions).reshape(original[:-1])


def cic_paint_dx(displacements, halo_size=0, sharding=None, weight=1.0, chunk_size=2**24):
    """``jaxpm.painting.cic_paint_dx``: particle ``i`` sits at lattice point
    ``i`` plus ``displacements[i]``; returns the painted mesh of shape
    ``displacements.shape[:-1]``.  ``chunk_size`` is accepted for
    compatibility (the kernel needs no chunking)."""
    _single_device(halo_size, sharding)
    disp = _f32(displacements)
    _lib.require_cuda(disp)
    shape = disp.shape[:-1]
    if len(shape) != 3:
        raise ValueError("displacements must have shape [nx, ny, nz, 3]")
    w, ws = None, 1.0
    if isinstance(weight, torch.Tensor) and weight.numel() > 1:
        if tuple(weight.shape) != tuple(shape):
            raise ValueError("Weight shape must match particle shape")
        w = _f32(weight)
    else:
        ws = float(weight)
    out = torch.empty(shape, dtype=torch.float32, device=disp.device)
    _lib.call("pmgb_cic_paint_dx_f32", _lib.ptr(out), *shape, _lib.ptr(disp), _lib.ptr(w), ws, 0,
              _lib.stream())
    return out


def cic_read_dx(grid_mesh, disp, halo_size=0, sharding=None):
    """``jaxpm.painting.cic_read_dx``: reads ``grid_mesh`` at lattice point
    ``i`` plus ``disp[i]``; output shape ``grid_mesh.shape``."""
    _single_device(halo_size, sharding)
    grid_mesh, disp = _f32(grid_mesh), _f32(disp)
    _lib.require_cuda(grid_mesh, disp)
    if disp.numel() != 3 * grid_mesh.numel():
        raise ValueError("disp must hold one displacement per mesh cell")
    out = torch.empty_like(grid_mesh)
    _lib.call("pmgb_cic_read_dx_f32", _lib.ptr(grid_mesh), *grid_mesh.shape, _lib.ptr(disp),
              _lib.ptr(out), _lib.stream())
    return out


def cic_weights(positions, mesh_shape):
    """Neighbour cells ``[Np, 8, 3]`` (int32, wrapped) and CIC weights
    ``[Np, 8]`` of every particle, in the reference's neighbour order
    (``jaxpm/painting.py:21-37``)."""
    pos = _f32(positions).reshape(-1, 3)
    _lib.require_cuda(pos)
    n = pos.shape[0]
    idx = torch.empty((n, 8, 3), dtype=torch.int32, device=pos.device)
    w = torch.empty((n, 8), dtype=torch.float32, device=pos.device)
    _lib.call("pmgb_cic_weights_f32", _lib.ptr(pos), n, *mesh_shape, _lib.ptr(idx), _lib.ptr(w),
              _lib.stream())
    return idx, w


def enmesh(disp):
    """Neighbour cells ``[N, 8, 3]`` (-1 where the reference drops the
    neighbour) and weights ``[N, 8]`` of the relative mode
    (``jaxpm/painting_utils.py:28-96``)."""
    disp = _f32(disp)
    _lib.require_cuda(disp)
    shape = disp.shape[:-1]
    n = math.prod(shape)
    idx = torch.empty((n, 8, 3), dtype=torch.int32, device=disp.device)
    w = torch.empty((n, 8), dtype=torch.float32, device=disp.device)
    _lib.call("pmgb_enmesh_f32", _lib.ptr(disp), *shape, _lib.ptr(idx), _lib.ptr(w),
              _lib.stream())
    return idx, w
