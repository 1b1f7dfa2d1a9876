"""Cloud-in-cell mass assignment, restated in NumPy (test infrastructure only).

Absolute mode follows ``jaxpm/painting.py:15-45`` (paint) and
``jaxpm/painting.py:78-106`` (read); relative mode follows
``jaxpm/painting_utils.py:28-96`` (``enmesh``), ``:99-131`` (scatter) and
``:168-187`` (gather), driven by ``jaxpm/painting.py:161-236``.

Every floating-point step is written in the reference's order and in the
requested dtype, so that float32 indices and per-neighbour weights can be
compared bit for bit with the CUDA kernels.

``cic_paint`` and ``cic_read`` hand absolute-mode work to the C statement of
the same arithmetic (``oracle/ccic.c`` via ``oracle/native.py``) when it is
built and ``NATIVE`` is true; ``tests/test_oracle.py`` holds the two
statements equal.
"""
import numpy as np

from . import native

# use the C statement of paint/read when it can be built (same arithmetic)
NATIVE = True


def _c(dtype):
    """The C oracle and its function suffix for ``dtype``, or None."""
    if not NATIVE or dtype not in (np.float32, np.float64):
        return None
    h = native.lib()
    if h is None:
        return None
    return h, ("f32" if dtype == np.float32 else "f64")

# Neighbour order of absolute mode, ``jaxpm/painting.py:24-25``.
CONNECTION_ABS = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1],
                           [1, 1, 0], [1, 0, 1], [0, 1, 1], [1, 1, 1]])

# Neighbour order of relative mode: bit d of the neighbour number is the
# offset along axis d, ``jaxpm/painting_utils.py:43-45``.
CONNECTION_REL = (np.arange(8)[:, None] >> np.arange(3)) & 1


def cic_weights(positions, mesh_shape, dtype=np.float32):
    """Per-particle neighbour cells and CIC weights, absolute mode.

    ``jaxpm/painting.py:21-37``: floor, add the connection offsets in float,
    ``1 - |x - c|`` per axis, product ``(k0*k1)*k2``, then ``int32`` cast and
    floor-modulo by the mesh shape.  Returns ``(idx [Np,8,3] int32,
    w [Np,8] dtype)``.
    """
    pos = np.asarray(positions, dtype=dtype).reshape(-1, 1, 3)
    floor = np.floor(pos)
    nc = floor + CONNECTION_ABS.astype(dtype)[None]
    k = dtype(1) - np.abs(pos - nc)
    w = (k[..., 0] * k[..., 1]) * k[..., 2]
    idx = np.mod(nc.astype(np.int32), np.asarray(mesh_shape, dtype=np.int32))
    return idx.astype(np.int32), w.astype(dtype)


def _flat(idx, mesh_shape):
    nx, ny, nz = mesh_shape
    return (idx[..., 0].astype(np.int64) * ny + idx[..., 1]) * nz + idx[..., 2]


def cic_paint(grid_mesh, positions, weight=1.0, dtype=np.float32):
    """``_cic_paint_impl`` (``jaxpm/painting.py:15-45``) for any particle count.

    The scalar-or-array weight multiplies the kernel after the product
    (``:30-33``).  Accumulation uses ``np.bincount`` (float64 sums, cast back
    to ``dtype``); the reference's ``lax.scatter_add`` order is unspecified on
    GPU, so only the summation order differs.
    """
    grid_mesh = np.asarray(grid_mesh, dtype=dtype)
    shape = grid_mesh.shape
    c = _c(dtype)
    if c is not None:
        h, sfx = c
        pos = np.ascontiguousarray(np.asarray(positions, dtype=dtype).reshape(-1, 3))
        acc = np.zeros(int(np.prod(shape)), np.float64)
        scalar = np.isscalar(weight) or np.ndim(weight) == 0
        wts = None if scalar else np.ascontiguousarray(
            np.broadcast_to(np.asarray(weight, dtype=dtype).reshape(-1), (len(pos),)))
        getattr(h, f"oc_paint_{sfx}")(acc.ctypes.data, *shape, pos.ctypes.data, len(pos),
                                      None if wts is None else wts.ctypes.data,
                                      float(weight) if scalar else 0.0)
        return (grid_mesh.astype(np.float64) + acc.reshape(shape)).astype(dtype)
    idx, w = cic_weights(positions, shape, dtype)
    if np.isscalar(weight) or np.ndim(weight) == 0:
        w = np.asarray(weight, dtype=dtype) * w
    else:
        w = np.asarray(weight, dtype=dtype).reshape(-1, 1) * w
    flat = _flat(idx, shape).reshape(-1)
    acc = np.bincount(flat, weights=w.reshape(-1).astype(np.float64),
                      minlength=int(np.prod(shape)))
    return (grid_mesh.astype(np.float64) + acc.reshape(shape)).astype(dtype)


def cic_read(grid_mesh, positions, dtype=np.float32):
    """``_cic_read_impl`` (``jaxpm/painting.py:78-106``): sum of the 8
    weighted neighbour values, output shaped ``positions.shape[:-1]``."""
    grid_mesh = np.asarray(grid_mesh, dtype=dtype)
    positions = np.asarray(positions, dtype=dtype)
    c = _c(dtype)
    if c is not None:
        h, sfx = c
        pos = np.ascontiguousarray(positions.reshape(-1, 3))
        mesh = np.ascontiguousarray(grid_mesh)
        out = np.empty(len(pos), dtype)
        getattr(h, f"oc_read_{sfx}")(mesh.ctypes.data, *mesh.shape, pos.ctypes.data, len(pos),
                                     out.ctypes.data)
        return out.reshape(positions.shape[:-1])
    idx, w = cic_weights(positions, grid_mesh.shape, dtype)
    vals = grid_mesh[idx[..., 0], idx[..., 1], idx[..., 2]]
    out = vals[:, 0] * w[:, 0]
    for j in range(1, 8):
        out = out + vals[:, j] * w[:, j]
    return out.reshape(positions.shape[:-1]).astype(dtype)


def _dkernel(pos, dtype):
    """Per-axis CIC factors and their derivatives for the absolute mode.

    d(1 - |u|)/du uses JAX's rule for ``abs`` (``select(u >= 0, 1, -1)``),
    and ``floor`` has a zero derivative.
    """
    floor = np.floor(pos)
    nc = floor + CONNECTION_ABS.astype(dtype)[None]
    u = pos - nc
    k = dtype(1) - np.abs(u)
    dk = np.where(u >= 0, dtype(-1), dtype(1)).astype(dtype)
    return k, dk


def cic_grad(grid_mesh, positions, dtype=np.float64):
    """``sum_j mesh[idx_j] * grad W_j(x)`` per particle ``[Np, 3]``: the
    position gradient of the interpolated field, with the derivative of each
    axis factor times the other two (``_dkernel``).  The C statement when it
    is built, else NumPy."""
    grid_mesh = np.ascontiguousarray(np.asarray(grid_mesh, dtype=dtype))
    pos = np.ascontiguousarray(np.asarray(positions, dtype=dtype).reshape(-1, 3))
    c = _c(dtype)
    if c is not None:
        h, sfx = c
        out = np.empty((len(pos), 3), dtype)
        getattr(h, f"oc_grad_{sfx}")(grid_mesh.ctypes.data, *grid_mesh.shape, pos.ctypes.data,
                                     len(pos), out.ctypes.data)
        return out
    idx, _ = cic_weights(pos, grid_mesh.shape, dtype)
    k, dk = _dkernel(pos.reshape(-1, 1, 3), dtype)
    m = grid_mesh[idx[..., 0], idx[..., 1], idx[..., 2]]
    gx = (m * dk[..., 0] * k[..., 1] * k[..., 2]).sum(-1)
    gy = (m * k[..., 0] * dk[..., 1] * k[..., 2]).sum(-1)
    gz = (m * k[..., 0] * k[..., 1] * dk[..., 2]).sum(-1)
    return np.stack([gx, gy, gz], -1)


def cic_paint_vjp(positions, mesh_shape, g_mesh, weight=1.0, dtype=np.float64):
    """Vector-Jacobian product of ``cic_paint`` w.r.t. positions and weight.

    Returns ``(g_pos [Np,3], g_weight [Np])``: the cotangent mesh read with
    the CIC weights gives the weight term; the position term uses the
    derivative of each axis factor times the other two.
    """
    pos = np.asarray(positions, dtype=dtype).reshape(-1, 1, 3)
    g_mesh = np.asarray(g_mesh, dtype=dtype)
    if _c(dtype) is not None:
        wt = (np.asarray(weight, dtype=dtype).reshape(-1, 1)
              if np.ndim(weight) else np.asarray(weight, dtype=dtype))
        gpos = cic_grad(g_mesh, pos, dtype) * wt
        return gpos, cic_read(g_mesh, pos.reshape(-1, 3), dtype)
    idx, _ = cic_weights(pos.reshape(-1, 3), mesh_shape, dtype)
    k, dk = _dkernel(pos, dtype)
    g = g_mesh[idx[..., 0], idx[..., 1], idx[..., 2]]
    wt = (np.asarray(weight, dtype=dtype).reshape(-1, 1)
          if np.ndim(weight) else np.asarray(weight, dtype=dtype))
    gx = (g * dk[..., 0] * k[..., 1] * k[..., 2]).sum(-1)
    gy = (g * k[..., 0] * dk[..., 1] * k[..., 2]).sum(-1)
    gz = (g * k[..., 0] * k[..., 1] * dk[..., 2]).sum(-1)
    gpos = np.stack([gx, gy, gz], -1) * wt
    gw = (g * k[..., 0] * k[..., 1] * k[..., 2]).sum(-1)
    return gpos, gw


def cic_read_vjp(grid_mesh, positions, g_out, dtype=np.float64):
    """Vector-Jacobian product of ``cic_read`` w.r.t. mesh and positions.

    ``g_mesh`` is the paint of the output cotangents; ``g_pos`` is the
    cotangent times the gradient of the interpolated field.
    """
    grid_mesh = np.asarray(grid_mesh, dtype=dtype)
    pos = np.asarray(positions, dtype=dtype).reshape(-1, 1, 3)
    g_out = np.asarray(g_out, dtype=dtype).reshape(-1)
    g_mesh = cic_paint(np.zeros(grid_mesh.shape, dtype), pos.reshape(-1, 3),
                       weight=g_out, dtype=dtype)
    if _c(dtype) is not None:
        return g_mesh, cic_grad(grid_mesh, pos, dtype) * g_out[:, None]
    idx, _ = cic_weights(pos.reshape(-1, 3), grid_mesh.shape, dtype)
    k, dk = _dkernel(pos, dtype)
    m = grid_mesh[idx[..., 0], idx[..., 1], idx[..., 2]]
    gx = (m * dk[..., 0] * k[..., 1] * k[..., 2]).sum(-1)
    gy = (m * k[..., 0] * dk[..., 1] * k[..., 2]).sum(-1)
    gz = (m * k[..., 0] * k[..., 1] * dk[..., 2]).sum(-1)
    gpos = np.stack([gx, gy, gz], -1) * g_out[:, None]
    return g_mesh, gpos


# --------------------------------------------------------------------------
# Relative mode
# --------------------------------------------------------------------------


def _jnp_remainder(x, y):
    """``jnp.remainder`` on floats: C ``fmod`` then shifted into the sign
    of the divisor (what ``%=`` does at ``jaxpm/painting_utils.py:58``)."""
    r = np.fmod(x, y)
    fix = (r != 0) & ((r < 0) != (y < 0))
    return np.where(fix, r + y, r)


def enmesh(pmid, disp, mesh_shape, dtype=np.float32):
    """Multilinear neighbours of ``pmid + disp`` with periodic wrap.

    ``jaxpm/painting_utils.py:47-69,84-96`` with ``cell_size = new_cell_size
    = 1``, ``offset = 0`` and ``base_shape = mesh_shape``: the wrap is taken
    in float before the floor, the displacement is re-centred with
    ``rint(d / L) * L``, and the weight is ``prod(1 - |d|)`` in neighbour
    order ``CONNECTION_REL``.  Returns ``(idx [Np,8,3] int32, w [Np,8])``.
    """
    pmid = np.asarray(pmid).reshape(-1, 3)
    disp = np.asarray(disp, dtype=dtype).reshape(-1, 3)
    L = np.asarray(mesh_shape, dtype=dtype)
    p = (pmid.astype(dtype) * dtype(1) + disp)[:, None, :]
    ni = p + CONNECTION_REL.astype(dtype)[None]
    ni = _jnp_remainder(ni, L)
    ni = np.floor(ni)  # floor_divide by a cell size of 1 for ni >= 0
    d = p - ni * dtype(1)
    d = d - np.rint(d / L) * L
    w = dtype(1) - np.abs(d)
    w = (w[..., 0] * w[..., 1]) * w[..., 2]
    return ni.astype(np.int32), w.astype(dtype)


def in_range(idx, mesh_shape):
    """Neighbours whose wrapped index lies inside the mesh."""
    return np.all((idx >= 0) & (idx < np.asarray(mesh_shape)), axis=-1)


def lattice(mesh_shape):
    """``uniform_particles`` on one device (``jaxpm/distributed.py:187-190``):
    integer lattice positions, ij indexing, shape ``[*mesh_shape, 3]``."""
    return np.stack(np.meshgrid(*[np.arange(s) for s in mesh_shape],
                                indexing='ij'), axis=-1)


def cic_paint_dx(disp, weight=1.0, dtype=np.float32):
    """``cic_paint_dx`` on one device (``jaxpm/painting.py:161-189``):
    particle ``i`` sits at lattice point ``i`` plus its displacement."""
    disp = np.asarray(disp, dtype=dtype)
    shape = disp.shape[:-1]
    idx, w = enmesh(lattice(shape), disp, shape, dtype)
    if np.ndim(weight):
        w = np.asarray(weight, dtype=dtype).reshape(-1, 1) * w
    else:
        w = w * dtype(weight)
    # out-of-range neighbours are dropped by the reference's scatter
    ok = in_range(idx, shape)
    flat = _flat(np.where(ok[..., None], idx, 0), shape)[ok]
    acc = np.bincount(flat, weights=w[ok].astype(np.float64),
                      minlength=int(np.prod(shape)))
    return acc.reshape(shape).astype(dtype)


def cic_read_dx(grid_mesh, disp, dtype=np.float32):
    """``cic_read_dx`` on one device (``jaxpm/painting.py:218-236``)."""
    grid_mesh = np.asarray(grid_mesh, dtype=dtype)
    shape = grid_mesh.shape
    idx, w = enmesh(lattice(shape), disp, shape, dtype)
    # the reference gathers with mode='drop', fill_value=0
    ok = in_range(idx, shape)
    safe = np.where(ok[..., None], idx, 0)
    vals = np.where(ok, grid_mesh[safe[..., 0], safe[..., 1], safe[..., 2]], dtype(0))
    out = vals[:, 0] * w[:, 0]
    for j in range(1, 8):
        out = out + vals[:, j] * w[:, j]
    return out.reshape(shape).astype(dtype)
