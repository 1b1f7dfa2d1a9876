"""Snapshots: device arrays written to NumPy ``.npy`` files without holding
up the GPU (the reference gathers fields to the host and ``np.save``s them,
``notebooks/05-MultiHost_PM.py:151-177``).

``save_npy(path, tensor)`` takes the tensor's state in stream order (a
device copy into a staging buffer, unless ``staging=False``) and returns a
``Snapshot`` whose ``wait()`` joins the library's writer thread; the file is
an ordinary ``.npy`` that ``np.load`` reads.  ``stack_state`` gives the
``[2, Np, 3]`` stacked state of ``make_diffrax_ode`` users
(``jaxpm/ode.py:150-176``).
"""
import ctypes

import torch

from . import _lib

_DESCR = {torch.float32: ("<f4", 4), torch.float64: ("<f8", 8), torch.complex64: ("<c8", 8),
          torch.int32: ("<i4", 4), torch.int64: ("<i8", 8), torch.uint8: ("|u1", 1)}


class Snapshot:
    """A snapshot being written; ``wait()`` returns once the file is complete."""

    def __init__(self, handle, keep):
        self._handle = handle
        self._keep = keep  # staging buffer / source tensor, alive until written

    def wait(self):
        if self._handle is not None:
            h, self._handle = self._handle, None
            try:
                _lib.call("pmgb_snapshot_wait", h)
            finally:
                self._keep = None

    def __del__(self):
        try:
            self.wait()
        except Exception:
            pass


def save_npy(path, tensor, staging=True, stream=None):
    """Starts writing a CUDA tensor to ``path`` (``.npy``, C order) and
    returns a ``Snapshot``.  With ``staging`` the tensor may be modified
    right away (its state is copied on the device first); without, it must
    stay unchanged until ``wait()``."""
    if not tensor.is_cuda:
        raise ValueError("save_npy writes CUDA tensors")
    t = tensor.contiguous()
    if t.dtype not in _DESCR:
        raise TypeError(f"unsupported dtype {t.dtype}")
    descr, itemsize = _DESCR[t.dtype]
    shape = (ctypes.c_int64 * max(t.dim(), 1))(*t.shape)
    stage = torch.empty_like(t) if staging else None
    handle = ctypes.c_void_p()
    s = _lib.stream(t.device) if stream is None else stream
    _lib.call("pmgb_snapshot_begin_npy", str(path).encode(), _lib.ptr(t), descr.encode(),
              itemsize, ctypes.cast(shape, ctypes.c_void_p), t.dim(), _lib.ptr(stage),
              stage.numel() * itemsize if stage is not None else 0, s, ctypes.byref(handle))
    return Snapshot(handle, (stage, t))


def save_state(prefix, pos, vel, staging=True):
    """Writes ``prefix_pos.npy`` and ``prefix_vel.npy``; returns the two
    snapshots."""
    return (save_npy(f"{prefix}_pos.npy", pos, staging),
            save_npy(f"{prefix}_vel.npy", vel, staging))


def stack_state(pos, vel):
    """The ``[2, Np, 3]`` stacked state of ``make_diffrax_ode``."""
    return torch.stack([pos, vel])
