"""The allocation-free deterministic paint, called through the C ABI.

pmgb_cic_paint_deterministic_noalloc_f32 serves callers that cannot hand
out device memory (a framework's custom-call handler that only gets the
buffers its allocator made, or code running while another runtime's pool
owns the device memory): its fixed-point scratch is a static device array in
libpmgb instead of a caller workspace.  Its results must match the existing
deterministic entry point, pmgb_cic_paint_f32 with PMGB_PAINT_DETERMINISTIC,
on consecutive calls (the shared scratch is cleared by every call).  This
file is collected last so that a run stopping at the first failure has run
every other test already."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the paint parity bar of the other tests (relative L2)


def clustered(n, seed):
    rng = np.random.default_rng(seed)
    lattice = np.stack(np.meshgrid(*[np.arange(n)] * 3, indexing="ij"), -1).reshape(-1, 3)
    pos = lattice + rng.normal(0, 1.5, lattice.shape)
    clumps = rng.uniform(0, n, (4, 3))
    pos[: n**3 // 4] = clumps[rng.integers(0, 4, n**3 // 4)] + rng.normal(0, 0.5, (n**3 // 4, 3))
    return pos.astype(np.float32)


def test_noalloc_paint_matches_workspace_paint_on_consecutive_calls(cuda, lib):
    from jaxpm_gb300 import _lib
    n = 64
    s = _lib.stream()
    for seed in (0, 1):  # two calls in a row on different particles
        pos = torch.from_numpy(clustered(n, seed)).to(cuda)
        w = torch.rand(n**3, device=cuda, generator=torch.Generator(device=cuda).manual_seed(seed))
        ref = torch.empty((n,) * 3, device=cuda)
        wsb = lib.pmgb_cic_paint_workspace_size(n, n, n, n**3, _lib.PAINT_DETERMINISTIC)
        ws = torch.empty(wsb, dtype=torch.uint8, device=cuda)
        _lib.call("pmgb_cic_paint_f32", _lib.ptr(ref), n, n, n, _lib.ptr(pos), n**3, _lib.ptr(w),
                  0.5, _lib.PAINT_DETERMINISTIC, 0, _lib.ptr(ws), wsb, s)
        out = torch.full((n,) * 3, 7.0, device=cuda)  # overwritten (accumulate = 0)
        _lib.call("pmgb_cic_paint_deterministic_noalloc_f32", _lib.ptr(out), n, n, n,
                  _lib.ptr(pos), n**3, _lib.ptr(w), 0.5, 0, s)
        torch.cuda.synchronize()
        assert rel_l2(out.cpu(), ref.cpu()) < TOL
        assert torch.equal(out, ref)  # same fixed-point sums: identical bits


def test_noalloc_paint_accumulates_and_rejects_large_meshes(cuda, lib):
    from jaxpm_gb300 import _lib
    s = _lib.stream()
    base = torch.full((8, 8, 8), 2.0, device=cuda)
    pos = torch.tensor([[1.0, 2.0, 3.0], [4.5, 4.5, 4.5]], device=cuda)
    _lib.call("pmgb_cic_paint_deterministic_noalloc_f32", _lib.ptr(base), 8, 8, 8, _lib.ptr(pos),
              2, None, 1.0, 1, s)
    torch.cuda.synchronize()
    assert base[1, 2, 3].item() == 3.0 and base.sum().item() == pytest.approx(2.0 * 512 + 2)
    big = ctypes.c_void_p(base.data_ptr())  # never touched: rejected before any GPU work
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_cic_paint_deterministic_noalloc_f32", big, 256, 128, 128, None, 0, None,
                  1.0, 0, s)
    assert e.value.status == 1 and "at most" in str(e.value)
