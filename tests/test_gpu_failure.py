"""Failure detection on the GPU without a fault: a bounded mbarrier wait
that runs out reports it through a status word, the context stays usable,
and the engine turns the tile kernels' failed-wait counter into an
exception (``pmgb_check_stats``) instead of returning invalid positions.

The reference raises Python exceptions on bad input
(``jaxpm/pm.py:22-25``, ``jaxpm/painting.py:171-173``); a device-side
failure here becomes the same kind of exception on the host."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_reports(cuda, lib):
    from jaxpm_gb300 import _lib
    status = torch.full((1,), 7, dtype=torch.int32, device=cuda)
    # an mbarrier armed for 16 bytes that no copy delivers: the wait must end
    # after its poll limit with status 1
    _lib.call("pmgb_test_wait_timeout", 2000, _lib.ptr(status), _lib.stream())
    torch.cuda.synchronize()
    assert status.item() == 1
    # the context is still usable afterwards
    mesh = torch.zeros((8, 8, 8), device=cuda)
    pos = torch.tensor([[1.5, 2.5, 3.5]], device=cuda)
    _lib.call("pmgb_cic_paint_f32", _lib.ptr(mesh), 8, 8, 8, _lib.ptr(pos), 1, None, 1.0,
              _lib.PAINT_ATOMIC, 0, None, 0, _lib.stream())
    torch.cuda.synchronize()
    assert mesh.sum().item() == pytest.approx(1.0)


def test_check_stats_raises_on_a_failed_wait(cuda, lib):
    from jaxpm_gb300 import _lib
    stats = torch.tensor([0, 0, 1], dtype=torch.int32, device=cuda)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_check_stats", _lib.ptr(stats), _lib.stream())
    assert e.value.status == 3 and "spin limit" in str(e.value)
    stats.zero_()
    assert _lib.call("pmgb_check_stats", _lib.ptr(stats), _lib.stream()) == 0


def test_engine_raises_instead_of_returning_abandoned_work(cuda, lib):
    """The counter a timed-out tile kernel sets (stats[2]) is set on the host
    here; run() and vjp() must raise rather than return."""
    from jaxpm_gb300 import _lib, cosmology, simulate
    n = 16
    rng = np.random.default_rng(0)
    lat = np.stack(np.meshgrid(*[np.arange(n)] * 3, indexing="ij"), -1).reshape(-1, 3)
    x = torch.from_numpy((lat + rng.normal(0, 0.5, lat.shape)).astype(np.float32)).to(cuda)
    v = torch.zeros_like(x)
    eng = simulate.SortedFastPM((n,) * 3, cosmology.Planck15(), 0.1, 1.0, 2, device=cuda)
    eng.load(x, v)
    eng.run()  # clean run: no exception
    eng.load(x, v)
    eng.stats_buf[2] = 1
    with pytest.raises(_lib.PmgbError):
        eng.run()
    eng.load(x, v)
    eng.run(check=False)
    eng.stats_buf[2] = 1
    with pytest.raises(_lib.PmgbError):
        eng.check()
