"""Snapshots of device arrays to .npy files (the library's writer thread),
read back with numpy: bit-exact contents, the state at the call (staging),
multi-chunk arrays, spectra, and errors surfacing at wait()."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_snapshot_takes_the_state_at_the_call(cuda, tmp_path):
    from jaxpm_gb300 import snapshot
    x = torch.randn((100003, 3), device=cuda)
    ref = x.cpu().numpy().copy()
    snap = snapshot.save_npy(tmp_path / "x.npy", x)
    x.add_(1.0)  # after the call: not in the file
    snap.wait()
    got = np.load(tmp_path / "x.npy")
    assert got.dtype == np.float32 and got.shape == (100003, 3)
    assert np.array_equal(got, ref)


def test_snapshot_without_staging_and_multichunk(cuda, tmp_path):
    from jaxpm_gb300 import snapshot
    n = 40_000_003  # 160 MB: several 32 MB pinned chunks, the last one partial
    x = torch.arange(n, dtype=torch.float32, device=cuda) * 0.5
    snap = snapshot.save_npy(tmp_path / "big.npy", x, staging=False)
    snap.wait()
    got = np.load(tmp_path / "big.npy", mmap_mode="r")
    assert got.shape == (n,)
    assert got[0] == 0.0 and got[-1] == np.float32((n - 1) * 0.5)
    assert np.array_equal(got[::99991], x[::99991].cpu().numpy())


def test_snapshot_of_a_spectrum_and_the_stacked_state(cuda, tmp_path):
    from jaxpm_gb300 import distributed, snapshot
    m = torch.randn((16, 16, 16), device=cuda)
    spec = distributed.fft3d(m)
    snapshot.save_npy(tmp_path / "s.npy", spec).wait()
    assert np.array_equal(np.load(tmp_path / "s.npy"), spec.cpu().numpy())
    pos, vel = torch.randn((10, 3), device=cuda), torch.randn((10, 3), device=cuda)
    st = snapshot.stack_state(pos, vel)
    assert st.shape == (2, 10, 3) and torch.equal(st[1], vel)
    a, b = snapshot.save_state(str(tmp_path / "state"), pos, vel)
    a.wait()
    b.wait()
    assert np.array_equal(np.load(tmp_path / "state_vel.npy"), vel.cpu().numpy())


def test_snapshot_error_surfaces_at_wait(cuda, tmp_path):
    from jaxpm_gb300 import _lib, snapshot
    x = torch.zeros(10, device=cuda)
    snap = snapshot.save_npy(tmp_path / "missing_dir" / "x.npy", x)
    with pytest.raises(_lib.PmgbError) as e:
        snap.wait()
    assert "cannot open" in str(e.value)
