"""The autotuner of the sorted run loop: it times every candidate launch
configuration on the caller's workload, keeps the fastest, caches it per
(mesh, particles, steps, GPU, ABI) and applies it; the tuned run gives the
same state as the default one (the schedule changes only the order of the
floating-point sums)."""
import json

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import cic

pytestmark = pytest.mark.gpu


def test_autotune_chooses_caches_and_keeps_results(cuda, lib, tmp_path, monkeypatch):
    from jaxpm_gb300 import _lib, autotune, cosmology, simulate
    monkeypatch.setenv("PMGB_TUNE_CACHE", str(tmp_path / "tuning.json"))
    shape = (64, 64, 64)
    rng = np.random.default_rng(1)
    lat = cic.lattice(shape).reshape(-1, 3)
    x0 = torch.from_numpy((lat + rng.normal(0, 1.0, lat.shape)).astype(np.float32)).to(cuda)
    v0 = torch.from_numpy(rng.normal(0, 0.4, lat.shape).astype(np.float32)).to(cuda)
    eng = simulate.SortedFastPM(shape, cosmology.Planck15(), 0.1, 1.0, 4, device=cuda)
    default = _lib.get_tuning()
    try:
        eng.load(x0, v0)
        eng.run()
        ref = eng.state()
        choice, report = autotune.tune_run(eng, x0, v0)
        assert choice in list(autotune.candidates())
        assert len(report) == len(list(autotune.candidates()))
        assert all(np.isfinite(v) and v > 0 for v in report.values())
        assert _lib.get_tuning() == choice
        cached = json.load(open(tmp_path / "tuning.json"))
        assert list(cached.values()) == [choice]
        again, rep2 = autotune.tune_run(eng, x0, v0)  # from the cache
        assert again == choice and rep2 == {}
        eng.load(x0, v0)
        eng.run()
        got = eng.state()
        assert rel_l2(got[0].cpu() - x0.cpu(), ref[0].cpu() - x0.cpu()) < 1e-5
        assert rel_l2(got[1].cpu(), ref[1].cpu()) < 1e-5
        # every candidate gives the same state
        for cand in autotune.candidates():
            _lib.set_tuning(**cand)
            eng.load(x0, v0)
            eng.run()
            assert rel_l2(eng.state()[1].cpu(), ref[1].cpu()) < 1e-5, cand
    finally:
        _lib.set_tuning(**default)
