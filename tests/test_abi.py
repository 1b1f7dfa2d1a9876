"""The C ABI library: it builds, loads, exports every declared symbol and
rejects bad arguments on the host (no GPU work is issued here)."""
import ctypes
import os
import re

import numpy as np

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "pmgb.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pmgb_\w+)\s*\(", text)))


def test_header_declares_the_hot_path():
    names = declared_symbols()
    for must in ["pmgb_cic_paint_f32", "pmgb_cic_read_f32", "pmgb_cic_read3_f32",
                 "pmgb_kspace_forces_f32", "pmgb_fft_r2c_f32", "pmgb_fft_c2r_f32",
                 "pmgb_pm_forces_f32", "pmgb_fpm_step_f32", "pmgb_pm_forces_vjp_f32",
                 "pmgb_cic_paint_dx_f32", "pmgb_cic_read_dx_f32"]:
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    from jaxpm_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == declared_symbols()


def test_version_and_empty_error(lib):
    assert lib.pmgb_version() >= 100
    assert lib.pmgb_last_error() == b""


def test_bad_shape_is_rejected_before_any_gpu_work(lib):
    from jaxpm_gb300 import _lib
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_cic_paint_f32", None, 0, 4, 4, None, 0, None, 1.0, 0, 0, None, 0, None)
    assert e.value.status == 1 and "mesh shape" in str(e.value)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_cic_paint_f32", ctypes.c_void_p(16), 4, 4, 4, None, 10, None, 1.0, 0, 0,
                  None, 0, None)
    assert "pos is NULL" in str(e.value)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_cic_paint_f32", ctypes.c_void_p(16), 4, 4, 4, None, 0, None, 1.0, 7, 0,
                  None, 0, None)
    assert "paint mode" in str(e.value)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_kspace_forces_f32", ctypes.c_void_p(16), ctypes.c_void_p(16), 10, 4, 4, 4,
                  0.0, 2, 0, 1.0, None)
    assert "grad_order" in str(e.value)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_power_spectrum_f32", ctypes.c_void_p(16), 4, 4, 4, 1.0, 1.0, 1.0,
                  ctypes.c_void_p(16), 5000, ctypes.c_void_p(16), ctypes.c_void_p(16),
                  ctypes.c_void_p(16), None)
    assert "n_edges" in str(e.value)


def test_workspace_queries(lib):
    assert lib.pmgb_pm_workspace_size(64, 64, 64, 64**3, 0) >= 64**3 * 4 * 7
    assert lib.pmgb_pm_workspace_size(64, 64, 64, 64**3, 2) > lib.pmgb_pm_workspace_size(
        64, 64, 64, 64**3, 0)
    assert lib.pmgb_cic_paint_workspace_size(8, 8, 8, 10, 2) == 8 * 512
    assert lib.pmgb_cic_paint_workspace_size(8, 8, 8, 10, 0) == 0
    assert lib.pmgb_pm_workspace_size(0, 8, 8, 1, 0) == 0


def test_batched_table_queries(lib):
    """The batched calls' host side: struct layout, workspace sizing (shape
    groups share pools) and table validation, without a GPU."""
    from jaxpm_gb300 import _lib
    assert ctypes.sizeof(_lib.Sim) == 24
    shapes = [(64,) * 3, (96,) * 3, (64,) * 3, (128,) * 3]
    t = _lib.sim_table(shapes, [int(np.prod(s)) for s in shapes])
    nbytes = lib.pmgb_batch_workspace_size(t, len(shapes))
    cells = sum(int(np.prod(s)) for s in shapes)
    # density + 3 force meshes + 3 cotangent meshes (f32) and one half spectrum (c64)
    assert nbytes >= cells * 4 * 7 + cells * 8 // 2
    assert nbytes < cells * 4 * 7 + cells * 8 * 2
    np_total, cells_total = ctypes.c_int64(), ctypes.c_int64()
    _lib.call("pmgb_batch_counts", t, len(shapes), ctypes.byref(np_total),
              ctypes.byref(cells_total))
    assert np_total.value == cells and cells_total.value == cells
    assert lib.pmgb_batch_workspace_size(t, 0) == 0
    bad = _lib.sim_table([(16, 16, 16)], [-1])
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_batch_counts", bad, 1, None, None)
    assert "np is negative" in str(e.value)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_batch_init", t, len(shapes), None, 0, None)
    assert "NULL" in str(e.value)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_fpm_step_batched_f32", t, len(shapes), None, None, None, None, 0.0,
                  None, None, 0, None)
    assert "pos is NULL" in str(e.value)


@pytest.mark.parametrize("shape", [(), (7,), (3, 4), (2, 1000000, 3), (16, 16, 9)])
@pytest.mark.parametrize("descr", ["<f4", "<c8", "<u4"])
def test_npy_header_is_read_by_numpy(lib, shape, descr):
    """The snapshot writer's .npy header (host-only): numpy parses it and
    finds the dtype and shape, and it is a multiple of 64 bytes."""
    import io
    from jaxpm_gb300 import _lib
    arr = (ctypes.c_int64 * max(len(shape), 1))(*shape)
    n = lib.pmgb_npy_header(descr.encode(), ctypes.cast(arr, ctypes.c_void_p), len(shape),
                            None, 0)
    assert n % 64 == 0 and n > 0
    buf = ctypes.create_string_buffer(n)
    assert lib.pmgb_npy_header(descr.encode(), ctypes.cast(arr, ctypes.c_void_p), len(shape),
                               buf, n) == n
    f = io.BytesIO(buf.raw)
    assert np.lib.format.read_magic(f) == (1, 0)
    got_shape, fortran, dtype = np.lib.format.read_array_header_1_0(f)
    assert got_shape == tuple(shape) and not fortran and dtype == np.dtype(descr)
    assert f.tell() == n


def test_failure_check_entry_points_validate_on_the_host(lib):
    """pmgb_check_stats with no counters is a no-op; the wait-timeout probe
    rejects an out-of-range limit and a NULL status before any launch."""
    from jaxpm_gb300 import _lib
    assert _lib.call("pmgb_check_stats", None, None) == 0
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_test_wait_timeout", 0, ctypes.c_void_p(16), None)
    assert e.value.status == 1 and "spin_limit" in str(e.value)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_test_wait_timeout", 1 << 21, ctypes.c_void_p(16), None)
    assert "spin_limit" in str(e.value)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_test_wait_timeout", 100, None, None)
    assert "status is NULL" in str(e.value)


def test_tuning_round_trip_and_ranges(lib):
    """pmgb_set_tuning / pmgb_get_tuning round-trip every field and reject
    values outside their ranges on the host, leaving the settings as they
    were."""
    from jaxpm_gb300 import _lib
    before = _lib.get_tuning()
    try:
        _lib.set_tuning(gather_static_quarters=2, gather_ctas_per_sm=3, resort_ctas_per_sm=6,
                        resort_priority=1)
        assert _lib.get_tuning() == {"gather_static_quarters": 2, "gather_ctas_per_sm": 3,
                                     "resort_ctas_per_sm": 6, "resort_priority": 1}
        for bad in ({"gather_static_quarters": 5}, {"gather_ctas_per_sm": -1},
                    {"resort_ctas_per_sm": 33}, {"resort_priority": 2}):
            with pytest.raises(_lib.PmgbError) as e:
                _lib.set_tuning(**bad)
            assert e.value.status == 1
            assert _lib.get_tuning()["resort_ctas_per_sm"] == 6
    finally:
        _lib.set_tuning(**before)


def test_sorted_path_limits_are_checked_on_the_host(lib):
    """The sorted path's limits (32-bit particle slots, at most 256 tiles per
    axis) and the piecewise return's arguments are rejected before any GPU
    work, with the status and message of an invalid argument."""
    from jaxpm_gb300 import _lib
    P = ctypes.c_void_p(256)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_tile_sort_f32", P, None, None, 1 << 32, 64, 64, 64, P, None, P, P,
                  1 << 20, None)
    assert e.value.status == 1 and "32 bits" in str(e.value)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_tile_sort_dest_f32", P, None, None, 1000, 4096, 8, 8, P, None, P, P, P,
                  1 << 20, None)
    assert e.value.status == 1 and "tiles" in str(e.value)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_tile_sort_dest_f32", P, None, None, 1000, 64, 64, 64, P, None, P, None,
                  P, 1 << 20, None)
    assert "dest is NULL" in str(e.value)
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_gather3_f32", P, -1, P, 4, ctypes.c_void_p(1 << 20), None)
    assert e.value.status == 1 and "n_in" in str(e.value)
    with pytest.raises(_lib.PmgbError) as e:  # out overlaps the source
        _lib.call("pmgb_gather3_f32", ctypes.c_void_p(4096), 100, P, 10,
                  ctypes.c_void_p(4096 + 40), None)
    assert "overlap" in str(e.value)
    assert _lib.call("pmgb_gather3_f32", None, 0, None, 0, None, None) == 0  # nothing to do


def test_run_timing_switch_and_empty_read(lib):
    """pmgb_set_run_timing takes 0 or 1; pmgb_run_timing reports an error
    before any timed run (no GPU work)."""
    from jaxpm_gb300 import _lib
    with pytest.raises(_lib.PmgbError) as e:
        _lib.call("pmgb_set_run_timing", 2)
    assert e.value.status == 1
    _lib.set_run_timing(True)
    try:
        with pytest.raises(_lib.PmgbError) as e:
            _lib.run_timing()
        assert e.value.status == 1 and "no timed run" in str(e.value)
    finally:
        _lib.set_run_timing(False)
