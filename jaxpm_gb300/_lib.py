"""ctypes binding of ``libpmgb.so`` (the C ABI declared in ``include/pmgb.h``).

The library is loaded from ``jaxpm_gb300/_lib/libpmgb.so`` (built in-tree
by ``jaxpm_gb300.build``).  There is no fallback: if the library is missing
or fails to load, every GPU entry point raises ``PmgbUnavailable``.
Device buffers are torch CUDA tensors; calls are issued on the current
torch CUDA stream.
"""
import ctypes
import os

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libpmgb.so")

PMGB_OK = 0
PAINT_ATOMIC = 0
PAINT_BINNED = 1
PAINT_DETERMINISTIC = 2

_STATUS = {
    1: "invalid argument",
    2: "workspace",
    3: "CUDA error",
    4: "cuFFT error",
    5: "unsupported",
}

c_int, c_int64, c_float, c_size_t = ctypes.c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_size_t
P = ctypes.c_void_p

# name: (restype, argtypes)
SIGNATURES = {
    "pmgb_version": (c_int, []),
    "pmgb_last_error": (ctypes.c_char_p, []),
    "pmgb_launch_count": (ctypes.c_uint64, []),
    "pmgb_cic_paint_workspace_size": (c_size_t, [c_int, c_int, c_int, c_int64, c_int]),
    "pmgb_cic_paint_f32": (c_int, [P, c_int, c_int, c_int, P, c_int64, P, c_float, c_int, c_int,
                                   P, c_size_t, P]),
    "pmgb_cic_paint_deterministic_noalloc_f32": (c_int, [P, c_int, c_int, c_int, P, c_int64, P,
                                                         c_float, c_int, P]),
    "pmgb_check_stats": (c_int, [P, P]),
    "pmgb_read_potential_kick_drift_paint_perm_f32": (c_int, [P, c_int, c_int, c_int, P, P, P, P,
                                                              P, c_int64, c_float, c_float, P, P,
                                                              c_size_t, P, P]),
    "pmgb_tile_resort_index": (c_int, [c_int64, c_int, c_int, c_int, P, P, P, P, P, c_size_t,
                                       P]),
    "pmgb_gather_u32": (c_int, [P, P, c_int64, P, P]),
    "pmgb_test_wait_timeout": (c_int, [ctypes.c_uint32, P, P]),
    "pmgb_cic_read_f32": (c_int, [P, c_int, c_int, c_int, P, c_int64, P, P]),
    "pmgb_cic_read3_f32": (c_int, [P, c_int64, c_int, c_int, c_int, P, c_int64, P, P]),
    "pmgb_cic_weights_f32": (c_int, [P, c_int64, c_int, c_int, c_int, P, P, P]),
    "pmgb_cic_paint_vjp_f32": (c_int, [P, c_int, c_int, c_int, P, c_int64, P, c_float, P, P, P]),
    "pmgb_cic_read_vjp_f32": (c_int, [P, c_int, c_int, c_int, P, c_int64, P, P, P, P]),
    "pmgb_cic_paint_dx_f32": (c_int, [P, c_int, c_int, c_int, P, P, c_float, c_int, P]),
    "pmgb_cic_read_dx_f32": (c_int, [P, c_int, c_int, c_int, P, P, P]),
    "pmgb_enmesh_f32": (c_int, [P, c_int, c_int, c_int, P, P, P]),
    "pmgb_fft_r2c_f32": (c_int, [P, P, c_int, c_int, c_int, c_int, P]),
    "pmgb_fft_c2r_f32": (c_int, [P, P, c_int, c_int, c_int, c_int, c_int, P]),
    "pmgb_fft3_supported": (c_int, [c_int, c_int, c_int]),
    "pmgb_fft3_pitch": (c_int, [c_int]),
    "pmgb_fft3_r2c_f32": (c_int, [P, P, c_int, c_int, c_int, c_int, P]),
    "pmgb_fft3_c2r_f32": (c_int, [P, P, c_int, c_int, c_int, c_int, P]),
    "pmgb_set_fft_path": (c_int, [c_int]),
    "pmgb_get_tuning": (c_int, [P]),
    "pmgb_set_tuning": (c_int, [P]),
    "pmgb_set_run_timing": (c_int, [c_int]),
    "pmgb_run_timing": (c_int, [P, P, P, P]),
    "pmgb_fft_path": (c_int, []),
    "pmgb_mesh_forces_workspace_size": (c_size_t, [c_int, c_int, c_int]),
    "pmgb_mesh_forces_f32": (c_int, [P, P, c_int, c_int, c_int, c_float, P, c_size_t, P]),
    "pmgb_mesh_forces_vjp_f32": (c_int, [P, P, c_int, c_int, c_int, c_float, P, c_size_t, P]),
    "pmgb_mesh_potential_f32": (c_int, [P, P, c_int, c_int, c_int, c_float, P, c_size_t, P]),
    "pmgb_read_potential_kick_drift_paint_binned_f32": (c_int, [P, c_int, c_int, c_int, P, P,
                                                                c_int64, c_float, c_float, P, P,
                                                                c_size_t, P, P]),
    "pmgb_kspace_forces_f32": (c_int, [P, P, c_int64, c_int, c_int, c_int, c_float, c_int, c_int,
                                       c_float, P]),
    "pmgb_kspace_forces_vjp_f32": (c_int, [P, c_int64, P, c_int, c_int, c_int, c_float, c_int,
                                           c_int, c_float, P]),
    "pmgb_kspace_invlaplace_f32": (c_int, [P, c_int, c_int, c_int, c_int, c_float, P]),
    "pmgb_kspace_longrange_f32": (c_int, [P, c_int, c_int, c_int, c_float, P]),
    "pmgb_kspace_gradient_f32": (c_int, [P, P, c_int, c_int, c_int, c_int, c_int, P]),
    "pmgb_read3_kick_drift_f32": (c_int, [P, c_int64, c_int, c_int, c_int, P, P, c_int64,
                                          c_float, c_float, P, P]),
    "pmgb_kick_f32": (c_int, [P, P, c_int64, c_float, P]),
    "pmgb_drift_f32": (c_int, [P, P, c_int64, c_float, P]),
    "pmgb_pm_workspace_size": (c_size_t, [c_int, c_int, c_int, c_int64, c_int]),
    "pmgb_pm_forces_f32": (c_int, [P, c_int64, c_int, c_int, c_int, c_float, c_int, P, P,
                                   c_size_t, P]),
    "pmgb_fpm_step_f32": (c_int, [P, P, c_int64, c_int, c_int, c_int, c_float, c_float, c_float,
                                  c_int, P, c_size_t, P]),
    "pmgb_fpm_step_plain_f32": (c_int, [P, P, c_int64, c_int, c_int, c_int, c_float, c_float,
                                        c_float, P, c_size_t, P]),
    "pmgb_pm_forces_vjp_f32": (c_int, [P, c_int64, c_int, c_int, c_int, c_float, c_int, P, P, P,
                                       c_size_t, P]),
    "pmgb_linear_field_colour_f32": (c_int, [P, c_int, c_int, c_int, c_float, c_float, c_float,
                                             P, P, c_int, c_float, P]),
    "pmgb_lpt2_source_workspace_size": (c_size_t, [c_int, c_int, c_int]),
    "pmgb_lpt2_source_f32": (c_int, [P, P, c_int, c_int, c_int, P, c_size_t, P]),
    "pmgb_lpt_combine_f32": (c_int, [P, P, c_int64, c_float, c_float, P, P]),
    "pmgb_tile_sort_workspace_size": (c_size_t, [c_int, c_int, c_int, c_int64]),
    "pmgb_tile_sort_f32": (c_int, [P, P, P, c_int64, c_int, c_int, c_int, P, P, P, P, c_size_t,
                                   P]),
    "pmgb_unpermute3_f32": (c_int, [P, P, c_int64, P, P]),
    "pmgb_permute3_f32": (c_int, [P, P, c_int64, P, P]),
    "pmgb_tile_sort_dest_f32": (c_int, [P, P, P, c_int64, c_int, c_int, c_int, P, P, P, P, P,
                                        c_size_t, P]),
    "pmgb_gather3_f32": (c_int, [P, c_int64, P, c_int64, P, P]),
    "pmgb_fpm_coef_cotangents_f32": (c_int, [P, P, P, P, c_int64, c_int, c_int, c_int, P, P,
                                             c_int64, P, P]),
    "pmgb_read3_kick_drift_binned_f32": (c_int, [P, c_int64, c_int, c_int, c_int, P, P, c_int64,
                                                 c_float, c_float, P, c_size_t, P, P]),
    "pmgb_cic_paint_sorted_f32": (c_int, [P, c_int, c_int, c_int, P, c_int64, P, c_size_t, P, P]),
    "pmgb_tile_scatter_f32": (c_int, [P, P, P, c_int64, c_int, c_int, c_int, P, P, P, P, P,
                                      c_size_t, P]),
    "pmgb_fpm_step_sorted_f32": (c_int, [P, P, P, P, P, P, c_int64, c_int, c_int, c_int, c_float,
                                         c_float, c_float, P, c_size_t, P, c_size_t, P, P, P, P,
                                         P]),
    "pmgb_read3_kick_drift_paint_binned_f32": (c_int, [P, c_int64, c_int, c_int, c_int, P, P,
                                                       c_int64, c_float, c_float, P, P,
                                                       c_size_t, P, P]),
    "pmgb_fpm_run_sorted_f32": (c_int, [P, P, P, P, P, P, c_int64, c_int, c_int, c_int, c_int,
                                        P, P, c_float, P, c_size_t, P, c_size_t, P, P]),
    "pmgb_fpm_run_sorted_record_f32": (c_int, [P, P, P, P, P, P, c_int64, c_int, c_int, c_int,
                                               c_int, P, P, c_float, P, c_size_t, P, c_size_t, P,
                                               P, P, P, P]),
    "pmgb_fpm_run_sorted_record_pot_f32": (c_int, [P, P, P, P, P, P, c_int64, c_int, c_int,
                                                   c_int, c_int, P, P, c_float, P, c_size_t, P,
                                                   c_size_t, P, P, P, P, P]),
    "pmgb_tile_key_count": (c_int64, [c_int, c_int, c_int]),
    "pmgb_fpm_step_sorted_vjp_f32": (c_int, [P, P, P, P, P, P, P, P, c_int64, c_int, c_int, c_int,
                                             c_float, c_float, c_float, P, c_size_t, P, P]),
    "pmgb_fpm_step_sorted_vjp_pot_f32": (c_int, [P, P, P, P, P, P, P, P, c_int64, c_int, c_int,
                                                 c_int, c_float, c_float, c_float, P, c_size_t, P,
                                                 P]),
    "pmgb_power_spectrum_f32": (c_int, [P, c_int, c_int, c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, P, c_int, P, P, P, P]),
    "pmgb_lpt2_source_vjp_f32": (c_int, [P, P, P, c_int, c_int, c_int, P, c_size_t, P]),
    "pmgb_npy_header": (c_size_t, [ctypes.c_char_p, P, c_int, P, c_size_t]),
    "pmgb_snapshot_begin_npy": (c_int, [ctypes.c_char_p, P, ctypes.c_char_p, c_int, P, c_int, P,
                                        c_size_t, P, P]),
    "pmgb_snapshot_wait": (c_int, [P]),
    "pmgb_batch_workspace_size": (c_size_t, [P, c_int]),
    "pmgb_batch_init": (c_int, [P, c_int, P, c_size_t, P]),
    "pmgb_batch_release": (c_int, [P]),
    "pmgb_batch_counts": (c_int, [P, c_int, P, P]),
    "pmgb_cic_paint_batched_f32": (c_int, [P, c_int, P, P, P, c_size_t, P]),
    "pmgb_pm_forces_batched_f32": (c_int, [P, c_int, P, P, c_float, P, c_size_t, P]),
    "pmgb_fpm_step_batched_f32": (c_int, [P, c_int, P, P, P, P, c_float, P, P, c_size_t, P]),
    "pmgb_fpm_step_batched_vjp_f32": (c_int, [P, c_int, P, P, P, P, P, c_float, P, c_size_t,
                                              P]),
}


class Sim(ctypes.Structure):
    """``pmgb_sim``: one simulation of a batch (mesh shape, particle count)."""
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("np", ctypes.c_int64)]


def sim_table(shapes, counts):
    """A ctypes ``pmgb_sim`` array for mesh ``shapes`` and particle ``counts``."""
    arr = (Sim * len(shapes))()
    for i, (sh, n) in enumerate(zip(shapes, counts)):
        arr[i].nx, arr[i].ny, arr[i].nz = (int(v) for v in sh)
        arr[i].reserved = 0
        arr[i].np = int(n)
    return arr


class Tuning(ctypes.Structure):
    """``pmgb_tuning``: launch choices of the tile-sorted run loop."""
    _fields_ = [("gather_static_quarters", ctypes.c_int32),
                ("gather_ctas_per_sm", ctypes.c_int32),
                ("resort_ctas_per_sm", ctypes.c_int32),
                ("resort_priority", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 4)]


def get_tuning():
    t = Tuning()
    call("pmgb_get_tuning", ctypes.byref(t))
    return {"gather_static_quarters": t.gather_static_quarters,
            "gather_ctas_per_sm": t.gather_ctas_per_sm,
            "resort_ctas_per_sm": t.resort_ctas_per_sm,
            "resort_priority": t.resort_priority}


def set_tuning(gather_static_quarters=3, gather_ctas_per_sm=0, resort_ctas_per_sm=0,
               resort_priority=0):
    t = Tuning()
    t.gather_static_quarters = int(gather_static_quarters)
    t.gather_ctas_per_sm = int(gather_ctas_per_sm)
    t.resort_ctas_per_sm = int(resort_ctas_per_sm)
    t.resort_priority = int(resort_priority)
    call("pmgb_set_tuning", ctypes.byref(t))


def set_run_timing(enable):
    """Switches the run loop's launch timing on or off (``pmgb_set_run_timing``)."""
    call("pmgb_set_run_timing", 1 if enable else 0)


def run_timing():
    """The last timed run's mean milliseconds per launch of its gathers, force
    evaluations and re-sorts (``pmgb_run_timing``; its stream must have been
    synchronised)."""
    g, f, r = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    n = ctypes.c_int()
    call("pmgb_run_timing", ctypes.byref(g), ctypes.byref(f), ctypes.byref(r), ctypes.byref(n))
    return {"read_kick_drift": g.value, "forces": f.value, "sort": r.value, "steps": n.value}


class PmgbError(RuntimeError):
    """A libpmgb call returned an error status."""


class PmgbUnavailable(RuntimeError):
    """libpmgb.so is not built or cannot be loaded."""


_lib = None


def load():
    """Loads (once) and returns the ctypes handle of libpmgb.so."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise PmgbUnavailable(
            f"{LIB_PATH} is missing: build it with `python -m jaxpm_gb300.build`")
    try:
        lib = ctypes.CDLL(LIB_PATH)
    except OSError as e:
        raise PmgbUnavailable(f"cannot load {LIB_PATH}: {e}") from e
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def call(name, *args):
    """Calls ``name`` and raises ``PmgbError`` on a non-zero status."""
    lib = load()
    status = getattr(lib, name)(*args)
    if status != PMGB_OK:
        msg = lib.pmgb_last_error().decode(errors="replace")
        kind = _STATUS.get(status, f"status {status}")
        err = PmgbError(f"{name}: {kind}: {msg}")
        err.status = status
        raise err
    return status


def ptr(t):
    """Device pointer of a tensor (None/NULL for None)."""
    if t is None:
        return None
    return ctypes.c_void_p(t.data_ptr())


def stream(device=None):
    """The current torch CUDA stream as a cudaStream_t value."""
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def require_cuda(*tensors):
    """Checks that every tensor is a contiguous float32/complex64 CUDA tensor
    on one device; the GPU path has no CPU fallback."""
    dev = None
    for t in tensors:
        if t is None:
            continue
        if not t.is_cuda:
            raise ValueError("jaxpm_gb300 runs on CUDA tensors only; got a tensor on "
                             f"{t.device}")
        if not t.is_contiguous():
            raise ValueError("jaxpm_gb300 expects contiguous tensors")
        if dev is None:
            dev = t.device
        elif t.device != dev:
            raise ValueError(f"tensors on different devices: {dev} and {t.device}")
    return dev
