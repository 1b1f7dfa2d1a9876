"""Builds and loads ``oracle/ccic.c``, the C statement of the oracle's CIC
paint and read (test infrastructure only).

``build()`` compiles it with ``gcc -O2 -fopenmp -ffp-contract=off`` into
``oracle/_build/libccic.so`` (git-ignored; rebuilt on each machine).
``lib()`` returns the loaded library, building it on first use, or None
when no C compiler is available, in which case ``oracle/cic.py`` keeps to
its NumPy statement.
"""
import ctypes
import os
import subprocess
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "ccic.c")
OUT = os.path.join(HERE, "_build", "libccic.so")

_LOCK = threading.Lock()
_LIB = [None, False]  # library, load attempted


def build(force=False):
    """Compiles the C oracle; returns the library path."""
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) > os.path.getmtime(SRC):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    tmp = OUT + f".{os.getpid()}.tmp"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
           SRC, "-o", tmp, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"gcc failed on {SRC}:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


def _declare(lib):
    P = ctypes.c_void_p
    I = ctypes.c_int
    L = ctypes.c_int64
    for sfx, real in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
        f = getattr(lib, f"oc_read_{sfx}")
        f.argtypes = [P, I, I, I, P, L, P]
        f.restype = None
        f = getattr(lib, f"oc_paint_{sfx}")
        f.argtypes = [P, I, I, I, P, L, P, real]
        f.restype = None
        f = getattr(lib, f"oc_grad_{sfx}")
        f.argtypes = [P, I, I, I, P, L, P]
        f.restype = None
        f = getattr(lib, f"oc_weights_{sfx}")
        f.argtypes = [P, L, I, I, I, P, P]
        f.restype = None
    lib.oc_threads.argtypes = []
    lib.oc_threads.restype = I


def lib():
    """The loaded C oracle, or None where it cannot be built."""
    with _LOCK:
        if not _LIB[1]:
            _LIB[1] = True
            try:
                path = build()
                handle = ctypes.CDLL(path)
                _declare(handle)
                _LIB[0] = handle
            except (OSError, RuntimeError):
                _LIB[0] = None
        return _LIB[0]


def threads():
    h = lib()
    return int(h.oc_threads()) if h is not None else 1
