"""Builds ``libpmgb.so`` in-tree from ``jaxpm_gb300/csrc/*.cu`` for sm_103a.

Each translation unit is compiled by ``nvcc`` in parallel, then linked
into ``jaxpm_gb300/_lib/libpmgb.so`` against the shared CUDA runtime and
cuFFT.  Host code is compiled with ``-ffp-contract=off`` so that float32
tables computed on the host do not depend on the machine's FMA contraction.
Usage: ``python -m jaxpm_gb300.build [--force]``.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libpmgb.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home():
    return os.environ.get("CUDA_HOME", "/usr/local/cuda")


def nvcc():
    return os.path.join(cuda_home(), "bin", "nvcc")


def sources():
    return sorted(os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _mtime(p):
    return os.path.getmtime(p) if os.path.exists(p) else -1.0


def compile_flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                   "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE]


def _compile(src, verbose):
    obj = os.path.join(OBJ_DIR, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc()] + compile_flags() + ["-c", src, "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, (r.stdout + r.stderr)


def build(force=False, verbose=False):
    """Compiles every kernel source and links the shared library; returns
    its path.  Rebuilds only when a source or header is newer than it."""
    os.makedirs(OBJ_DIR, exist_ok=True)
    srcs = sources()
    newest = max(_mtime(p) for p in srcs + headers() + [os.path.abspath(__file__)])
    if not force and _mtime(LIB) > newest:
        return LIB
    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    libdir = os.path.join(cuda_home(), "lib64")
    tmp = LIB + ".tmp"
    cmd = ([nvcc()] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] +
           ["-cudart", "shared", "-L", libdir, "-lcufft",
            "-Xlinker", "-rpath," + libdir])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
