"""Build the CUDA shared library ``libgwlnl.so`` in-tree with nvcc for sm_103a.

The translation units compile in parallel; the library lands in
``bilby_gb300/_lib/``.  ``python -m bilby_gb300._build`` builds it from the
command line; ``__graft_entry__.build()`` calls :func:`build`.

``build(checked=True)`` (``--checked``) builds the debug variant
``libgwlnl_check.so`` with ``-DGWL_CHECK``: the kernels test the indices they
read from host-built tables before each access and report a failed test as
GWL_ERR_CHECK.  Setting ``GWL_CHECKED=1`` in the environment makes
``bilby_gb300._capi`` load that variant.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_lib", "obj")
LIB_PATH = os.path.join(OUT_DIR, "libgwlnl.so")
CHECKED_LIB_PATH = os.path.join(OUT_DIR, "libgwlnl_check.so")
SOURCES = ["gwl_capi.cu", "gwl_kernels.cu", "gwl_marg.cu", "gwl_marg_window.cu", "gwl_mb_fft.cu", "gwl_source.cu",
           "gwl_noalloc.cu", "gwl_priors.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build bilby_gb300")
    return path


def _compile(src: str, extra: list[str], obj_dir: str = OBJ_DIR) -> str:
    obj = os.path.join(obj_dir, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


def _stale(lib: str = LIB_PATH) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "gwlnl.h"), __file__]
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None,
          checked: bool = False) -> str:
    """Compile every translation unit and link ``libgwlnl.so`` (with
    ``checked``, ``libgwlnl_check.so``); returns its path."""
    lib = CHECKED_LIB_PATH if checked else LIB_PATH
    obj_dir = OBJ_DIR + "_check" if checked else OBJ_DIR
    if not force and not _stale(lib) and not extra:
        return lib
    os.makedirs(obj_dir, exist_ok=True)
    extra = list(extra or []) + (["-DGWL_CHECK"] if checked else [])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, obj_dir), SOURCES))
    cmd = [nvcc(), *ARCH, "-shared", "-o", lib, *objs, "-lcudart", "-lcublas", "-ldl"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else None, checked="--checked" in sys.argv)
