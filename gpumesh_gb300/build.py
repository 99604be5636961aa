"""Build libgpumesh_gb300.so in-tree with nvcc for sm_103a.

Each translation unit is compiled in parallel into gpumesh_gb300/_build/,
then linked into gpumesh_gb300/_lib/libgpumesh_gb300.so.  A unit is rebuilt
when it or any header under csrc/ or include/ is newer than its object.

build(checked=True) builds the bounds-checked variant instead
(-DGM_BOUNDS_CHECK, objects in _build/checked/,
_lib/libgpumesh_gb300_checked.so): every connectivity and neighbourhood
index the kernels read is checked against its array's length.  Setting
GPUMESH_GB300_LIB=checked makes gpumesh_gb300._native load it.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libgpumesh_gb300.so")
LIB_CHECKED = os.path.join(LIBDIR, "libgpumesh_gb300_checked.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                     "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(ROOT, "include", "*.h"))


def _compile(src: str, verbose_ptxas: bool, checked: bool = False) -> str:
    obj = os.path.join(BUILD, "checked" if checked else "", os.path.basename(src) + ".o")
    defs = ["-DGM_BOUNDS_CHECK=1"] if checked else []
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest and not verbose_ptxas:
        return obj
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVCC_FLAGS + defs + (["-Xptxas", "-v"] if verbose_ptxas else []) + ["-c", src, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + defs + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose_ptxas: bool = False, checked: bool = False) -> str:
    lib = LIB_CHECKED if checked else LIB
    os.makedirs(os.path.join(BUILD, "checked") if checked else BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(os.cpu_count() or 8, 16, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas, checked), srcs))
    if not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return lib


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv, checked="--checked" in sys.argv))
