"""In-tree build of libdfxgpu.so for sm_103a (no cmake).

Every CUDA translation unit is compiled by nvcc with
``-gencode arch=compute_103a,code=sm_103a`` in parallel, the host set-up
code by g++, and the objects are linked into ``dolfinx_gb300/_lib/``.
Objects are rebuilt only when a source or header is newer.
"""

from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OUT = os.path.join(PKG, "_lib")
OBJ = os.path.join(PKG, "_build")
LIBNAME = "libdfxgpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA extension cannot be built")
    return cand


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(obj, src, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src, *deps])


def _compile(src: str, verbose_ptxas: bool) -> str:
    name = os.path.splitext(os.path.basename(src))[0]
    obj = os.path.join(OBJ, name + ".o")
    if not _stale(obj, src, _headers()) and not verbose_ptxas:
        return obj
    if src.endswith(".cu"):
        cmd = [nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++20", "--expt-relaxed-constexpr",
               "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
    else:
        # -ffp-contract=off: a*b+c rounds twice on aarch64 as on x86-64
        # (no FMA contraction), so the host set-up gives the same doubles
        # on both, and the same as the device's explicitly unfused
        # arithmetic where the two must agree bit for bit.
        cmd = ["g++", "-O3", "-std=c++20", "-fPIC", "-Wall", "-ffp-contract=off", "-I", INCLUDE,
               "-I", "/usr/local/cuda/include", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        print(r.stderr)
    return obj


def build(verbose_ptxas: bool = False) -> str:
    """Compile and link libdfxgpu.so; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    lib = os.path.join(OUT, LIBNAME)
    if not os.path.exists(lib) or any(os.path.getmtime(o) > os.path.getmtime(lib) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", lib, *objs, "-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return lib


if __name__ == "__main__":
    import sys
    print(build(verbose_ptxas="-v" in sys.argv))
