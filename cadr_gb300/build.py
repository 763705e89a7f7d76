"""Build recipe of libcadr_cuda.so (the C ABI of the pass, CUDA for sm_103a).

Every .cu file under cadr_gb300/csrc is compiled by nvcc with
`-gencode arch=compute_103a,code=sm_103a` in parallel, then linked into
cadr_gb300/_lib/libcadr_cuda.so (kept in-tree, git-ignored).  No cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libcadr_cuda.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
              "-prec-div=true", "-prec-sqrt=true", "-fmad=false", "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources() -> list:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target: str, deps: list) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _build_cuda(obj_dir: str, lib: str, defines: list, force: bool, ptxas_info: bool = False,
                verbose: bool = False) -> str:
    """Compiles every .cu under csrc into obj_dir (in parallel, skipping
    objects newer than their sources and headers) and links them into lib."""
    os.makedirs(obj_dir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "cadr_cuda.h"))
    srcs = sources()
    objs = [os.path.join(obj_dir, os.path.basename(s)[:-3] + ".o") for s in srcs]
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(pair):
        src, obj = pair
        if not force and not ptxas_info and not _stale(obj, [src] + headers):
            return ""
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *defines, *extra, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        logs = list(ex.map(compile_one, zip(srcs, objs)))
    if verbose or ptxas_info:
        for lg in logs:
            if lg:
                sys.stderr.write(lg)
    if force or _stale(lib, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", lib, *objs, "-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return lib


def build(verbose: bool = False, ptxas_info: bool = False, force: bool = False) -> str:
    _build_cuda(OUT_DIR, LIB, [], force, ptxas_info, verbose)
    build_facade(force=force)
    return LIB


CHECKED_DIR = os.path.join(OUT_DIR, "checked")
CHECKED_LIB = os.path.join(OUT_DIR, "libcadr_cuda_checked.so")


def build_checked(force: bool = False) -> str:
    """The bounds-checked build of the same sources (CADR_BOUNDS_CHECK
    defined): every index a kernel derives itself is checked before the
    access it guards, a failed check sets CADR_DEVERR_BOUNDS and skips the
    access.  For tests on small cases; it is not the product library."""
    return _build_cuda(CHECKED_DIR, CHECKED_LIB, ["-DCADR_BOUNDS_CHECK"], force)


FACADE_DIR = os.path.join(HERE, "facade")
FACADE_LIB = os.path.join(OUT_DIR, "libcadr.so")


def build_facade(force: bool = False) -> str:
    """The C++ facade (include/CadR/*.h) over the C ABI: libcadr.so, which
    links libcadr_cuda.so from the same directory."""
    srcs = sorted(os.path.join(FACADE_DIR, f) for f in os.listdir(FACADE_DIR) if f.endswith(".cpp"))
    inc = os.path.join(ROOT, "include")
    deps = srcs + [os.path.join(inc, "cadr_cuda.h")] + [
        os.path.join(inc, "CadR", f) for f in os.listdir(os.path.join(inc, "CadR"))]
    if not force and not _stale(FACADE_LIB, deps + [LIB]):
        return FACADE_LIB
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-Wall", "-I", inc, *srcs, "-o", FACADE_LIB,
           "-L", OUT_DIR, "-lcadr_cuda", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"facade build failed:\n{r.stdout}\n{r.stderr}")
    return FACADE_LIB


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="--ptxas" in sys.argv, force="--force" in sys.argv))
