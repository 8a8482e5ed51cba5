"""In-tree build of the native parts (no setuptools, no cmake).

* ``lib/libgbx.so``    -- the CUDA C-ABI library (``csrc/*.cu``), compiled for
  sm_103a only.  This is the product.
* ``lib/_globule.so``  -- the seeded random-walk workload generator.

Translation units compile in parallel; objects are rebuilt only when a source
or header is newer than them.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
REPO = os.path.dirname(PKG)
INCLUDE = os.path.join(REPO, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA library cannot be built")


def _newer(src_paths, out) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(p) > t for p in src_paths)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def library_path() -> str:
    return os.path.join(LIBDIR, "libgbx.so")


def globule_library() -> str:
    out = os.path.join(LIBDIR, "_globule.so")
    src = os.path.join(CSRC, "globule_walk.c")
    if _newer([src], out):
        os.makedirs(LIBDIR, exist_ok=True)
        _run(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-std=c11", "-o", out, src, "-lm"])
    return out


def build_cuda(verbose: bool = False, extra_flags=None) -> str:
    """Compile every ``csrc/*.cu`` for sm_103a and link ``lib/libgbx.so``."""
    nvcc = _nvcc()
    os.makedirs(OBJDIR, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    flags = NVCC_FLAGS + list(extra_flags or [])
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _newer([src] + headers, obj):
            jobs.append([nvcc, *ARCH, *flags, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            logs = list(ex.map(_run, jobs))
    out = library_path()
    if jobs or _newer(objs, out):
        _run([nvcc, *ARCH, "-shared", "-o", out, *objs, "-lcudart", "-lcuda", "-lgomp"])
    if verbose:
        for line in logs:
            if line.strip():
                print(line)
    return out


def build_all(verbose: bool = False) -> None:
    globule_library()
    build_cuda(verbose=verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    print("built", library_path())
