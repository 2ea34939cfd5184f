"""Build the CUDA library ``libnsgb.so`` in-tree with nvcc for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel to an object file
under ``_build/`` and the objects are linked into ``_lib/libnsgb.so`` (both
git-ignored).  A unit is recompiled only when it, or a header, is newer than
its object.  ``build_checked()`` builds the bounds-checking variant
``_lib/libnsgb_checked.so`` (NSGB_CHECK_BOUNDS; objects under
``_build/checked/``), which the tests load on their own.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libnsgb.so")
LIB_CHECKED = os.path.join(LIBDIR, "libnsgb_checked.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-I", INCLUDE, "-I", CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnsgb.so")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(INCLUDE, "nsgb.h"))
    return hs


def _compile(src: str, verbose_ptxas: bool, objdir: str = BUILD, defines=()) -> tuple[str, str]:
    obj = os.path.join(objdir, src[:-3] + ".o")
    cmd = [nvcc(), *ARCH, *NVFLAGS, *[f"-D{d}" for d in defines], "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int | None = None) -> str:
    """Compile and link libnsgb.so if stale; return its path."""
    return _build_lib(LIB, BUILD, (), force, verbose_ptxas, jobs, ())


def build_checked(force: bool = False, jobs: int | None = None) -> str:
    """Compile and link the bounds-checking libnsgb_checked.so if stale.  Its
    internal references bind to its own definitions (-Bsymbolic), so it can be
    loaded into a process that also holds libnsgb.so."""
    return _build_lib(LIB_CHECKED, os.path.join(BUILD, "checked"), ("NSGB_CHECK_BOUNDS",), force, False, jobs,
                      ("-Xlinker", "-Bsymbolic"))


def _build_lib(lib: str, objdir: str, defines, force: bool, verbose_ptxas: bool, jobs, link_flags) -> str:
    os.makedirs(objdir, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    newest_hdr = max(os.path.getmtime(h) for h in _headers())
    todo = []
    for s in srcs:
        obj = os.path.join(objdir, s[:-3] + ".o")
        src_t = max(os.path.getmtime(os.path.join(CSRC, s)), newest_hdr)
        if force or verbose_ptxas or not os.path.exists(obj) or os.path.getmtime(obj) < src_t:
            todo.append(s)
    logs = {}
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            for s, (obj, log) in zip(todo, ex.map(lambda s: _compile(s, verbose_ptxas, objdir, defines), todo)):
                logs[s] = log
    objs = [os.path.join(objdir, s[:-3] + ".o") for s in srcs]
    if todo or not os.path.exists(lib) or os.path.getmtime(lib) < max(os.path.getmtime(o) for o in objs):
        tmp = lib + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", *link_flags, "-o", tmp, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    if verbose_ptxas:
        for s, log in logs.items():
            sys.stderr.write(f"==== {s}\n{log}")
    return lib


if __name__ == "__main__":
    if "--checked" in sys.argv:
        print(build_checked(force="--force" in sys.argv))
    else:
        print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
