"""Build libimdgpu.so (sm_103a) in-tree with nvcc.

Each translation unit compiles in parallel to an object under
imd_gb300/_build/, then one link step writes imd_gb300/libimdgpu.so.
Run as `python -m imd_gb300.build` or through __graft_entry__.build().

`python -m imd_gb300.build --check` (build(check=True)) writes the
bounds-checked variant, compiled with -DIMDGPU_CHECK, to
imd_gb300/libimdgpu_check.so (objects under imd_gb300/_build_check/).
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
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libimdgpu.so")
BUILD_CHECK = os.path.join(HERE, "_build_check")
LIB_CHECK = os.path.join(HERE, "libimdgpu_check.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr",
           "-I" + os.path.join(ROOT, "include")]
SOURCES = ["system.cu", "forces.cu", "mixed.cu", "batch.cu", "learn.cu", "noalloc.cu", "output.cu",
           "potfile.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str], bdir: str = BUILD) -> str:
    obj = os.path.join(bdir, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    cmd = [nvcc()] + ARCH + NVFLAGS + extra + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj


def _stale(lib: str) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(ROOT, "include", "imdgpu.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None,
          check: bool = False) -> str:
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    lib, bdir = (LIB_CHECK, BUILD_CHECK) if check else (LIB, BUILD)
    if not force and not _stale(lib):
        return lib
    os.makedirs(bdir, exist_ok=True)
    extra = list(extra or []) + (["-DIMDGPU_CHECK"] if check else [])
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, bdir), srcs))
    tmp = lib + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib)
    if verbose:
        print("built", lib)
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None,
          check="--check" in sys.argv)
