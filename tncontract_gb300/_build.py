"""Build recipe for the in-tree native library ``_lib/libtncontract_gb300.so``.

Each ``csrc/*.cu`` translation unit is compiled for sm_103a (GB300) in
parallel with nvcc, then linked into one shared library against the shared
CUDA runtime (so it shares the runtime that PyTorch already loaded).  The
build is incremental: nothing is recompiled when the library is newer than
every source and header.  No cmake, no setuptools.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUTDIR = os.path.join(PKG, "_lib")
BUILDDIR = os.path.join(ROOT, "_build")
LIBNAME = "libtncontract_gb300.so"
LIBPATH = os.path.join(OUTDIR, LIBNAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-O3", "--expt-relaxed-constexpr"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tncontract_gb300")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def _deps():
    return (_sources() + glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(ROOT, "include", "*.h")) + [__file__])


def up_to_date() -> bool:
    if not os.path.exists(LIBPATH):
        return False
    t = os.path.getmtime(LIBPATH)
    return all(os.path.getmtime(p) <= t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link the library; returns its path.  Raises on failure."""
    if not force and up_to_date():
        return LIBPATH
    nvcc = _nvcc()
    os.makedirs(OUTDIR, exist_ok=True)
    os.makedirs(BUILDDIR, exist_ok=True)
    procs = []
    objs = []
    for src in _sources():
        obj = os.path.join(BUILDDIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        cmd = [nvcc] + NVCC_FLAGS + ["-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out.decode(errors="replace")))
        elif verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
    if failed:
        msg = "\n".join("%s:\n%s" % f for f in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    tmp = LIBPATH + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-cudart=shared", "-o", tmp] + objs + \
        ["-Xlinker", "-rpath=/usr/local/cuda/lib64"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIBPATH)
    return LIBPATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
