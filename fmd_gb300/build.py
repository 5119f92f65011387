"""Build the GB300 engine in-tree (no cmake, no pip install).

    python -m fmd_gb300.build          # libfmd.so

Output (git-ignored):
  fmd_gb300/lib/libfmd.so   host C (fmd.h API) + sm_103a CUDA engine (fmdg.h)

The test infrastructure (the CPU oracle) has its own recipe,
oracle/build.py.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIBFMD = os.path.join(LIBDIR, "libfmd.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_libfmd(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cu = sorted(glob.glob(os.path.join(PKG, "csrc", "cuda", "*.cu")))
    cc = sorted(glob.glob(os.path.join(PKG, "csrc", "host", "*.c")))
    hdrs = glob.glob(os.path.join(PKG, "csrc", "*", "*.h*")) + glob.glob(os.path.join(INC, "*.h"))
    jobs = []
    objs = []
    for f in cu:
        o = os.path.join(BUILD, "cu_" + os.path.basename(f)[:-3] + ".o")
        objs.append(o)
        if _stale(o, [f] + hdrs):
            jobs.append([nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-I" + INC, "-c", f, "-o", o])
    for f in cc:
        o = os.path.join(BUILD, "c_" + os.path.basename(f)[:-2] + ".o")
        objs.append(o)
        if _stale(o, [f] + hdrs):
            jobs.append(["gcc", "-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-I" + INC,
                         "-I/usr/local/cuda/include", "-c", f, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for out in ex.map(_run, jobs):
            if verbose and out.strip():
                print(out)
    if _stale(LIBFMD, objs):
        _run([nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", LIBFMD, "-lm"])
    return LIBFMD


def build(verbose=False):
    return build_libfmd(verbose)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
