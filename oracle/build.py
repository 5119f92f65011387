"""Build recipe of the test infrastructure under oracle/ (never linked into
the product library):

  oracle/liboracle.so       the CPU restatement of the reference's hot path
                            (fmd_oracle.c): the checker of the parity tests and
                            the timed CPU baseline
  oracle/_ref/libfmdref.so  the reference compiled from its own, unmodified
                            sources with single-process shims (Makefile.ref),
                            only where those sources are present: the
                            reference checkout at $FMD_REFERENCE, default
                            /root/reference (absent on the GPU host)

    python oracle/build.py
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
ORACLE_LIB = os.path.join(HERE, "liboracle.so")


def reference_src():
    return os.environ.get("FMD_REFERENCE", "/root/reference")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle():
    src = os.path.join(HERE, "fmd_oracle.c")
    deps = [src] + glob.glob(os.path.join(HERE, "*.h"))
    if _stale(ORACLE_LIB, deps):
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              "-I" + HERE, src, "-o", ORACLE_LIB, "-lm"])
    return ORACLE_LIB


def build_reference():
    """Compile the reference from its own sources (only where present)."""
    ref = reference_src()
    if not os.path.isdir(os.path.join(ref, "src")):
        return None
    _run(["make", "-s", "-C", ROOT, "-f", "oracle/Makefile.ref", "REF=" + ref, "-j8"])
    return os.path.join(HERE, "_ref", "libfmdref.so")


def build_all():
    build_oracle()
    build_reference()


if __name__ == "__main__":
    build_all()
    print(ORACLE_LIB)
