"""The drop-in boundary seen from C (programs written against FMD relink
unchanged: `gcc prog.c -lfmd`, examples/01_argon.c:9).

CPU, with the reference checkout ($FMD_REFERENCE, default /root/reference;
skipped without it):
  * the reference's four example programs (examples/0[1-4]_*.c) compile
    unchanged against include/fmd.h -- implicit declarations, incompatible
    pointer types and int conversions are errors -- and link with -lfmd
    against libfmd.so;
  * both headers declare the same prototypes (gcc -aux-info, normalised);
  * every struct typedef of the reference header has the same size and
    member offsets, and every enumerator the same value, under both.
GPU: tests/c/argon_relink.c -- the argon example's call sequence from a
state file -- compiled against include/fmd.h, linked with -lfmd and run;
its printed temperature / total-energy series (T, E relative 1e-9) and the
state and configuration files it writes (numbers within 1e-8) match the
same source compiled against the reference's fmd.h and run on the
reference library (golden argon_c.npz, tests/golden/make_golden.py).
"""
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "fmd_gb300", "lib")
REF = os.environ.get("FMD_REFERENCE", "/root/reference")
CFLAGS = ["-std=c11", "-O1", "-Werror=implicit-function-declaration", "-Werror=incompatible-pointer-types",
          "-Werror=int-conversion"]

needs_ref = pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "src", "fmd.h")),
                               reason="reference checkout absent")


def _gcc(args, cwd=None):
    r = subprocess.run(["gcc", *args], capture_output=True, text=True, cwd=cwd)
    assert r.returncode == 0, r.stderr[-3000:]
    return r


@needs_ref
@pytest.mark.parametrize("example", ["01_argon.c", "02_collision.c", "03_ttm1.c", "04_ttm2.c"])
def test_reference_examples_relink(lib, example):
    src = os.path.join(REF, "examples", example)
    with tempfile.TemporaryDirectory() as work:
        exe = os.path.join(work, example[:-2] + ".x")
        _gcc([*CFLAGS, src, "-I" + INC, "-L" + LIBDIR, "-lfmd", "-lm", "-o", exe])
        assert os.path.getsize(exe) > 0


def _prototypes(inc):
    with tempfile.TemporaryDirectory() as work:
        c = os.path.join(work, "t.c")
        open(c, "w").write("#include <fmd.h>\n")
        aux = os.path.join(work, "aux.txt")
        _gcc(["-std=c11", "-fsyntax-only", "-aux-info", aux, "-I" + inc, c])
        lines = [ln for ln in open(aux) if "fmd.h" in ln]
    return sorted(re.sub(r"/\*.*?\*/", "", ln).strip() for ln in lines)


@needs_ref
def test_same_prototypes():
    ours, theirs = _prototypes(INC), _prototypes(os.path.join(REF, "src"))
    assert len(theirs) > 50
    assert ours == theirs


def _layout_program(header_text):
    """C source printing sizeof / offsetof of every struct typedef and the
    value of every enumerator of the given header text."""
    body = []
    txt = re.sub(r"/\*.*?\*/", "", header_text, flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    for m in re.finditer(r"typedef\s+struct\s*(?:\w+\s*)?\{(.*?)\}\s*(\w+)\s*;", txt, flags=re.S):
        fields, name = m.group(1), m.group(2)
        body.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for decl in fields.split(";"):
            ids = re.findall(r"(\w+)\s*(?:\[[^\]]*\])?\s*$", decl.strip())
            for f in ids:
                body.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    for m in re.finditer(r"typedef\s+enum\s*\{(.*?)\}\s*(\w+)\s*;", txt, flags=re.S):
        for e in re.findall(r"\b(FMD_\w+)", m.group(1)):
            body.append(f'printf("{e} %d\\n", (int){e});')
    return "#include <stddef.h>\n#include <stdio.h>\n#include <fmd.h>\nint main(void)\n{\n" + \
        "\n".join("    " + b for b in body) + "\n    return 0;\n}\n"


@needs_ref
def test_same_layouts_and_enums():
    prog = _layout_program(open(os.path.join(REF, "src", "fmd.h")).read())
    outs = []
    with tempfile.TemporaryDirectory() as work:
        c = os.path.join(work, "layout.c")
        open(c, "w").write(prog)
        for inc in (INC, os.path.join(REF, "src")):
            exe = os.path.join(work, "layout.x")
            _gcc(["-std=c11", c, "-I" + inc, "-o", exe])
            outs.append(subprocess.run([exe], capture_output=True, text=True, check=True).stdout)
    assert outs[0].count("\n") > 40
    assert outs[0] == outs[1]


def _numbers(raw):
    toks = raw.decode().split()
    num, txt = [], []
    for t in toks:
        try:
            num.append(float(t))
        except ValueError:
            txt.append(t)
    return np.array(num), txt


@pytest.mark.gpu
def test_argon_program_matches_reference(gpu_lib):
    g = dict(np.load(os.path.join(HERE, "golden", "argon_c.npz")))
    with tempfile.TemporaryDirectory() as work:
        exe = os.path.join(work, "argon.x")
        _gcc([*CFLAGS, os.path.join(HERE, "c", "argon_relink.c"), "-I" + INC, "-L" + LIBDIR, "-lfmd",
              "-Wl,-rpath," + LIBDIR, "-o", exe])
        st = os.path.join(work, "state0.stt")
        open(st, "wb").write(g["state0"].tobytes())
        out = os.path.join(work, "out") + "/"
        os.makedirs(out)
        r = subprocess.run([exe, st, out, "0.4"], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        files = sorted(os.listdir(out))
        got = {f: open(os.path.join(out, f), "rb").read() for f in files}
    assert files == list(g["files"])
    mine = [ln.split() for ln in r.stdout.splitlines()]
    ref = [ln.split() for ln in g["stdout"].tobytes().decode().splitlines()]
    assert [m[0] for m in mine] == [q[0] for q in ref]
    ticks_m = np.array([[float(v) for v in m[1:]] for m in mine if m[0] == "tick"])
    ticks_r = np.array([[float(v) for v in q[1:]] for q in ref if q[0] == "tick"])
    assert ticks_m.shape == ticks_r.shape and len(ticks_r) == 9
    np.testing.assert_allclose(ticks_m[:, 0], ticks_r[:, 0], rtol=0, atol=1e-12)
    np.testing.assert_allclose(ticks_m[:, 1:], ticks_r[:, 1:], rtol=1e-9, atol=0)
    assert mine[-1] == ref[-1]
    for f in files:
        nm, tm = _numbers(got[f])
        nr, tr = _numbers(g["file:" + f].tobytes())
        assert tm == tr, f
        assert nm.shape == nr.shape, f
        assert np.abs(nm - nr).max() <= 1e-8, (f, np.abs(nm - nr).max())
