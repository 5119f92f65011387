"""State and configuration files (fmd_io_saveState, src/misc.c:310-422;
fmd_matt_saveConfiguration in XYZ, CSV and VTF modes, src/matter.c:650-829)
against the files the reference writes (tests/golden/io_*.npz, made by
tests/golden/make_golden.py).

Right after distribution the files must be byte-identical (same atoms, same
order, same formatting).  After the case's run the positions agree to the
trajectory tolerance only: the state file's numbers within 1e-8, the
configurations' two-decimal coordinates within one unit of the last digit,
every other token identical.
"""
import os
import re
import tempfile

import numpy as np
import pytest

import cases

HERE = os.path.dirname(os.path.abspath(__file__))
MODES = [("xyz", 1), ("csv", 2), ("vtf", 3)]

pytestmark = pytest.mark.gpu


def _files(lib, md, work, tag):
    out = {}
    lib.fmd_io_setSaveDirectory(md, (work + "/").encode())
    lib.fmd_io_saveState(md, (tag + ".stt").encode())
    out[tag + "_state"] = open(os.path.join(work, tag + ".stt"), "rb").read()
    for name, mode in MODES:
        before = set(os.listdir(work))
        lib.fmd_io_setSaveConfigMode(md, mode)
        lib.fmd_matt_saveConfiguration(md)
        new = sorted(set(os.listdir(work)) - before)
        assert len(new) == 1, (name, new)
        out[tag + "_" + name] = open(os.path.join(work, new[0]), "rb").read()
        os.remove(os.path.join(work, new[0]))
    return out


NUM = re.compile(r"^[-+]?\d+(\.\d*)?([eE][-+]?\d+)?,?$")


def _close(ours, ref, tol):
    a, b = ours.decode().split(), ref.decode().split()
    assert len(a) == len(b)
    for u, w in zip(a, b):
        if NUM.match(w) and ("." in w or "e" in w):
            assert abs(float(u.rstrip(",")) - float(w.rstrip(","))) <= tol, (u, w)
        else:
            assert u == w, (u, w)


@pytest.mark.parametrize("name", ["lj_small", "hybrid"])
def test_files_match_reference(gpu_lib, name):
    lib = gpu_lib
    ref = dict(np.load(os.path.join(HERE, "golden", "io_" + name + ".npz")))
    ref = {k: bytes(v) for k, v in ref.items()}
    case = cases.CASES[name]
    with tempfile.TemporaryDirectory() as work:
        md, _ = cases.setup(lib, name, work)
        lib.fmd_dync_integrate(md, case["run"][1], 0.0, case["run"][2])
        ours = _files(lib, md, work, "s0")
        cases.run(lib, name, md, None)
        ours.update(_files(lib, md, work, "s1"))
        lib.fmd_free(md)
    for key in ("s0_state", "s0_xyz", "s0_csv", "s0_vtf"):
        assert ours[key] == ref[key], key
    _close(ours["s1_state"], ref["s1_state"], 1e-8)
    for key in ("s1_xyz", "s1_csv", "s1_vtf"):
        _close(ours[key], ref[key], 0.0100001)
