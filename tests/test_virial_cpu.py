"""CPU: the oracle's pair virial W = sum over pairs of r_ij . F_ij.

The reference computes no virial on its hot path (its only one,
src/misc.c:66-82, is static, never called, and sums x . F, which is wrong
under periodic images), so no golden vector pins W.  The restatement
(oracle/fmd_oracle.c, pair_update) is pinned instead by two independent
checks on the reference's own golden states:
  * LJ and Morse: a brute-force numpy sum over minimum-image pairs within
    the cutoff with the reference's pair formulas (src/lj.h:35-56,
    src/morse.h:35-56);
  * every potential, EAM included: U depends on pair distances only, so
    W = -dU/d(ln s) for a uniform scaling s of positions and box; central
    finite differences of the oracle's energy (h = 1e-6) agree to 1e-7.
"""
import os
import sys
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import pyoracle  # noqa: E402
from fmd_gb300 import workloads  # noqa: E402

CASES = {
    "lj_small": ((21.04,) * 3, (1, 1, 1), [("Ar", 39.948)], [("lj", 0, 0, 3.405, 0.0104, 8.5125)]),
    "morse_open": ((21.69, 21.69, 40.0), (1, 1, 0), [("Cu", 63.546)], [("morse", 0, 0, 0.3429, 1.3588, 2.866, 8.0)]),
    "eam": ((28.92,) * 3, (1, 1, 1), [("Cu", 63.546)], [("eam", 0, 0)]),
}


def _oracle(name, setfl, s=1.0):
    box, pbc, kinds, pots = CASES[name]
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    n = len(g["s0_x"])
    o = pyoracle.Oracle()
    o.setup(np.asarray(box) * s, pbc, g["nc"], np.asarray(g["cellh"]) * s, kinds, pots, setfl)
    o.upload(g["s0_cell"], g["s0_x"] * s, np.zeros((n, 3)), np.zeros(n, np.uint32), np.zeros(n, np.int32),
             np.arange(n, dtype=np.uint32), int(np.prod(g["nc"])))
    o.forces(-1)
    d = o.dump()
    o.close()
    return d, g


def _brute_force(name, x):
    box, pbc, _, pots = CASES[name]
    p = pots[0]
    l = np.asarray(box)
    W = 0.0
    for i in range(len(x) - 1):
        rv = x[i] - x[i + 1:]
        for d in range(3):
            if pbc[d]:
                rv[:, d] -= l[d] * np.round(rv[:, d] / l[d])
        r2 = (rv * rv).sum(1)
        if p[0] == "lj":
            sig, eps, rc = p[3], p[4], p[5]
            r2 = r2[r2 < rc * rc]
            s6 = (sig * sig / r2) ** 3
            W += (12.0 * 4.0 * eps * (s6 * s6 - 0.5 * s6)).sum()        # r . F = f r^2
        else:
            D0, al, r0, rc = p[3], p[4], p[5], p[6]
            r = np.sqrt(r2[r2 < rc * rc])
            e1 = np.exp(-al * (r - r0))
            W += (2.0 * al * D0 * (e1 * e1 - e1) * r).sum()
    return W


@pytest.mark.parametrize("name", ["lj_small", "morse_open"])
def test_virial_brute_force(name):
    d, g = _oracle(name, None)
    W = _brute_force(name, np.asarray(g["s0_x"]))
    assert abs(d["virial"] - W) <= 1e-11 * max(abs(W), abs(d["pe"])), (d["virial"], W)


@pytest.mark.parametrize("name", ["lj_small", "morse_open", "eam"])
def test_virial_is_scaling_derivative(name):
    h = 1e-6
    with tempfile.TemporaryDirectory() as work:
        setfl = workloads.write_analytic_eam(os.path.join(work, "a.eam.alloy")) if name == "eam" else None
        d, _ = _oracle(name, setfl)
        up, _ = _oracle(name, setfl, 1.0 + h)
        dn, _ = _oracle(name, setfl, 1.0 - h)
    fd = -(up["pe"] - dn["pe"]) / (2.0 * h)
    assert abs(d["virial"] - fd) <= 1e-7 * max(abs(fd), abs(d["pe"])), (d["virial"], fd)
