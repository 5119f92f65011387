"""GPU parity against the CPU oracle (oracle/fmd_oracle.c, pinned to the
reference's golden vectors by tests/test_oracle_cpu.py) at sizes beyond the
golden fixtures, and size-independent checks at the full benchmark size.

binary64 tolerances: forces <= 1e-10 of max |F|, energies <= 1e-10
relative, pair virial <= 1e-10 of max(|W|, |PE|), positions after 30
steps <= 1e-9 A, cell order exact.
mixed mode: forces <= 1e-5 of max |F|, energy <= 1e-6 relative, pair
virial <= 1e-5 of max(|W|, |PE|).
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np
import pytest

import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle  # noqa: E402
from fmd_gb300 import api, workloads  # noqa: E402

pytestmark = pytest.mark.gpu


def _lj32k():
    x, v = workloads.fcc_state(20, 20, 20, 5.26, 100.0, 39.948, seed=31, disp=0.05)
    return dict(box=(105.2,) * 3, pbc=(1, 1, 1), kinds=[("Ar", 39.948)],
                pots=[("lj", 0, 0, 3.405, 0.0104, 8.5125)], x=x, v=v, kind=np.zeros(len(x), np.uint32),
                group=np.zeros(len(x), np.int32), dt=0.002)


def _eam16k():
    x, v = workloads.fcc_state(16, 16, 16, 3.615, 300.0, 63.546, seed=32, disp=0.04)
    return dict(box=(57.84,) * 3, pbc=(1, 1, 1), kinds=[("Cu", 63.546)], pots=[("eam", 0, 0)],
                x=x, v=v, kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), dt=0.001)


def _morse_slab():
    rng = np.random.default_rng(33)
    x, v = workloads.fcc_state(12, 12, 6, 3.615, 300.0, 63.546, seed=33, origin=(0.0, 0.0, 12.0), disp=0.03)
    px = workloads.fcc_sites(2, 2, 2, 3.615, origin=(18.0, 18.0, 40.0))
    pv = np.tile([0.0, 0.0, -45.0], (len(px), 1)) + rng.standard_normal((len(px), 3))
    ex = np.array([[5.0, 5.0, 59.8], [30.0, 20.0, 0.1]])
    ev = np.array([[0.0, 0.0, 40.0], [0.0, 0.0, -40.0]])
    x = np.concatenate([x, px, ex])
    v = np.concatenate([v, pv, ev])
    return dict(box=(43.38, 43.38, 60.0), pbc=(1, 1, 0), kinds=[("Cu", 63.546)],
                pots=[("morse", 0, 0, 0.3429, 1.3588, 2.866, 8.0)], x=x, v=v,
                kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), dt=0.001)


def _hybrid():
    xc, vc = workloads.fcc_state(6, 6, 6, 3.615, 300.0, 63.546, seed=34, origin=(3.0, 10.0, 10.0), disp=0.03)
    xa, va = workloads.fcc_state(4, 4, 4, 5.26, 60.0, 39.948, seed=35, origin=(30.0, 10.0, 10.0), disp=0.03)
    va[:, 0] -= 6.0
    return dict(box=(56.0, 42.0, 42.0), pbc=(1, 1, 1), kinds=[("Cu", 63.546), ("Ar", 39.948)],
                pots=[("eam", 0, 0), ("lj", 1, 1, 3.4, 0.0104, 8.5), ("lj", 0, 1, 2.87, 0.0652, 7.175)],
                x=np.concatenate([xc, xa]), v=np.concatenate([vc, va]),
                kind=np.concatenate([np.zeros(len(xc), np.uint32), np.ones(len(xa), np.uint32)]),
                group=np.zeros(len(xc) + len(xa), np.int32), dt=0.001)


def _morse_nc2():
    """Smallest Morse cube of the served stream: l = 18.075 A, two cells per
    axis (each cell is its own upper and lower neighbour, with two images)."""
    x, v = workloads.fcc_state(5, 5, 5, 3.615, 600.0, 63.546, seed=36, disp=0.05)
    x = np.mod(x, 18.075)
    return dict(box=(18.075,) * 3, pbc=(1, 1, 1), kinds=[("Cu", 63.546)],
                pots=[("morse", 0, 0, 0.3429, 1.3588, 2.866, 8.0)], x=x, v=v,
                kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), dt=0.001)


SPECS = {"lj32k": _lj32k, "eam16k": _eam16k, "morse_slab": _morse_slab, "hybrid": _hybrid,
         "morse_nc2": _morse_nc2}


def build_both(lib, spec, work, precision=0):
    md = C.c_void_p(lib.fmd_create())
    lib.fmd_io_setShowErrorMessages(md, False)
    lib.fmd_box_setSubdomains(md, 1, 1, 1)
    lib.fmd_box_setSize(md, *spec["box"])
    lib.fmd_box_setPBC(md, *[bool(b) for b in spec["pbc"]])
    names = [k[0] for k in spec["kinds"]]
    api.set_atom_kinds(lib, md, names, [k[1] for k in spec["kinds"]])
    setfl = None
    for p in spec["pots"]:
        if p[0] == "lj":
            lib.fmd_pot_lj_apply(md, *p[1:])
        elif p[0] == "morse":
            lib.fmd_pot_morse_apply(md, *p[1:])
        else:
            setfl = os.path.join(work, "analytic.eam.alloy")
            if not os.path.exists(setfl):
                workloads.write_analytic_eam(setfl)
            pot = lib.fmd_pot_eam_alloy_load(md, setfl.encode())
            lib.fmd_pot_apply(md, p[1], p[2], pot)
    spath = os.path.join(work, "state.stt")
    api.write_state(spath, 0.0, spec["box"], spec["pbc"], names, spec["kind"], spec["group"], spec["x"], spec["v"])
    lib.fmd_io_loadState(md, spath.encode(), False)
    lib.L.fmdx_set_precision.argtypes = [C.c_void_p, C.c_int]
    lib.L.fmdx_set_precision(md, precision)
    lib.L.fmdx_distribute.argtypes = [C.c_void_p]
    assert lib.L.fmdx_distribute(md) == 0
    d = lib.dump(md)
    nc, cellh, _, _ = lib.grid(md)
    o = pyoracle.Oracle()
    o.setup(spec["box"], spec["pbc"], nc, cellh, spec["kinds"], spec["pots"], setfl)
    o.upload(d["cell"], d["x"], d["v"], d["kind"], d["group"], d["id"], int(np.prod(nc)))
    return md, o


@pytest.mark.parametrize("name", list(SPECS))
def test_gpu_vs_oracle_fp64(gpu_lib, name):
    spec = SPECS[name]()
    with tempfile.TemporaryDirectory() as work:
        md, o = build_both(gpu_lib, spec, work)
        dt = spec["dt"]
        gpu_lib.fmd_dync_integrate(md, -1, 0.0, dt)
        g0 = gpu_lib.dump(md)
        o.forces(-1)
        r0 = o.dump()
        np.testing.assert_array_equal(g0["id"], r0["id"])
        fmax = np.abs(r0["F"]).max()
        assert np.abs(g0["F"] - r0["F"]).max() <= 1e-10 * fmax
        assert abs(g0["pe"] - r0["pe"]) <= 1e-10 * abs(r0["pe"])
        # pair virial (relative to the larger of |W| and |PE|: W of a
        # near-equilibrium crystal can be small)
        assert abs(g0["virial"] - r0["virial"]) <= 1e-10 * max(abs(r0["virial"]), abs(r0["pe"]))
        nsteps = 30
        gpu_lib.fmd_dync_integrate(md, -1, (nsteps - 0.5) * dt, dt)
        g1 = gpu_lib.dump(md)
        o.vv(nsteps, dt)
        r1 = o.dump()
        assert len(g1["id"]) == len(r1["id"])
        np.testing.assert_array_equal(g1["cell"], r1["cell"])
        np.testing.assert_array_equal(g1["id"], r1["id"])
        assert np.abs(g1["x"] - r1["x"]).max() <= 1e-9
        assert np.abs(g1["v"] - r1["v"]).max() <= 1e-9
        gpu_lib.fmd_free(md)
        o.close()


@pytest.mark.parametrize("name", list(SPECS))
def test_gpu_vs_oracle_mixed(gpu_lib, name):
    spec = SPECS[name]()
    with tempfile.TemporaryDirectory() as work:
        md, o = build_both(gpu_lib, spec, work, precision=1)
        gpu_lib.fmd_dync_integrate(md, -1, 0.0, spec["dt"])
        g0 = gpu_lib.dump(md)
        o.forces(-1)
        r0 = o.dump()
        err = np.abs(g0["F"] - r0["F"]).max() / np.abs(r0["F"]).max()
        assert err <= 1e-5, err
        assert abs(g0["pe"] - r0["pe"]) <= 1e-6 * abs(r0["pe"])
        # the virial sums pair terms f r^2 that cancel like the forces do:
        # the force bound, relative to max(|W|, |PE|)
        assert abs(g0["virial"] - r0["virial"]) <= 1e-5 * max(abs(r0["virial"]), abs(r0["pe"]))
        gpu_lib.fmd_free(md)
        o.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_full_size_invariants(gpu_lib, precision):
    """256000-atom EAM benchmark system, 40 steps: every atom kept exactly
    once, every atom in the cell its position selects (floor(x/cellh)),
    total momentum conserved, total energy conserved to 1e-6 relative."""
    w = dict(cells=(40, 40, 40), a=3.615)
    with tempfile.TemporaryDirectory() as work:
        lib = gpu_lib
        md = C.c_void_p(lib.fmd_create())
        lib.fmd_box_setSubdomains(md, 1, 1, 1)
        lib.fmd_box_setSize(md, *[c * w["a"] for c in w["cells"]])
        lib.fmd_box_setPBC(md, True, True, True)
        api.set_atom_kinds(lib, md, ["Cu"], [63.546])
        setfl = workloads.write_analytic_eam(os.path.join(work, "a.eam.alloy"))
        pot = lib.fmd_pot_eam_alloy_load(md, setfl.encode())
        lib.fmd_pot_apply(md, 0, 0, pot)
        lib.L.fmdx_set_seed.argtypes = [C.c_void_p, C.c_ulonglong]
        lib.L.fmdx_set_seed(md, 2)
        lib.L.fmdx_set_precision.argtypes = [C.c_void_p, C.c_int]
        lib.L.fmdx_set_precision(md, precision)
        lib.fmd_matt_makeCuboidFCC(md, 0.0, 0.0, 0.0, *w["cells"], w["a"], 0, 0, 300.0)
        lib.fmd_dync_integrate(md, -1, 0.0, 0.001)
        e0 = lib.fmd_matt_getTotalEnergy(md)
        p = (C.c_double * 3)()
        lib.fmd_dync_integrate(md, -1, 0.0395, 0.001)
        e1 = lib.fmd_matt_getTotalEnergy(md)
        lib.fmd_matt_getMomentum(md, p)
        d = lib.dump(md)
        nc, cellh, l, _ = lib.grid(md)
        lib.fmd_free(md)
    n = 4 * 40 ** 3
    assert len(d["id"]) == n
    assert np.array_equal(np.sort(d["id"]), np.arange(n, dtype=np.uint32))
    ic = np.floor(d["x"] / cellh).astype(np.int64)
    flat = ic[:, 2] + nc[2] * (ic[:, 1] + nc[1] * ic[:, 0])
    assert np.array_equal(flat, d["cell"])
    assert np.all(np.diff(d["cell"]) >= 0)
    mv = np.abs(d["v"]).sum() * 63.546
    assert np.abs(np.array(p[:])).max() <= 1e-9 * mv
    assert abs(e1 - e0) <= 1e-6 * abs(e0), (e0, e1)
