"""GPU: the allocation-free pair-force entry point (fmdg_pair_forces_noalloc)
against the allocating engine (fmdg_compute_forces) on the same atoms.

It serves callers that cannot let a library call cudaMalloc (graph capture,
caller-owned memory pools, serving loops that must not synchronise), so the
test allocates every input and output itself (through torch) and calls the
entry point twice in a row -- an LJ system, then a Morse system with open
faces -- checking each result against the allocating path and against the
reference's own step-0 forces (golden vectors) to the binary64 parity
tolerance used throughout (1e-10 of max |F|, 1e-10 relative energy).  A
two-kind LJ mixture is checked against the CPU oracle, and an atom kind
outside the pair table comes back as NaN forces.  This file is collected
last so a failure here does not hide other results.
"""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-10


class Pair(C.Structure):
    _fields_ = [("cat", C.c_int), ("iloc", C.c_int), ("jloc", C.c_int), ("pad", C.c_int), ("p", C.c_double * 4)]


class Thermo(C.Structure):
    _fields_ = [("kinetic", C.c_double), ("temperature", C.c_double), ("momentum", C.c_double * 3),
                ("potential", C.c_double), ("count", C.c_double), ("virial", C.c_double)]


def _case(name):
    g = dict(np.load(os.path.join(HERE, "golden", name + ".npz")))
    if name == "lj":
        pair = Pair(cat=1)
        pair.p[0], pair.p[1], pair.p[2] = 4 * 0.0104, 3.405 ** 2, 8.5125 ** 2
        box, pbc, mass = (52.6, 52.6, 52.6), (1, 1, 1), 39.948
    else:
        pair = Pair(cat=3)
        pair.p[0], pair.p[1], pair.p[2], pair.p[3] = 0.3429, 1.3588, 2.866, 8.0 ** 2
        box, pbc, mass = (21.69, 21.69, 40.0), (1, 1, 0), 63.546
    return g, pair, box, pbc, mass


def _allocating(L, g, pair, box, pbc, mass, kind=None):
    s = C.c_void_p()
    assert L.fmdg_create(C.byref(s), 0) == 0
    nc = np.ascontiguousarray(g["nc"], np.int32)
    cellh = np.ascontiguousarray(g["cellh"], np.float64)
    l = np.array(box, np.float64)
    pb = np.array(pbc, np.int32)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    assert L.fmdg_set_box(s, P(l), P(pb), P(nc), P(cellh)) == 0
    masses = np.atleast_1d(np.asarray(mass, np.float64)) / 9.6485332907e+03
    assert L.fmdg_set_kinds(s, len(masses), P(masses), None) == 0
    assert L.fmdg_set_pairs(s, pair if isinstance(pair, C.Array) else C.byref(pair)) == 0
    n = len(g["s0_id"])
    counts = np.bincount(g["s0_cell"], minlength=int(np.prod(nc))).astype(np.int32)
    x = np.ascontiguousarray(g["s0_x"])
    v = np.zeros_like(x)
    kind = np.zeros(n, np.uint32) if kind is None else np.ascontiguousarray(kind, np.uint32)
    grp = np.zeros(n, np.int32)
    ids = np.ascontiguousarray(g["s0_id"], np.uint32)
    assert L.fmdg_upload(s, n, P(counts), P(x), P(v), P(kind), P(grp), P(ids)) == 0
    assert L.fmdg_compute_forces(s, -1) == 0
    F = np.zeros((n, 3))
    assert L.fmdg_download(s, None, None, None, P(F), None, None, None, None) == 0
    th = Thermo()
    assert L.fmdg_get_thermo(s, C.byref(th)) == 0
    L.fmdg_destroy(s)
    return F, th.potential, counts


def _bind(L):
    L.fmdg_pair_forces_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    L.fmdg_last_error.restype = C.c_char_p


def _noalloc(torch, L, g, pair, box, pbc, counts, nkinds=1, kind=None):
    """One call of the entry point on caller-owned device memory (torch)."""
    dev = torch.device("cuda:0")
    n = len(g["s0_id"])
    cell_start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    x_d = torch.tensor(np.ascontiguousarray(g["s0_x"].T), dtype=torch.float64, device=dev)
    kind_np = np.zeros(n, np.int32) if kind is None else np.asarray(kind, np.int32)
    kind_d = torch.tensor(kind_np, device=dev)
    cs_d = torch.tensor(cell_start, device=dev)
    co_d = torch.tensor(g["s0_cell"].astype(np.int32), device=dev)
    F_d = torch.full((3, n), float("nan"), dtype=torch.float64, device=dev)
    pe_d = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    nc = np.ascontiguousarray(g["nc"], np.int32)
    l = np.array(box, np.float64)
    pb = np.array(pbc, np.int32)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    stream = torch.cuda.current_stream(dev).cuda_stream
    pairs = pair if isinstance(pair, C.Array) else C.byref(pair)
    rc = L.fmdg_pair_forces_noalloc(n, P(nc), P(pb), P(l), nkinds, pairs, x_d.data_ptr(), kind_d.data_ptr(),
                                    cs_d.data_ptr(), co_d.data_ptr(), F_d.data_ptr(), pe_d.data_ptr(),
                                    C.c_void_p(stream))
    assert rc == 0, L.fmdg_last_error()
    torch.cuda.synchronize(dev)
    return F_d.cpu().numpy().T, float(pe_d.cpu()[0])


def test_noalloc_matches_allocating(gpu_lib):
    torch = pytest.importorskip("torch")
    L = gpu_lib.L
    _bind(L)
    for name in ("lj", "morse_open"):
        g, pair, box, pbc, mass = _case(name)
        F_ref, pe_ref, counts = _allocating(L, g, pair, box, pbc, mass)
        F, pe = _noalloc(torch, L, g, pair, box, pbc, counts)
        fmax = np.abs(F_ref).max()
        assert np.abs(F - F_ref).max() <= TOL * fmax, name
        assert abs(pe - pe_ref) <= TOL * abs(pe_ref), (name, pe, pe_ref)
        # the reference's own step-0 forces of the same atoms (same order)
        assert np.abs(F - g["s0_F"]).max() <= TOL * np.abs(g["s0_F"]).max(), name


def _two_kind_lj():
    """The golden LJ argon atoms as a two-kind mixture: kind = atom id % 2,
    three LJ pair types (one cutoff, so the cell grid is unchanged)."""
    rc = 8.5125
    params = {(0, 0): (3.405, 0.0104), (1, 1): (3.30, 0.0120), (0, 1): (3.35, 0.0112)}
    table = (Pair * 4)()
    for (a, b), (sig, eps) in params.items():
        for i, j in ((a, b), (b, a)):
            t = table[i * 2 + j]
            t.cat = 1
            t.p[0], t.p[1], t.p[2] = 4 * eps, sig * sig, rc * rc
    pots = [("lj", a, b, sig, eps, rc) for (a, b), (sig, eps) in params.items()]
    return table, pots


def test_noalloc_two_kinds_against_oracle(gpu_lib):
    torch = pytest.importorskip("torch")
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import pyoracle
    L = gpu_lib.L
    _bind(L)
    g, _, box, pbc, _ = _case("lj")
    kind = (np.asarray(g["s0_id"]) % 2).astype(np.uint32)
    table, pots = _two_kind_lj()
    F_ref, pe_ref, counts = _allocating(L, g, table, box, pbc, [39.948, 30.0], kind=kind)
    for _ in range(2):       # two calls in a row share the scratch array
        F, pe = _noalloc(torch, L, g, table, box, pbc, counts, nkinds=2, kind=kind)
        assert np.abs(F - F_ref).max() <= TOL * np.abs(F_ref).max()
        assert abs(pe - pe_ref) <= TOL * abs(pe_ref)
    o = pyoracle.Oracle(threads=4)
    nc = np.asarray(g["nc"], np.int32)
    o.setup(box, pbc, nc, np.asarray(g["cellh"]), [("Ar", 39.948), ("X", 30.0)], pots)
    n = len(kind)
    o.upload(g["s0_cell"], g["s0_x"], np.zeros((n, 3)), kind, np.zeros(n, np.int32), g["s0_id"], int(np.prod(nc)))
    o.forces(-1)
    d = o.dump()
    o.close()
    assert (d["id"] == g["s0_id"]).all()
    assert np.abs(F - d["F"]).max() <= TOL * np.abs(d["F"]).max()
    assert abs(pe - d["pe"]) <= TOL * abs(d["pe"])


def test_noalloc_kind_outside_table(gpu_lib):
    # the kernel's own check: no pair-table read, NaN forces for the atoms
    # that meet the bad kind, NaN energy
    torch = pytest.importorskip("torch")
    L = gpu_lib.L
    _bind(L)
    g, pair, box, pbc, mass = _case("lj")
    n = len(g["s0_id"])
    counts = np.bincount(g["s0_cell"], minlength=int(np.prod(g["nc"]))).astype(np.int32)
    kind = np.zeros(n, np.int32)
    kind[7] = 5
    F, pe = _noalloc(torch, L, g, pair, box, pbc, counts, kind=kind)
    assert np.isnan(F[7]).all() and np.isnan(pe)
    assert np.isfinite(F).all(axis=1).sum() > n // 2


def test_noalloc_rejects_oversize(gpu_lib):
    L = gpu_lib.L
    L.fmdg_pair_forces_noalloc.argtypes = [C.c_int] + [C.c_void_p] * 3 + [C.c_int] + [C.c_void_p] * 8
    L.fmdg_last_error.restype = C.c_char_p
    nc = np.array([1, 1, 1], np.int32)
    l = np.array([10.0, 10.0, 10.0])
    pair = Pair(cat=1)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    rc = L.fmdg_pair_forces_noalloc(2_000_000, P(nc), P(nc), P(l), 1, C.byref(pair), None, None, None, None,
                                    None, None, None)
    assert rc != 0
    assert b"limit" in L.fmdg_last_error()
