"""GPU: the allocation-free pair-force entry point (fmdg_pair_forces_noalloc)
against the allocating engine (fmdg_compute_forces) on the same atoms.

It serves callers that cannot let a library call cudaMalloc (graph capture,
caller-owned memory pools, serving loops that must not synchronise), so the
test allocates every input and output itself (through torch) and calls the
entry point twice in a row -- an LJ system, then a Morse system with open
faces -- checking each result against the allocating path to the binary64
parity tolerance used throughout (1e-10 of max |F|, 1e-10 relative energy).
This file is collected last so a failure here does not hide other results.
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
                ("potential", C.c_double), ("count", C.c_double), ("pad", C.c_double)]


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


def _allocating(L, g, pair, box, pbc, mass):
    s = C.c_void_p()
    assert L.fmdg_create(C.byref(s), 0) == 0
    nc = np.ascontiguousarray(g["nc"], np.int32)
    cellh = np.ascontiguousarray(g["cellh"], np.float64)
    l = np.array(box, np.float64)
    pb = np.array(pbc, np.int32)
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    assert L.fmdg_set_box(s, P(l), P(pb), P(nc), P(cellh)) == 0
    m = np.array([mass / 9.6485332907e+03])
    assert L.fmdg_set_kinds(s, 1, P(m), None) == 0
    assert L.fmdg_set_pairs(s, C.byref(pair)) == 0
    n = len(g["s0_id"])
    counts = np.bincount(g["s0_cell"], minlength=int(np.prod(nc))).astype(np.int32)
    x = np.ascontiguousarray(g["s0_x"])
    v = np.zeros_like(x)
    kind = np.zeros(n, np.uint32)
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


def test_noalloc_matches_allocating(gpu_lib):
    torch = pytest.importorskip("torch")
    L = gpu_lib.L
    L.fmdg_pair_forces_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]
    L.fmdg_last_error.restype = C.c_char_p
    dev = torch.device("cuda:0")
    for name in ("lj", "morse_open"):
        g, pair, box, pbc, mass = _case(name)
        F_ref, pe_ref, counts = _allocating(L, g, pair, box, pbc, mass)
        n = len(g["s0_id"])
        cell_start = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
        x_d = torch.tensor(np.ascontiguousarray(g["s0_x"].T), dtype=torch.float64, device=dev)
        kind_d = torch.zeros(n, dtype=torch.int32, device=dev)
        cs_d = torch.tensor(cell_start, device=dev)
        co_d = torch.tensor(g["s0_cell"].astype(np.int32), device=dev)
        F_d = torch.full((3, n), float("nan"), dtype=torch.float64, device=dev)
        pe_d = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        nc = np.ascontiguousarray(g["nc"], np.int32)
        l = np.array(box, np.float64)
        pb = np.array(pbc, np.int32)
        P = lambda a: a.ctypes.data_as(C.c_void_p)
        stream = torch.cuda.current_stream(dev).cuda_stream
        rc = L.fmdg_pair_forces_noalloc(n, P(nc), P(pb), P(l), 1, C.byref(pair), x_d.data_ptr(),
                                        kind_d.data_ptr(), cs_d.data_ptr(), co_d.data_ptr(), F_d.data_ptr(),
                                        pe_d.data_ptr(), C.c_void_p(stream))
        assert rc == 0, L.fmdg_last_error()
        torch.cuda.synchronize(dev)
        F = F_d.cpu().numpy().T
        pe = float(pe_d.cpu()[0])
        fmax = np.abs(F_ref).max()
        assert np.abs(F - F_ref).max() <= TOL * fmax, name
        assert abs(pe - pe_ref) <= TOL * abs(pe_ref), (name, pe, pe_ref)


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
