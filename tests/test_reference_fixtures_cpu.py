"""CPU: the reference's own example data files (examples/data, recorded in
the golden .npz of the cases that use them, so no reference checkout is
needed) through libfmd.so's host set-up:

  * the Mishin copper setfl Cu01.eam.alloy: fmd_pot_eam_getLatticeParameter
    returns the 3.615 A of the file's header (src/eam.c:604-619), the
    known answer the fixture carries;
  * the r^2-grid spline tables libfmd builds from it (src/eam.c:376-555,
    restated in fmd_pot.c) are bit-identical to the oracle's, which is pinned
    to the reference's own forces on this potential
    (test_oracle_cpu.py::test_oracle_matches_reference[eam_cu01]).
No GPU call is made: the set-up is host code.
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np
import pytest

import cases

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import pyoracle  # noqa: E402


def _setfl(work):
    g = dict(np.load(os.path.join(HERE, "golden", "eam_cu01.npz")))
    cases.write_data(work, cases.golden_data(g))
    return os.path.join(work, "Cu01.eam.alloy")


def test_cu01_lattice_parameter(lib):
    with tempfile.TemporaryDirectory() as work:
        path = _setfl(work)
        md = C.c_void_p(lib.fmd_create())
        lib.L.fmd_pot_eam_alloy_load.restype = C.c_void_p
        lib.L.fmd_pot_eam_alloy_load.argtypes = [C.c_void_p, C.c_char_p]
        pot = lib.L.fmd_pot_eam_alloy_load(md, path.encode())
        assert pot
        f = lib.L.fmd_pot_eam_getLatticeParameter
        f.restype = C.c_double
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p]
        assert f(md, C.c_void_p(pot), b"Cu") == 3.615
        lib.fmd_free(md)


def test_cu01_tables_match_oracle(lib):
    from fmd_gb300 import serve
    L = serve.bind(lib)
    with tempfile.TemporaryDirectory() as work:
        path = _setfl(work)
        md = L.fmd_create()
        pot = L.fmd_pot_eam_alloy_load(md, path.encode())
        assert pot
        ne, nrho, nr2 = C.c_int(), C.c_int(), C.c_int()
        drho, dr2, rc2 = C.c_double(), C.c_double(), C.c_double()
        L.fmdx_eam_tables(pot, C.byref(ne), C.byref(nrho), C.byref(drho), C.byref(nr2), C.byref(dr2),
                          C.byref(rc2), None, None, None, None, None, None)
        assert ne.value == 1
        tabs = [np.zeros(nrho.value), np.zeros(nrho.value)] + [np.zeros(nr2.value) for _ in range(4)]
        ptr = [t.ctypes.data_as(C.POINTER(C.c_double)) for t in tabs]
        L.fmdx_eam_tables(pot, C.byref(ne), C.byref(nrho), C.byref(drho), C.byref(nr2), C.byref(dr2),
                          C.byref(rc2), *ptr)
        L.fmd_free(md)
        o = pyoracle.Oracle()
        names = C.create_string_buffer(256)
        cut = C.c_double()
        assert o.L.oracle_load_setfl(o.o, path.encode(), names, 256, C.byref(cut)) == 1
        assert names.value.decode().split() == ["Cu"]
        assert cut.value * cut.value == rc2.value
        for which, mine in enumerate(tabs):
            n = C.c_int()
            o.L.oracle_eam_table(o.o, 0, which, None, C.byref(n))
            assert n.value == len(mine), which
            theirs = np.zeros(n.value)
            o.L.oracle_eam_table(o.o, 0, which, theirs.ctypes.data_as(C.c_void_p), None)
            # phi[0] is FLT_MAX in both (src/eam.c:460-477)
            np.testing.assert_array_equal(mine, theirs, err_msg=str(which))
        o.close()


@pytest.mark.parametrize("name", ["ttm2", "ttm2_cu"])
def test_ttm_tables_match_reference(name):
    """Host-side TTM set-up without a device (fmd_create, the turi, the
    fmd_ttm_set* calls): the type-2 tables of libfmd (read from the same
    files, converted, spline-prepared) against the reference's, and the
    unit conversions and laser constants that do not depend on the atoms."""
    import ctypes as C
    import tempfile

    import cases
    from fmd_gb300 import api, load
    lib = load()
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name + ".npz")))
    case = cases.CASES[name]
    with tempfile.TemporaryDirectory() as work:
        cases.write_data(work, cases.golden_data(g))
        md = C.c_void_p(lib.fmd_create())
        lib.fmd_io_setShowErrorMessages(md, False)
        lib.fmd_box_setSubdomains(md, 1, 1, 1)
        lib.fmd_box_setSize(md, *case["box"])
        lib.fmd_box_setPBC(md, *[bool(b) for b in case["pbc"]])
        api.set_atom_kinds(lib, md, case["names"], [cases.MASS[n] for n in case["names"]])
        cases.setup_turi(lib, md, dict(case["turi"]), work)
        lib.L.fmdx_ttm_params.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        pd = np.zeros(17)
        pk = np.zeros(9, np.int32)
        tabs = (C.c_void_p * 6)()
        assert lib.L.fmdx_ttm_params(md, pd.ctypes.data, pk.ctypes.data, tabs) == 0
        tables = {}
        for w, key in enumerate(("T_C", "Ct", "C_DD", "T_G", "Gt", "G_DD")):
            n = int(pk[3] if w < 3 else pk[4])
            tables[key] = np.ctypeslib.as_array(C.cast(tabs[w], C.POINTER(C.c_double)), shape=(n,)).copy()
        lib.fmd_free(md)
    cases.check_ttm_tables(tables, g)
    # Zhigilei constants, dz2, laser constants, cell volume, window, tcellh
    same = [3, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16]
    np.testing.assert_array_equal(pd[same], g["ttm_pd"][same])
    np.testing.assert_array_equal(pk[[0, 1, 3, 4, 5, 6, 7, 8]], g["ttm_pk"][[0, 1, 3, 4, 5, 6, 7, 8]])
