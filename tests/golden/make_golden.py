"""Generate the golden vectors in tests/golden/ from the reference FMD library.

Run from the repository root in a container that has the reference sources:

    make -f oracle/Makefile.ref REF=/root/reference
    python tests/golden/make_golden.py

The reference is compiled unmodified as a single-rank CPU library
(oracle/_ref/libfmdref.so) and driven through its own fmd.h API with the
cases of tests/cases.py; white-box dumps come from oracle/ref_probe.c.
Outputs: tests/golden/<case>.npz and tests/golden/bin_<case>.npz.  Cases
that load the reference's example data files (examples/data: the Mishin
copper setfl, the type-2 TTM tables) record those files' bytes in their .npz
(keys data:<file name>), so the tests run without a reference checkout.
The full-size cases of cases.FULL_CASES (minutes of single-threaded
reference time each) are generated by name only:

    python tests/golden/make_golden.py ttm_slab_full
    python tests/golden/make_golden.py eam256k_full
    python tests/golden/make_golden.py morse_collision_full
"""
from __future__ import annotations

import ctypes as C
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from fmd_gb300 import api  # noqa: E402
import cases  # noqa: E402

REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libfmdref.so")
# the reference's example data files (examples/data), read from its checkout
REF_DATA = os.path.join(os.environ.get("FMD_REFERENCE", "/root/reference"), "examples", "data")


def ttm_params(lib, md):
    """The reference's derived parameters of the active 1-D TTM turi
    (oracle/ref_probe.c oref_ttm_params, oref_ttm_table) for the oracle's
    TTM restatement: ttm_pd (17 doubles), ttm_pk (9 ints), type-2 tables."""
    d = np.zeros(17)
    k = np.zeros(9, np.int32)
    if lib.L.oref_ttm_params(C.c_void_p(md.value), d.ctypes.data_as(C.c_void_p), k.ctypes.data_as(C.c_void_p)) != 0:
        return {}
    out = dict(ttm_pd=d, ttm_pk=k)
    if k[0] == 2:
        for w, key in enumerate(("T_C", "Ct", "C_DD", "T_G", "Gt", "G_DD")):
            buf = np.zeros(int(k[3] if w < 3 else k[4]))
            lib.L.oref_ttm_table(C.c_void_p(md.value), w, buf.ctypes.data_as(C.c_void_p))
            out["ttm_tab_" + key] = buf
    return out


def golden_case(lib, name, work):
    case = cases.CASES[name]
    data = {f: open(os.path.join(REF_DATA, f), "rb").read() for f in case.get("data", ())}
    md, st = cases.setup(lib, name, work, data=data)
    grp, dt = case["run"][1], case["run"][2]
    rec = cases.Recorder(lib)
    if "turi" in case:
        rec.record_fields(md, case["turi"]["_handle"])
        lib.fmd_setEventHandler(md, None, rec.cb)
    lib.fmd_dync_integrate(md, grp, 0.0, dt)
    d0 = lib.dump(md)
    nc, cellh, l, pbc = lib.grid(md)
    cases.run(lib, name, md, rec)
    d1 = lib.dump(md)
    out = dict(state_x=st["x"], state_v=st["v"], state_kind=st["kind"], state_group=st["group"],
               nc=nc, cellh=cellh,
               s0_cell=d0["cell"], s0_id=d0["id"], s0_x=d0["x"], s0_F=d0["F"], s0_vaream=d0["vaream"],
               s0_pe=np.array(d0["pe"]),
               s1_cell=d1["cell"], s1_id=d1["id"], s1_x=d1["x"], s1_v=d1["v"], s1_F=d1["F"],
               s1_pe=np.array(d1["pe"]), thermo=np.array(rec.rows),
               errors=np.array(rec.errors, dtype=np.int64).reshape(-1, 2),
               time_iteration=np.array(lib.wb("time_iteration")(md) if lib.has("oref_time_iteration") else -1))
    for f, raw in data.items():       # recorded so the tests need no reference checkout
        out["data:" + f] = np.frombuffer(raw, dtype=np.uint8)
    if "turi" in case:
        ev = [(t, tu, f) for (t, tu, f, _) in rec.fields]
        out["field_events"] = np.array(ev, dtype=np.float64).reshape(-1, 3)
        for k, (t, tu, f, vals) in enumerate(rec.fields):
            if vals is not None:
                out["field_%03d" % k] = vals
        ttm = lib.ttm_1d(md)
        if ttm is not None:
            for kk, vv in ttm.items():
                out["ttm_" + kk] = vv
            out.update(ttm_params(lib, md))
    lib.fmd_free(md)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "N0", len(d0["id"]), "N1", len(d1["id"]), "PE0", d0["pe"], "rows", len(rec.rows),
          "errors", rec.errors)


def golden_full(lib, name, work):
    """A full-size case (cases.FULL_CASES): the initial state is regenerated
    from its seed by the test, so only the observables are kept -- the
    thermo series, the potential energy before and after, the final state
    of the atoms with the lowest ids, every field-update event with its
    array, the final TTM state and the atom count."""
    case = cases.FULL_CASES[name]
    md, st = cases.setup(lib, name, work)
    rec = cases.Recorder(lib)
    if "turi" in case:
        rec.record_fields(md, case["turi"]["_handle"])
        lib.fmd_setEventHandler(md, None, rec.cb)
    lib.fmd_dync_integrate(md, case["run"][1], 0.0, case["run"][2])
    pe0 = lib.dump(md)["pe"]
    cases.run(lib, name, md, rec)
    d1 = lib.dump(md)
    out = dict(n0=np.array(len(st["x"])), n1=np.array(len(d1["id"])), thermo=np.array(rec.rows),
               s0_pe=np.array(pe0), s1_pe=np.array(d1["pe"]),
               errors=np.array(rec.errors, dtype=np.int64).reshape(-1, 2))
    if "sample" in case:
        order = np.argsort(d1["id"])
        if case.get("spread"):      # ids spread over the whole range
            sel = order[np.unique(np.linspace(0, len(order) - 1, case["sample"]).astype(np.int64))]
        else:                       # the lowest ids
            sel = order[:case["sample"]]
        out.update(sample_id=d1["id"][sel], sample_x=d1["x"][sel], sample_v=d1["v"][sel], sample_F=d1["F"][sel],
                   F_absmax=np.array(np.abs(d1["F"]).max()))
    if "turi" in case:
        ev = [(t, tu, f) for (t, tu, f, _) in rec.fields]
        out["field_events"] = np.array(ev, dtype=np.float64).reshape(-1, 3)
        for k, (t, tu, f, vals) in enumerate(rec.fields):
            if vals is not None:
                out["field_%03d" % k] = vals
        for kk, vv in lib.ttm_1d(md).items():
            out["ttm_" + kk] = vv
        out.update(ttm_params(lib, md))
    lib.fmd_free(md)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, "N", out["n0"], out["n1"], "rows", len(rec.rows), "errors", rec.errors)


def golden_binning(lib, name, work, rounds=4, seed=99):
    """Displace atoms (some across cell and periodic faces) and let the
    reference re-bin them; records the cell and in-cell order after each
    round (src/misc.c:268-308, src/md-ghost.c:827-869)."""
    case = cases.CASES[name]
    md, st = cases.setup(lib, name, work)
    lib.fmd_dync_integrate(md, case["run"][1], 0.0, case["run"][2])
    nc, cellh, l, pbc = lib.grid(md)
    rng = np.random.default_rng(seed)
    recs = {}
    d = lib.dump(md)
    recs["r0_cell"], recs["r0_id"], recs["r0_x"] = d["cell"], d["id"], d["x"]
    for r in range(1, rounds + 1):
        x = d["x"].copy()
        n = len(x)
        disp = rng.standard_normal((n, 3)) * 0.2 * cellh
        big = rng.random(n) < 0.15
        disp[big] = rng.uniform(-0.97, 0.97, (big.sum(), 3)) * cellh
        disp = np.clip(disp, -0.97 * cellh, 0.97 * cellh)
        x += disp
        recs["in%d_x" % r] = x
        lib.set_state(md, x, None)
        lib.wb("refresh")(md)
        d = lib.dump(md)
        recs["r%d_cell" % r], recs["r%d_id" % r], recs["r%d_x" % r] = d["cell"], d["id"], d["x"]
        print("bin", name, "round", r, "N", len(d["id"]))
    lib.fmd_free(md)
    np.savez_compressed(os.path.join(HERE, "bin_" + name + ".npz"), nc=nc, cellh=cellh, rounds=rounds, **recs)


IO_MODES = [("xyz", 1), ("csv", 2), ("vtf", 3)]


def io_files(lib, md, work, tag):
    """Files the reference writes for the current state: fmd_io_saveState
    (src/misc.c:310-422) and fmd_matt_saveConfiguration in every mode
    (src/matter.c:650-829), read back as bytes."""
    out = {}
    lib.fmd_io_setSaveDirectory(md, (work + "/").encode())
    lib.fmd_io_saveState(md, (tag + ".stt").encode())
    out[tag + "_state"] = open(os.path.join(work, tag + ".stt"), "rb").read()
    for name, mode in IO_MODES:
        before = set(os.listdir(work))
        lib.fmd_io_setSaveConfigMode(md, mode)
        lib.fmd_matt_saveConfiguration(md)
        new = sorted(set(os.listdir(work)) - before)
        assert len(new) == 1, (name, new)
        out[tag + "_" + name] = open(os.path.join(work, new[0]), "rb").read()
        os.remove(os.path.join(work, new[0]))
    return out


def golden_io(lib, name, work):
    """State and configuration files of case `name` right after distribution
    and after the case's run."""
    case = cases.CASES[name]
    md, st = cases.setup(lib, name, work)
    lib.fmd_dync_integrate(md, case["run"][1], 0.0, case["run"][2])
    files = io_files(lib, md, work, "s0")
    cases.run(lib, name, md, None)
    files.update(io_files(lib, md, work, "s1"))
    lib.fmd_free(md)
    np.savez_compressed(os.path.join(HERE, "io_" + name + ".npz"),
                        **{k: np.frombuffer(v, dtype=np.uint8) for k, v in files.items()})
    print("io", name, {k: len(v) for k, v in files.items()})


ARGON_C = os.path.join(os.path.dirname(HERE), "c", "argon_relink.c")
ARGON_C_DURATION = 0.4


def argon_c_state(path):
    """The seeded initial state of the C relink program (FCC argon 10^3
    cells, 100 K)."""
    from fmd_gb300 import workloads
    x, v = workloads.fcc_state(10, 10, 10, 5.26, 100.0, 39.948, seed=61, disp=0.05)
    n = len(x)
    api.write_state(path, 0.0, (52.6,) * 3, (1, 1, 1), ["Ar"], np.zeros(n, np.uint32), np.zeros(n, np.int32), x, v)


def golden_argon_c(work):
    """tests/c/argon_relink.c compiled unchanged against the reference's own
    fmd.h and linked with the reference library: its printed series and the
    files it writes."""
    import subprocess
    ref_inc = os.path.join(os.environ.get("FMD_REFERENCE", "/root/reference"), "src")
    exe = os.path.join(work, "argon_ref.x")
    subprocess.run(["gcc", "-std=c11", "-O2", "-Werror=implicit-function-declaration", ARGON_C, "-I" + ref_inc,
                    REF_LIB, "-Wl,-rpath," + os.path.dirname(REF_LIB), "-o", exe], check=True)
    st = os.path.join(work, "state0.stt")
    argon_c_state(st)
    out = os.path.join(work, "out") + "/"
    os.makedirs(out)
    r = subprocess.run([exe, st, out, repr(ARGON_C_DURATION)], check=True, capture_output=True, text=True)
    files = {f: open(os.path.join(out, f), "rb").read() for f in sorted(os.listdir(out))}
    rec = {"stdout": np.frombuffer(r.stdout.encode(), np.uint8),
           "state0": np.frombuffer(open(st, "rb").read(), np.uint8),
           "files": np.array(sorted(files))}
    for f, raw in files.items():
        rec["file:" + f] = np.frombuffer(raw, np.uint8)
    np.savez_compressed(os.path.join(HERE, "argon_c.npz"), **rec)
    print("argon_c", r.stdout.count("tick"), "ticks", sorted(files))


def main():
    names = sys.argv[1:] or list(cases.CASES)
    if len(names) > 1 or not sys.argv[1:]:
        # one process per case: the reference's fmd_free reads the instance
        # after freeing it (src/misc.c:650-660), so instances are not reused
        import subprocess
        for name in names + ([] if sys.argv[1:] else ["bin_lj", "bin_morse_open", "io_lj_small", "io_hybrid",
                                                        "argon_c"]):
            subprocess.run([sys.executable, os.path.abspath(__file__), name], check=True)
        return
    lib = api.Lib(REF_LIB, prefix="oref_")
    with tempfile.TemporaryDirectory() as work:
        for name in names:
            if name == "argon_c":
                golden_argon_c(work)
            elif name in cases.FULL_CASES:
                golden_full(lib, name, work)
            elif name.startswith("bin_"):
                golden_binning(lib, name[4:], work)
            elif name.startswith("io_"):
                golden_io(lib, name[3:], work)
            else:
                golden_case(lib, name, work)



if __name__ == "__main__":
    main()
