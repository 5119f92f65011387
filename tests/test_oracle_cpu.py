"""CPU: the restated oracle (oracle/fmd_oracle.c) reproduces the golden
vectors produced by the reference FMD library -- step-0 forces, energies,
EAM F'(rho), the thermodynamic series, final positions and the exact cell
order after refreshes.  This pins the oracle used by the GPU parity tests."""
import os
import sys
import tempfile

import numpy as np
import pytest

import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")

from fmd_gb300 import workloads  # noqa: E402
import pyoracle  # noqa: E402


def oracle_for_case(name, g, work, threads=1):
    case = cases.CASES[name]
    kinds = [(n, cases.MASS[n]) for n in case["names"]]
    pots = []
    setfl = None
    cases.write_data(work, cases.golden_data(g))
    for p in case["pots"]:
        if p[0] == "eam_analytic":
            setfl = os.path.join(work, "analytic.eam.alloy")
            if not os.path.exists(setfl):
                workloads.write_analytic_eam(setfl)
            pots.append(("eam", p[1], p[2]))
        elif p[0] == "eam_file":
            setfl = os.path.join(work, p[3])
            pots.append(("eam", p[1], p[2]))
        else:
            pots.append(p)
    o = pyoracle.Oracle(threads=threads)
    o.setup(case["box"], case["pbc"], g["nc"], g["cellh"], kinds, pots, setfl)
    ids = g["s0_id"]
    o.upload(g["s0_cell"], g["s0_x"], g["state_v"][ids], g["state_kind"][ids], g["state_group"][ids], ids,
             int(np.prod(g["nc"])))
    return o


def run_oracle_case(name, threads=1):
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    case = cases.CASES[name]
    r = case["run"]
    grp, dt = r[1], r[2]
    with tempfile.TemporaryDirectory() as work:
        o = oracle_for_case(name, g, work, threads)
    o.forces(grp)
    d0 = o.dump()
    thermostat = 1 if r[0] == "equilibrate" else 0
    tau, T0 = (r[3], r[4]) if thermostat else (1.0, 0.0)
    th = o.thermo(grp)
    rows = [(0.0, th.temperature, th.kinetic + th.potential, th.kinetic)]
    done = 0
    while done < case["steps"]:
        k = min(case["every"], case["steps"] - done)
        assert o.vv(k, dt, grp, thermostat, tau, T0) == 0
        done += k
        th = o.get_thermo()
        rows.append((done * dt, th.temperature, th.kinetic + th.potential, th.kinetic))
    d1 = o.dump()
    o.close()
    return g, d0, d1, np.array(rows)


@pytest.mark.parametrize("name", [n for n in cases.CASES if "turi" not in cases.CASES[n]])
def test_oracle_matches_reference(name):
    g, d0, d1, rows = run_oracle_case(name)
    np.testing.assert_array_equal(d0["id"], g["s0_id"])
    fmax = np.abs(g["s0_F"]).max()
    assert np.abs(d0["F"] - g["s0_F"]).max() <= 1e-12 * fmax
    assert abs(d0["pe"] - float(g["s0_pe"])) <= 1e-12 * abs(float(g["s0_pe"]))
    if name in ("eam", "hybrid", "eam_cu01"):
        assert np.abs(d0["vaream"] - g["s0_vaream"]).max() <= 1e-12 * np.abs(g["s0_vaream"]).max()
    gt = g["thermo"]
    assert rows.shape[0] == gt.shape[0]
    np.testing.assert_allclose(rows[:, 1:], gt[:, 1:], rtol=1e-10, atol=1e-10)
    np.testing.assert_array_equal(d1["id"], g["s1_id"])
    np.testing.assert_array_equal(d1["cell"], g["s1_cell"])
    assert np.abs(d1["x"] - g["s1_x"]).max() <= 1e-9


@pytest.mark.parametrize("name", ["lj", "morse_open"])
def test_oracle_binning_order(name):
    b = dict(np.load(os.path.join(GOLDEN, "bin_" + name + ".npz")))
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    with tempfile.TemporaryDirectory() as work:
        o = oracle_for_case(name, g, work)
    for r in range(1, int(b["rounds"]) + 1):
        o.set_state(b["in%d_x" % r], None)
        assert o.refresh() == 0
        d = o.dump()
        np.testing.assert_array_equal(d["id"], b["r%d_id" % r])
        np.testing.assert_array_equal(d["cell"], b["r%d_cell" % r])
        np.testing.assert_array_equal(d["x"], b["r%d_x" % r])
        o.set_state(d["x"], None)
    o.close()


def test_oracle_threads_agree():
    """The OpenMP variant (per-thread buffers) gives the same forces."""
    g, d0, _, _ = run_oracle_case("eam", threads=1)
    g2, e0, _, _ = run_oracle_case("eam", threads=4)
    assert np.abs(d0["F"] - e0["F"]).max() <= 1e-13 * np.abs(d0["F"]).max()


TTM_CASES = [n for n in cases.CASES if cases.CASES[n].get("turi", {}).get("cat", 0) in (1, 2)]


def run_oracle_ttm(name, threads=1):
    """The oracle on a TTM golden case: the run's first turi update and
    forces, then the case's symplectic-Euler steps; returns (golden, thermo
    rows, TTM arrays, final dump)."""
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    case = cases.CASES[name]
    grp, dt = case["run"][1], case["run"][2]
    with tempfile.TemporaryDirectory() as work:
        o = oracle_for_case(name, g, work, threads)
    tables = {k[len("ttm_tab_"):]: g[k] for k in g if k.startswith("ttm_tab_")}
    o.ttm_setup(g["ttm_pd"], g["ttm_pk"], case["turi"]["Te"], tables)
    # a run's start (src/integrators.c:181-197): the turi update at the
    # current time, then the forces with the friction term
    o.set_time(0.0, dt)
    o.turi_update()
    o.forces(grp)
    th = o.thermo(grp)
    rows = [(0.0, th.temperature, th.kinetic + th.potential, th.kinetic)]
    done = 0
    while done < case["steps"]:
        k = min(case["every"], case["steps"] - done)
        o.se_steps(k, dt, grp)
        done += k
        th = o.thermo(grp)
        rows.append((done * dt, th.temperature, th.kinetic + th.potential, th.kinetic))
    t = o.ttm_1d()
    d1 = o.dump()
    o.close()
    return g, np.array(rows), t, d1


def test_oracle_ttm_threads_agree():
    """The OpenMP pair loops under the TTM step give the same electron
    temperatures and positions as one thread."""
    _, r1, t1, d1 = run_oracle_ttm("ttm_slab", threads=1)
    _, r4, t4, d4 = run_oracle_ttm("ttm_slab", threads=4)
    lo, hi = 1, len(t1["Te"]) - 1
    assert np.abs(t1["Te"][lo:hi] - t4["Te"][lo:hi]).max() <= 1e-11 * np.abs(t1["Te"][lo:hi]).max()
    assert np.abs(d1["x"] - d4["x"]).max() <= 1e-9


@pytest.mark.parametrize("name", TTM_CASES)
def test_oracle_ttm_matches_reference(name):
    """The oracle's two-temperature restatement (turi fields, activation,
    electron solver types 1 and 2, friction term, symplectic Euler) on the
    reference's TTM cases, with the reference's derived TTM parameters from
    the golden file: the final Te, Ti, xi, vcm and atom counts per cell to
    1e-10, the thermo series to 1e-9, the final cell order exact and the
    positions within 1e-9 A."""
    g, rows, t, d1 = run_oracle_ttm(name)
    lo, hi = 1, len(g["ttm_Te"]) - 1
    np.testing.assert_array_equal(t["num"][lo:hi], g["ttm_num"][lo:hi])

    def rel(a, b):
        ok = np.isfinite(b)
        assert np.array_equal(ok, np.isfinite(a))
        return float(np.abs(a[ok] - b[ok]).max() / max(np.abs(b[ok]).max(), 1e-300)) if ok.any() else 0.0

    errs = {q: rel(t[q][lo:hi], g["ttm_" + q][lo:hi]) for q in ("Te", "Ti", "xi", "vcm")}
    print(name, "oracle TTM vs reference:", errs)
    assert max(errs.values()) <= 1e-10, errs
    np.testing.assert_allclose(rows[:, 1:], g["thermo"][:, 1:], rtol=1e-9, atol=1e-9)
    np.testing.assert_array_equal(d1["id"], g["s1_id"])
    np.testing.assert_array_equal(d1["cell"], g["s1_cell"])
    assert np.abs(d1["x"] - g["s1_x"]).max() <= 1e-9


@pytest.mark.parametrize("name", ["ttm1", "ttm_slab", "ttm_slab_full"])
def test_ttm1_params_match_reference(name):
    """The oracle side's derivation of a type-1 TTM turi's parameters from
    the fmd.h-level inputs (pyoracle.ttm1_params: geometry, units, laser,
    front surface, activation threshold) gives the reference's own values
    bit for bit (what the compiled reference left in its ttm_t)."""
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    case = cases.case_of(name)
    tu = case["turi"]
    x = case["state"]()["x"] if name in cases.FULL_CASES else g["state_x"]
    pd, pk = pyoracle.ttm1_params(case["box"], tu["dims"][2], x, tu["gamma"], tu["K"], tu["G"], tu["laser"],
                                  tu["frac"], tu["ratio"])
    used = [i for i in range(17) if i not in (10, 11, 12)]   # (Zhigilei K: type 2 only)
    np.testing.assert_array_equal(pd[used], g["ttm_pd"][used])
    np.testing.assert_array_equal(pk[[0, 1, 2, 5, 6, 7, 8]], g["ttm_pk"][[0, 1, 2, 5, 6, 7, 8]])
