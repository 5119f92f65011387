"""Full-size runs of the reference-path configurations through the fmd.h
API on the GPU.

* argon LJ, 4000 atoms: 2 ps Berendsen equilibration (tau 0.1 ps, 100 K)
  then 10 000 NVE steps at 2 fs; trajectories diverge chaotically, so the
  NVE energy drift (max |E(t) - E(0)| / |E(0)| over 20 samples) is compared:
  binary64 and mixed precision within 2x the oracle's drift (+1e-7).
* EAM copper, 256 000 atoms: the NVE drift of each precision within 2x the
  oracle's over the first 2000 steps (the configured potential collapses
  the crystal later on), the step-0 potential energy, and the forces
  against the oracle at the positions of step 250 (the configuration starts
  on exact lattice sites, where the forces vanish); 100 binary64 steps
  against the compiled reference's run (thermo series, energies, final
  state of 2048 atoms).
* Morse collision, 512 000-atom slab + a 20 A projectile sphere at 2 km/s,
  periodic x, y, 100 A vacuum in z: step-0 forces against the oracle
  (binary64 1e-10, mixed 1e-5 of max |F|), then 200 steps: no atom lost
  before the impact, transverse momentum conserved (binary64: to 1e-9 of
  sum |m v|; mixed: centre-of-mass velocity change below 1e-4 A/ps); 100
  binary64 steps against the compiled reference's run of the same protocol.
* laser-heated EAM slab with a 1-D TTM grid (20 x 20 x 100 FCC cells =
  160 000 atoms, vacuum above and below, 50 TTM cells along z): 120 steps
  around the pulse against the compiled reference's run of the same
  protocol: every field event and array, the final Te, Ti, xi and counts
  per cell to 1e-10.
"""
import ctypes as C
import os
import sys
import tempfile

import numpy as np
import pytest

import cases
from test_parity_oracle_gpu import build_both

from fmd_gb300 import api, workloads

pytestmark = pytest.mark.gpu


def _energy(lib, md):
    return lib.fmd_matt_getTotalEnergy(md)


def _lj4000():
    x, v = workloads.fcc_state(10, 10, 10, 5.26, 100.0, 39.948, seed=1)
    return dict(box=(52.6,) * 3, pbc=(1, 1, 1), kinds=[("Ar", 39.948)],
                pots=[("lj", 0, 0, 3.405, 0.0104, 8.5125)], x=x, v=v, kind=np.zeros(len(x), np.uint32),
                group=np.zeros(len(x), np.int32), dt=0.002)


def _drift(series):
    e = np.asarray(series)
    assert np.all(np.isfinite(e))
    return float(np.abs(e - e[0]).max() / abs(e[0]))


def test_lj_argon_nve_drift(gpu_lib):
    lib = gpu_lib
    spec = _lj4000()
    drifts = {}
    with tempfile.TemporaryDirectory() as work:
        for prec in (0, 1):
            md, o = build_both(lib, spec, work, precision=prec)
            lib.fmd_dync_equilibrate(md, -1, 2.0, 0.002, 0.1, 100.0)
            es = [_energy(lib, md)]
            for _ in range(20):
                lib.fmd_dync_integrate(md, -1, 1.0, 0.002)
                es.append(_energy(lib, md))
            drifts[prec] = _drift(es)
            lib.fmd_free(md)
            if prec == 1:
                # the oracle: the same protocol in binary64 on the host
                o.set_threads(os.cpu_count() or 1)
                o.forces(-1)
                o.thermo(-1)          # the first Berendsen scale needs T
                o.vv(1000, 0.002, -1, 1, 0.1, 100.0)
                th = o.get_thermo()
                eo = [th.kinetic + th.potential]
                for _ in range(20):
                    o.vv(500, 0.002)
                    th = o.get_thermo()
                    eo.append(th.kinetic + th.potential)
                drifts["oracle"] = _drift(eo)
            o.close()
    bound = 2.0 * drifts["oracle"] + 1e-7
    assert drifts[0] <= bound, drifts
    assert drifts[1] <= bound, drifts


def _eam256k():
    x, v = workloads.fcc_state(40, 40, 40, 3.615, 300.0, 63.546, seed=2)
    return dict(box=(40 * 3.615,) * 3, pbc=(1, 1, 1), kinds=[("Cu", 63.546)], pots=[("eam", 0, 0)], x=x, v=v,
                kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), dt=0.001)


def test_eam256k_full_size(gpu_lib):
    """The 256 000-atom EAM configuration (FCC 40^3, 300 K seed 2, dt 1 fs):
    NVE steps in each precision, the energy drift (max |E(t) - E(0)| /
    |E(0)| over samples every 250 steps) within 2x the oracle's drift on the
    same protocol (+1e-7); the step-0 potential energy against the oracle
    (binary64 1e-10, mixed 1e-7 relative); and the forces against the
    binary64 oracle at the positions of step 250 of each run (binary64
    1e-10, mixed 1e-5 of max |F|).  The configuration starts from exact
    lattice sites, where every force vanishes by symmetry (the computed
    ones are rounding noise of ~1e-14 eV/A), so the forces are compared
    once the thermal velocities have displaced the atoms.  The configuration
    asks for 5000 steps, but its analytic EAM collapses the crystal after
    ~1000 steps and the oracle's (and the reference's) run stops before
    step 5000, so the drift is compared over the first 2000 steps.  The
    oracle's run takes many minutes of host time, so its record is kept in
    tests/golden/cfg1_drift.json (make_cfg1_drift.py)."""
    import json
    lib = gpu_lib
    spec = _eam256k()
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cfg1_drift.json")
    if not os.path.exists(path):
        pytest.skip("the oracle's drift record (make_cfg1_drift.py) is absent")
    ref = json.load(open(path))
    drifts, errs, pe_errs = {}, {}, {}
    nc = None
    with tempfile.TemporaryDirectory() as work:
        for prec in (0, 1):
            md, o = build_both(lib, spec, work, precision=prec)
            nc = lib.grid(md)[0]
            lib.fmd_dync_integrate(md, -1, 0.0, 0.001)
            pe0 = lib.dump(md)["pe"]
            o.set_threads(os.cpu_count() or 1)
            o.forces(-1)
            pe0_oracle = o.dump()["pe"]
            pe_errs[prec] = abs(pe0 - pe0_oracle) / abs(pe0_oracle)
            if prec == 0:
                e0_oracle = pe0_oracle + o.thermo(-1).kinetic
            es = [_energy(lib, md)]
            for seg in range(ref["steps"] // ref["every"]):
                lib.fmd_dync_integrate(md, -1, (ref["every"] - 0.5) * 0.001, 0.001)
                es.append(_energy(lib, md))
                if seg == 0:
                    # forces at the positions of step 250: the run's own state
                    # (its cell order) into the oracle
                    d = lib.dump(md)
                    o.upload(d["cell"], d["x"], d["v"], d["kind"], d["group"], d["id"], int(np.prod(nc)))
                    o.forces(-1)
                    r = o.dump()
                    np.testing.assert_array_equal(d["id"], r["id"])
                    errs[prec] = float(np.abs(d["F"] - r["F"]).max() / np.abs(r["F"]).max())
            o.close()
            drifts[prec] = _drift(es)
            lib.fmd_free(md)
    print("EAM 256k: force errors at step 250", errs, "step-0 PE errors", pe_errs, "drifts", drifts,
          "oracle drift", ref["drift"])
    assert errs[0] <= 1e-10 and errs[1] <= 1e-5, errs
    assert pe_errs[0] <= 1e-10 and pe_errs[1] <= 1e-7, pe_errs
    # the same initial total energy as the oracle's recorded run
    assert abs(ref["energies"][0] - e0_oracle) <= 1e-10 * abs(e0_oracle)
    bound = 2.0 * ref["drift"] + 1e-7
    assert drifts[0] <= bound and drifts[1] <= bound, (drifts, ref["drift"])


def _reference_run(lib, name, n_expect):
    """Run full-size case `name` (cases.FULL_CASES) in binary64 and compare
    it with the compiled reference's run of the same protocol
    (tests/golden/<name>.npz; the seeded state is regenerated here): the
    thermo series and the potential energy before and after to 1e-9, and
    the final positions (1e-8 A), velocities (1e-8 relative) and forces
    (1e-9 of the largest) of the sampled atoms.  Returns the deviations."""
    case = cases.FULL_CASES[name]
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name + ".npz")))
    state = case["state"]()
    assert len(state["x"]) == n_expect == int(g["n0"])
    with tempfile.TemporaryDirectory() as work:
        md, _ = cases.setup(lib, name, work, state)
        lib.fmd_dync_integrate(md, -1, 0.0, case["run"][2])
        pe0 = lib.dump(md)["pe"]
        rec = cases.Recorder(lib)
        cases.run(lib, name, md, rec)
        d1 = lib.dump(md)
        lib.fmd_free(md)
    assert rec.errors == [], rec.errors
    assert len(d1["id"]) == int(g["n1"])
    np.testing.assert_allclose(np.array(rec.rows)[:, 1:], g["thermo"][:, 1:], rtol=1e-9, atol=1e-9)
    # total potential energies to 1e-9: the reference adds every pair energy
    # (~5e7 for the Morse collision) into one binary64 accumulator in its
    # loop order, whose rounding alone reaches 1e-10 relative at this size
    # (the engine's per-atom double-float sums are the more accurate ones)
    pe_err = (abs(pe0 - float(g["s0_pe"])) / abs(float(g["s0_pe"])),
              abs(d1["pe"] - float(g["s1_pe"])) / abs(float(g["s1_pe"])))
    assert max(pe_err) <= 1e-9, pe_err
    pos = np.empty(int(d1["id"].max()) + 1, np.int64)
    pos[d1["id"]] = np.arange(len(d1["id"]))
    sel = pos[g["sample_id"]]
    dx = np.abs(d1["x"][sel] - g["sample_x"]).max()
    dv = np.abs(d1["v"][sel] - g["sample_v"]).max() / np.abs(g["sample_v"]).max()
    dF = np.abs(d1["F"][sel] - g["sample_F"]).max() / float(g["F_absmax"])
    print("%s vs the reference after %d steps: dx %.2e A, dv %.2e, dF %.2e, PE %.2e / %.2e"
          % (name, case["steps"], dx, dv, dF, pe_err[0], pe_err[1]))
    assert dx <= 1e-8 and dv <= 1e-8 and dF <= 1e-9, (dx, dv, dF)
    return dx, dv, dF


def test_eam256k_reference_run(gpu_lib):
    """The 256 000-atom EAM configuration, 100 binary64 steps, against the
    compiled reference's run of the same protocol (`_reference_run`; the
    2048 atoms with the lowest ids sampled)."""
    _reference_run(gpu_lib, "eam256k_full", 256000)


def test_morse_collision_reference_run(gpu_lib):
    """The Morse collision configuration (515 000 atoms, open z), 100
    binary64 steps, against the compiled reference's run of the same
    protocol (`_reference_run`; 2048 atoms sampled across the id range,
    slab and projectile)."""
    _reference_run(gpu_lib, "morse_collision_full", len(cases.FULL_CASES["morse_collision_full"]["state"]()["x"]))


def _collision(seed=3):
    box, x, v = cases.collision_atoms(seed)
    return dict(box=box, pbc=(1, 1, 0), kinds=[("Cu", 63.546)],
                pots=[("morse", 0, 0, 0.3429, 1.3588, 2.866, 8.0)], x=x, v=v,
                kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), dt=0.001)


@pytest.mark.parametrize("precision", [0, 1])
def test_morse_collision_full_size(gpu_lib, precision):
    lib = gpu_lib
    spec = _collision()
    n0 = len(spec["x"])
    assert n0 > 512000
    with tempfile.TemporaryDirectory() as work:
        md, o = build_both(lib, spec, work, precision=precision)
        lib.fmd_dync_integrate(md, -1, 0.0, 0.001)
        g0 = lib.dump(md)
        o.set_threads(os.cpu_count() or 1)
        o.forces(-1)
        r0 = o.dump()
        o.close()
        np.testing.assert_array_equal(g0["id"], r0["id"])
        tol = 1e-10 if precision == 0 else 1e-5
        err = np.abs(g0["F"] - r0["F"]).max() / np.abs(r0["F"]).max()
        assert err <= tol, err
        p0 = (C.c_double * 3)()
        lib.fmd_matt_getMomentum(md, p0)
        lib.fmd_dync_integrate(md, -1, 0.1995, 0.001)
        p1 = (C.c_double * 3)()
        lib.fmd_matt_getMomentum(md, p1)
        d = lib.dump(md)
        assert len(d["id"]) == n0
        m = 63.546 / workloads.MD_MASS_UNIT
        if precision == 0:
            scale = np.abs(d["v"]).sum() * m
            assert abs(p1[0] - p0[0]) <= 1e-9 * scale and abs(p1[1] - p0[1]) <= 1e-9 * scale
        else:
            # pair forces are exactly antisymmetric, but in a crystal every
            # atom's binary32 partial sums round alike, so the net force is
            # N times one rounding error, not sqrt(N) times: bound the
            # centre-of-mass velocity it leaves (A/ps)
            dv = np.hypot(p1[0] - p0[0], p1[1] - p0[1]) / (n0 * m)
            assert dv <= 1e-4, dv
        lib.fmd_free(md)


def test_ttm_slab_full_size(gpu_lib):
    """The TTM configuration's slab at full size (20 x 20 x 100 FCC cells,
    160 000 atoms, 50 electron cells), 120 binary64 steps around the pulse
    at 0.06 ps, against the reference run of the same protocol
    (tests/golden/ttm_slab_full.npz, made by make_golden.py from the
    compiled reference): the thermo series to 1e-9, every field-update
    event in order, every field array it carries (Te and the atomic fields)
    and the final Te, Ti, xi and atom counts per cell to 1e-10 relative; no
    error event, the electrons heated where the pulse arrives."""
    from test_parity_golden_gpu import TTM_TOL, FIELD_TOL, _rel
    lib = gpu_lib
    name = "ttm_slab_full"
    case = cases.FULL_CASES[name]
    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name + ".npz")))
    state = case["state"]()
    assert len(state["x"]) == 160000 == int(g["n0"])
    with tempfile.TemporaryDirectory() as work:
        md, _ = cases.setup(lib, name, work, state)
        rec = cases.Recorder(lib)
        rec.record_fields(md, case["turi"]["_handle"])
        lib.fmd_setEventHandler(md, None, rec.cb)
        lib.fmd_dync_integrate(md, -1, 0.0, case["run"][2])
        cases.run(lib, name, md, rec)
        assert rec.errors == [], rec.errors
        ttm = lib.ttm_1d(md)
        assert len(lib.dump(md)["id"]) == int(g["n1"])
        lib.fmd_free(md)
    # temperature, total and kinetic energy every 40 steps
    np.testing.assert_allclose(np.array(rec.rows)[:, 1:], g["thermo"][:, 1:], rtol=1e-9, atol=1e-9)
    ev = np.array([(t, tu, f) for (t, tu, f, _) in rec.fields]).reshape(-1, 3)
    np.testing.assert_array_equal(ev[:, 1:], g["field_events"][:, 1:])
    np.testing.assert_allclose(ev[:, 0], g["field_events"][:, 0], rtol=0, atol=1e-12)
    worst = {}
    for k, (t, _, f, vals) in enumerate(rec.fields):
        key = "field_%03d" % k
        if key not in g:
            continue
        cat = rec.field_cats.get(int(f))
        e = _rel(vals, g[key])
        worst[cat] = max(worst.get(cat, 0.0), e)
        assert e <= (TTM_TOL if cat == api.FMD_FIELD_TTM_TE else FIELD_TOL), (key, t, cat, e)
    lo, hi = 1, len(g["ttm_Te"]) - 1
    np.testing.assert_array_equal(ttm["num"][lo:hi], g["ttm_num"][lo:hi])
    errs = {q: _rel(ttm[q][lo:hi], g["ttm_" + q][lo:hi]) for q in ("Te", "xi", "Ti")}
    print("TTM slab 160k: field errors by category", worst, "final", errs)
    assert errs["Te"] <= TTM_TOL and errs["xi"] <= FIELD_TOL and errs["Ti"] <= FIELD_TOL, errs
    te = np.asarray(ttm["Te"])
    active = te >= 0.0
    assert active.sum() > 10 and np.all(np.isfinite(te[active])) and te[active].max() > 300.5
