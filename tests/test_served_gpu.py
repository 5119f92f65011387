"""Served mode (fmdg_srv_*): packed multi-job stepping.

* alone vs mix: a job's trajectory does not depend on the other jobs of its
  pack nor on the tuned block size: positions, velocities and forces
  bit-identical; the thermo record's block partial sums may group
  differently (energies within 1e-12 relative);
* pack vs the single-system path (different list, different summation
  order): binary64 positions within 1e-9 A and forces within 1e-9 of max |F|
  after 25 steps; mixed within 1e-6 A and 5e-5;
* pack vs the binary64 oracle at the pack's own final positions: forces,
  and the last thermo record's energy and pair virial
  within 1e-10 (binary64) and 1e-5 (mixed) of max |F|.

Hybrid jobs ("cuar": EAM copper beside Lennard-Jones argon, copper-argon
pairs Lennard-Jones) go through the same checks in packs of their own.
"""
import os
import sys
import tempfile

import numpy as np
import pytest

from fmd_gb300 import serve, workloads

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def L(gpu_lib):
    return serve.bind(gpu_lib.L)


@pytest.fixture(scope="module")
def eam(L):
    return serve.eam_tables(L)


def _job(pot, n, T, seed):
    j = dict(pot=pot, ncell=n, T=T, seed=seed)
    x, v, l = serve.job_atoms(j)
    return x, v, l


def _sys(pot, n, T, seed):
    """x, v, l (edge or three lengths), kind (None: all 0)"""
    j = dict(pot=pot, ncell=n, T=T, seed=seed)
    if pot in serve.HYBRID:
        x, v, kind, l = serve.hybrid_atoms(j)
        return x, v, l, kind
    x, v, l = serve.job_atoms(j)
    return x, v, l, None


ORACLE_POTS = {"lj": ([("Ar", 39.948)], [("lj", 0, 0, 3.405, 0.0104, 8.5125)]),
               "morse": ([("Cu", 63.546)], [("morse", 0, 0, 0.3429, 1.3588, 2.866, 8.0)]),
               "eam": ([("Cu", 63.546)], [("eam", 0, 0)]),
               "cuar": ([("Cu", 63.546), ("Ar", 39.948)],
                        [("eam", 0, 0), ("lj", 1, 1, 3.4, 0.0104, 8.5), ("lj", 0, 1, 2.87, 0.0652, 7.175)])}


def _thermo_close(a, b):
    for f in ("kinetic", "potential"):
        x, y = getattr(a, f), getattr(b, f)
        assert abs(x - y) <= 1e-12 * max(abs(x), abs(y), 1e-30), (f, x, y)


def _by_id(state):
    x, v, F, ids = state
    o = np.argsort(ids)
    return x[o], v[o], F[o]


@pytest.mark.parametrize("pot", ["lj", "morse", "eam", "cuar"])
@pytest.mark.parametrize("precision", [serve.PREC_FP64, serve.PREC_MIXED])
def test_pack_matches_single(L, eam, pot, precision):
    x, v, l, kind = _sys(pot, 6, 700.0, 11)
    steps = 25
    one = serve.Single(L, pot, x, v, l, precision=precision, eam=eam, kind=kind)
    one.steps(steps)
    xs, vs, Fs = _by_id(one.state())
    ts = one.thermo()
    one.close()
    srv = serve.Server(L, chunk_steps=8, eam=eam)
    srv.set_tuning(128)
    jid = srv.submit(pot, x, v, l, steps, precision=precision, keep_state=True, kind=kind)
    srv.drain()
    r = srv.result(jid)
    assert r.state == 2 and r.errbits == 0
    xp, vp, Fp = _by_id(srv.state(jid, len(x)))
    srv.close()
    tx, tf = (1e-9, 1e-9) if precision == serve.PREC_FP64 else (1e-6, 5e-5)
    assert np.abs(xs - xp).max() <= tx
    assert np.abs(Fs - Fp).max() <= tf * np.abs(Fs).max()
    e_s, e_p = ts.kinetic + ts.potential, r.last.kinetic + r.last.potential
    assert abs(e_s - e_p) <= (1e-10 if precision == serve.PREC_FP64 else 1e-6) * abs(e_s)


@pytest.mark.parametrize("pot,ncell", [("lj", 6), ("lj", 5), ("morse", 6), ("morse", 5), ("eam", 6), ("cuar", 6)])
@pytest.mark.parametrize("precision", [serve.PREC_FP64, serve.PREC_MIXED])
def test_pack_forces_vs_oracle(L, eam, pot, ncell, precision):
    """Forces of the packed skin-list kernels after 40 steps of a 1200 K
    cube (the list rebuilt on the way) against the binary64 oracle at the
    same positions.  LJ 5^3 cells: the list radius exceeds the cell (a
    two-cell stencil over three cells per axis); Morse 5^3: two cells per
    axis (a cell is its own upper and lower neighbour)."""
    import pyoracle
    x, v, l, kind = _sys(pot, ncell, 1200.0, 71)
    srv = serve.Server(L, chunk_steps=8, eam=eam)
    srv.set_skin(0.3)
    jid = srv.submit(pot, x, v, l, 40, precision=precision, keep_state=True, kind=kind)
    srv.drain()
    r = srv.result(jid)
    assert r.state == 2
    xp, vp, Fp, ids = srv.state(jid, len(x))
    srv.close()
    nc, cellh, order, counts = serve.host_binning3(xp, l, serve.job_rc(pot))
    kinds, pots = ORACLE_POTS[pot]
    with tempfile.TemporaryDirectory() as work:
        setfl = workloads.write_analytic_eam(os.path.join(work, "a.eam.alloy"))
        o = pyoracle.Oracle()
        o.setup(np.broadcast_to(l, (3,)), [1, 1, 1], nc, cellh, kinds, pots, setfl)
    n = len(xp)
    kp = np.zeros(n, np.uint32) if kind is None else kind[ids]
    ncell_all = int(np.prod(nc))
    o.upload(np.repeat(np.arange(ncell_all, dtype=np.int32), counts), xp[order], vp[order], kp[order],
             np.zeros(n, np.int32), ids[order], ncell_all)
    o.forces(-1)
    d = o.dump()
    o.close()
    Fo = np.zeros_like(Fp)
    Fo[d["id"]] = d["F"]
    Fq = np.zeros_like(Fp)
    Fq[ids] = Fp
    tol = 1e-10 if precision == serve.PREC_FP64 else 1e-5
    err = np.abs(Fq - Fo).max() / np.abs(Fo).max()
    assert err <= tol, err
    # the job's last thermo record (formed by the packed force kernel on its
    # last step, at these positions): energy and pair virial, relative to
    # max(|W|, |PE|) (a hot LJ gas has a small net energy: its pair terms
    # cancel); binary64 1e-10, mixed 1e-6 (energy) and 1e-5 (virial, whose
    # terms f r^2 cancel like the forces)
    scale = max(abs(d["virial"]), abs(d["pe"]))
    tol_pe, tol_w = (1e-10, 1e-10) if precision == serve.PREC_FP64 else (1e-6, 1e-5)
    assert abs(r.last.potential - d["pe"]) <= tol_pe * scale, (r.last.potential, d["pe"])
    assert abs(r.last.virial - d["virial"]) <= tol_w * scale, (r.last.virial, d["virial"])


def test_alone_vs_mix(L, eam):
    """Each job alone and in a mix of 12 jobs of three potentials, hybrid
    jobs and both precisions, uneven sizes and step counts, chunk boundaries falling
    inside jobs, the autotuner switching block sizes between chunks."""
    specs = [("eam", 6, 900.0, 21, 37, 1), ("lj", 5, 80.0, 22, 50, 1), ("morse", 5, 500.0, 23, 19, 1),
             ("eam", 9, 300.0, 24, 44, 1), ("lj", 7, 120.0, 25, 9, 0), ("morse", 7, 1100.0, 26, 31, 0),
             ("eam", 5, 1200.0, 27, 23, 0), ("lj", 6, 60.0, 28, 40, 1), ("morse", 6, 250.0, 29, 28, 1),
             ("cuar", 6, 400.0, 30, 26, 1), ("cuar", 5, 800.0, 31, 33, 0), ("cuar", 7, 200.0, 32, 17, 1)]
    jobs = [(_sys(p, n, T, s), st, pr, p) for (p, n, T, s, st, pr) in specs]
    alone = []
    for (x, v, l, kind), st, pr, p in jobs:
        srv = serve.Server(L, chunk_steps=8, eam=eam)
        jid = srv.submit(p, x, v, l, st, precision=pr, keep_state=True, kind=kind)
        srv.drain()
        alone.append((srv.result(jid), srv.state(jid, len(x))))
        srv.close()
    srv = serve.Server(L, chunk_steps=8, eam=eam)
    ids = [srv.submit(p, x, v, l, st, precision=pr, keep_state=True, kind=kind)
           for (x, v, l, kind), st, pr, p in jobs]
    srv.drain()
    st = srv.stats()
    assert st.finished == len(jobs) and st.failed == 0
    for k, jid in enumerate(ids):
        r = srv.result(jid)
        assert r.state == 2 and r.errbits == 0
        ra, (xa, va, Fa, ia) = alone[k]
        xm, vm, Fm, im = srv.state(jid, len(xa))
        np.testing.assert_array_equal(ia, im)
        np.testing.assert_array_equal(xa, xm)
        np.testing.assert_array_equal(va, vm)
        np.testing.assert_array_equal(Fa, Fm)
        _thermo_close(ra.last, r.last)
        _thermo_close(ra.first, r.first)
    srv.close()


@pytest.mark.parametrize("pot", ["lj", "morse", "eam", "cuar"])
def test_first_thermo_record(L, eam, pot):
    """A served job's record before its first step (formed at admission,
    read back at retirement) equals the single-system path's initial record
    of the same atoms."""
    x, v, l, kind = _sys(pot, 6, 600.0, 97)
    srv = serve.Server(L, chunk_steps=8, eam=eam)
    jid = srv.submit(pot, x, v, l, 10, precision=serve.PREC_FP64, kind=kind)
    srv.drain()
    r = srv.result(jid)
    srv.close()
    one = serve.Single(L, pot, x, v, l, precision=serve.PREC_FP64, eam=eam, kind=kind)
    th0 = one.th0
    one.close()
    assert r.state == 2 and r.first.kinetic > 0 and r.first.potential != 0
    for f in ("kinetic", "potential"):
        a, b = getattr(r.first, f), getattr(th0, f)
        assert abs(a - b) <= 1e-10 * max(abs(a), abs(b)), (f, a, b)


def test_admission_budget(L, eam):
    """A budget that holds about two jobs: every job still finishes, the
    admission accounting never exceeds the budget, results equal an
    unconstrained run's."""
    specs = [("lj", 6, 100.0, 41, 20), ("morse", 6, 300.0, 42, 12), ("eam", 7, 600.0, 43, 17),
             ("lj", 5, 90.0, 44, 30), ("eam", 6, 900.0, 45, 8), ("morse", 5, 700.0, 46, 25)]
    jobs = [(_job(p, n, T, s), st, p) for (p, n, T, s, st) in specs]
    free = serve.Server(L, chunk_steps=4, eam=eam)
    fids = [free.submit(p, x, v, l, st, keep_state=True) for (x, v, l), st, p in jobs]
    free.drain()
    sizes = [free.result(j).device_bytes for j in fids]
    budget = int(2.2 * max(sizes))
    tight = serve.Server(L, budget_bytes=budget, chunk_steps=4, eam=eam)
    tids = [tight.submit(p, x, v, l, st, keep_state=True) for (x, v, l), st, p in jobs]
    tight.drain()
    s = tight.stats()
    assert s.finished == len(jobs) and s.failed == 0
    assert s.bytes_peak <= budget
    for a, b, ((x, v, l), st, p) in zip(fids, tids, jobs):
        xa = free.state(a, len(x))
        xb = tight.state(b, len(x))
        for u, w in zip(xa, xb):
            np.testing.assert_array_equal(u, w)
    free.close()
    tight.close()


def test_oversize_job_fails_cleanly(L, eam):
    srv = serve.Server(L, budget_bytes=100000, chunk_steps=4, eam=eam)
    x, v, l = _job("lj", 6, 100.0, 51)
    jid = srv.submit("lj", x, v, l, 5)
    srv.drain()
    r = srv.result(jid)
    assert r.state == 3 and r.error == 3
    srv.close()


@pytest.mark.parametrize("pot", ["lj", "morse", "eam", "cuar"])
def test_mixed_force_error_bound(L, eam, pot):
    """Mixed precision against binary64 at identical positions of a
    thermalised cube (1200 K, 20 binary64 steps): max |F32 - F64| <= 1e-5
    max |F64|."""
    x, v, l, kind = _sys(pot, 7, 1200.0, 61)
    one = serve.Single(L, pot, x, v, l, precision=serve.PREC_FP64, eam=eam, kind=kind)
    one.steps(20)
    serve.check(L, L.fmdg_compute_forces(one.h, -1), "forces")
    F64 = one.state()[2]
    serve.check(L, L.fmdg_set_precision(one.h, serve.PREC_MIXED), "precision")
    serve.check(L, L.fmdg_compute_forces(one.h, -1), "forces")
    F32 = one.state()[2]
    one.close()
    err = np.abs(F32 - F64).max() / np.abs(F64).max()
    assert err <= 1e-5, err


@pytest.mark.parametrize("pot,ncell", [("lj", 6), ("morse", 5), ("morse", 8), ("eam", 10)])
def test_mixed_force_error_cold(L, eam, pot, ncell):
    """Cold crystals (50 K) have the smallest net forces, so the largest
    relative errors: the packed mixed-precision kernels after 24 steps
    against the binary64 oracle at the job's own positions, max |dF| <= 1e-5
    max |F| (the stream's coldest jobs are at 50 K)."""
    x, v, l, kind = _sys(pot, ncell, 50.0, 91)
    srv = serve.Server(L, chunk_steps=8, eam=eam)
    jid = srv.submit(pot, x, v, l, 24, precision=serve.PREC_MIXED, keep_state=True)
    srv.drain()
    assert srv.result(jid).state == 2
    xp, vp, Fp, ids = srv.state(jid, len(x))
    srv.close()
    Fo = _oracle_forces(pot, l, kind, xp, vp, ids)
    Fq = np.zeros_like(Fp)
    Fq[ids] = Fp
    err = np.abs(Fq - Fo).max() / np.abs(Fo).max()
    print(pot, ncell, "cold mixed force error %.3e" % err)
    assert err <= 1e-5, err


def test_more_jobs_than_one_pack(L, eam):
    """40 jobs of one category and precision need two packs (at most 32
    systems travel in one launch); every job still equals its run alone bit
    for bit."""
    jobs = [_job("lj", 5, 60.0 + 20.0 * k, 100 + k) for k in range(40)]
    srv = serve.Server(L, chunk_steps=8, eam=eam)
    ids = [srv.submit("lj", x, v, l, 21 + (k % 5), keep_state=True) for k, (x, v, l) in enumerate(jobs)]
    srv.drain()
    assert srv.stats().finished == 40
    for k in (0, 17, 33, 39):
        x, v, l = jobs[k]
        one = serve.Server(L, chunk_steps=8, eam=eam)
        jo = one.submit("lj", x, v, l, 21 + (k % 5), keep_state=True)
        one.drain()
        a = one.state(jo, len(x))
        one.close()
        b = srv.state(ids[k], len(x))
        for u, w in zip(a, b):
            np.testing.assert_array_equal(u, w)
    srv.close()


@pytest.mark.parametrize("precision", [serve.PREC_FP64, serve.PREC_MIXED])
def test_long_hot_run(L, eam, precision):
    """300 steps of a 1200 K argon gas: atoms cross periodic faces and each
    packed list is rebuilt many times (cells refreshed on rebuild steps
    only, slots renumbered at every rebuild).  binary64: positions within
    1e-8 A (minimum image) of the single-system path, which refreshes its
    cells every step; both precisions: final forces against the binary64
    oracle at the pack's own positions (1e-10 / 1e-5 of max |F|)."""
    import pyoracle
    x, v, l, kind = _sys("lj", 6, 1200.0, 81)
    steps = 300
    srv = serve.Server(L, chunk_steps=16, eam=eam)
    jid = srv.submit("lj", x, v, l, steps, precision=precision, keep_state=True)
    srv.drain()
    r = srv.result(jid)
    assert r.state == 2 and r.errbits == 0
    xp, vp, Fp, ids = srv.state(jid, len(x))
    srv.close()
    assert xp.min() >= 0.0 and xp.max() < l
    if precision == serve.PREC_FP64:
        one = serve.Single(L, "lj", x, v, l, precision=serve.PREC_FP64)
        one.steps(steps)
        xs, vs, Fs = _by_id(one.state())
        one.close()
        o = np.argsort(ids)
        d = xs - xp[o]
        d -= l * np.round(d / l)
        assert np.abs(d).max() <= 1e-8
    nc, cellh, order, counts = serve.host_binning3(xp, l, serve.job_rc("lj"))
    kinds, pots = ORACLE_POTS["lj"]
    o = pyoracle.Oracle()
    o.setup(np.broadcast_to(l, (3,)), [1, 1, 1], nc, cellh, kinds, pots, None)
    n = len(xp)
    ncell_all = int(np.prod(nc))
    o.upload(np.repeat(np.arange(ncell_all, dtype=np.int32), counts), xp[order], vp[order], np.zeros(n, np.uint32),
             np.zeros(n, np.int32), ids[order], ncell_all)
    o.forces(-1)
    dd = o.dump()
    o.close()
    Fo = np.zeros_like(Fp)
    Fo[dd["id"]] = dd["F"]
    Fq = np.zeros_like(Fp)
    Fq[ids] = Fp
    tol = 1e-10 if precision == serve.PREC_FP64 else 1e-5
    err = np.abs(Fq - Fo).max() / np.abs(Fo).max()
    assert err <= tol, err


def _oracle_forces(pot, l, kind, xp, vp, ids):
    import pyoracle
    nc, cellh, order, counts = serve.host_binning3(xp, l, serve.job_rc(pot))
    kinds, pots = ORACLE_POTS[pot]
    with tempfile.TemporaryDirectory() as work:
        setfl = workloads.write_analytic_eam(os.path.join(work, "a.eam.alloy"))
        o = pyoracle.Oracle()
        o.setup(np.broadcast_to(l, (3,)), [1, 1, 1], nc, cellh, kinds, pots, setfl)
    n = len(xp)
    kp = np.zeros(n, np.uint32) if kind is None else kind[ids]
    ncell_all = int(np.prod(nc))
    o.upload(np.repeat(np.arange(ncell_all, dtype=np.int32), counts), xp[order], vp[order], kp[order],
             np.zeros(n, np.int32), ids[order], ncell_all)
    o.forces(-1)
    d = o.dump()
    o.close()
    Fo = np.zeros_like(xp)
    Fo[d["id"]] = d["F"]
    return Fo


@pytest.mark.parametrize("pot", ["morse", "cuar"])
@pytest.mark.parametrize("precision", [serve.PREC_FP64, serve.PREC_MIXED])
def test_list_overflow_fallback(L, eam, pot, precision):
    """Lists of 32 entries per atom, far fewer than the neighbours: every
    atom scans its stencil directly (current positions relative to the
    cells of the last refresh, one image per neighbour -- the hybrid box has
    two cells along y and z, so cells recur in the stencil).  Against the
    same job with full lists: binary64 positions within 1e-12 A after 40
    steps at 1200 K, mixed within 1e-6 A; final forces against the binary64
    oracle (1e-10 / 1e-5)."""
    x, v, l, kind = _sys(pot, 6, 1200.0, 91)
    out = []
    for cap in (0, 32):
        srv = serve.Server(L, chunk_steps=8, eam=eam)
        srv.set_skin(0.3)
        srv.set_list_capacity(cap)
        jid = srv.submit(pot, x, v, l, 40, precision=precision, keep_state=True, kind=kind)
        srv.drain()
        assert srv.result(jid).state == 2
        out.append(srv.state(jid, len(x)))
        srv.close()
    (xa, va, Fa, ia), (xb, vb, Fb, ib) = out
    oa, ob = np.argsort(ia), np.argsort(ib)
    d = xa[oa] - xb[ob]
    d -= np.broadcast_to(l, (3,)) * np.round(d / np.broadcast_to(l, (3,)))
    assert np.abs(d).max() <= (1e-12 if precision == serve.PREC_FP64 else 1e-6)
    Fo = _oracle_forces(pot, l, kind, xb, vb, ib)
    Fq = np.zeros_like(Fb)
    Fq[ib] = Fb
    err = np.abs(Fq - Fo).max() / np.abs(Fo).max()
    assert err <= (1e-10 if precision == serve.PREC_FP64 else 1e-5), err


@pytest.mark.parametrize("pot,cap", [("lj", 0), ("morse", 0), ("eam", 0), ("cuar", 0), ("cuar", 32)])
def test_single_build_lanes_same_list(L, eam, pot, cap):
    """Skin-list builds with 1, 2, 4, 8, 16 and 32 threads per atom build the
    same list, entry for entry (also when it overflows): the same trajectory
    bit for bit, the binary32 partial sums flushing at the same entries.
    60 steps at 900 K include list rebuilds after the first build."""
    x, v, l, kind = _sys(pot, 6, 900.0, 95)
    res = []
    for lanes in (1, 2, 4, 8, 16, 32):
        one = serve.Single(L, pot, x, v, l, precision=serve.PREC_MIXED, eam=eam, kind=kind, list_capacity=cap,
                           build_lanes=lanes)
        one.steps(60)
        res.append(_by_id(one.state()))
        one.close()
    for r in res[1:]:
        for a, b in zip(res[0], r):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("precision", [serve.PREC_FP64, serve.PREC_MIXED])
def test_single_list_overflow_fallback(L, eam, precision):
    """The single-system path with lists of 32 entries: the same pairs in
    the same order as with full lists, so the same trajectory (binary64
    bit for bit; mixed within 1e-6 A: partial sums group differently)."""
    x, v, l, kind = _sys("cuar", 6, 900.0, 93)
    res = []
    for cap in (0, 32):
        one = serve.Single(L, "cuar", x, v, l, precision=precision, eam=eam, kind=kind, list_capacity=cap)
        one.steps(20)
        res.append(_by_id(one.state()))
        one.close()
    (xa, va, Fa), (xb, vb, Fb) = res
    if precision == serve.PREC_FP64:
        np.testing.assert_array_equal(xa, xb)
        np.testing.assert_array_equal(Fa, Fb)
    else:
        assert np.abs(xa - xb).max() <= 1e-6
