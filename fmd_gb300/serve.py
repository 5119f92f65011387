"""Python binding of the device engine's served mode (include/fmdg.h,
`fmdg_srv_*`) and the synthetic served job stream.

The served stream: independent MD jobs of FCC cubes with periodic faces,
arriving as a Poisson process; sizes log-uniform between 500 and 200 000
atoms rounded to 4 n^3 atoms; potential uniform over the argon
Lennard-Jones (a = 5.26 A, dt = 2 fs), copper Morse (a = 3.615 A, rc = 8 A,
dt = 1 fs) and the analytic copper EAM (a = 3.615 A, dt = 1 fs); Maxwell
velocities at a temperature uniform in [50, 1200] K; step counts uniform in
[1000, 20000].  Every cube satisfies l > 2 rc, the minimum-image condition
of the 27-cell stencil (Morse n = 5: l = 18.1 A > 16 A).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import tempfile

import numpy as np

from . import workloads

FMDG_POT_LJ, FMDG_POT_EAM, FMDG_POT_MORSE = 1, 2, 3
PREC_FP64, PREC_MIXED = 0, 1


class Pair(C.Structure):
    _fields_ = [("cat", C.c_int), ("iloc", C.c_int), ("jloc", C.c_int), ("pad", C.c_int),
                ("p", C.c_double * 4)]


class Thermo(C.Structure):
    _fields_ = [("kinetic", C.c_double), ("temperature", C.c_double), ("momentum", C.c_double * 3),
                ("potential", C.c_double), ("count", C.c_double), ("virial", C.c_double)]


class JobDesc(C.Structure):
    _fields_ = [("l", C.c_double * 3), ("pbc", C.c_int * 3), ("nkinds", C.c_int),
                ("mass", C.POINTER(C.c_double)), ("eam_elem", C.POINTER(C.c_int)),
                ("pairs", C.POINTER(Pair)), ("eam_key", C.c_int), ("n", C.c_int),
                ("x", C.POINTER(C.c_double)), ("v", C.POINTER(C.c_double)),
                ("kind", C.POINTER(C.c_uint)), ("steps", C.c_int), ("dt", C.c_double),
                ("precision", C.c_int), ("keep_state", C.c_int)]


class JobResult(C.Structure):
    _fields_ = [("state", C.c_int), ("error", C.c_int), ("n", C.c_int), ("steps", C.c_int),
                ("t_submit", C.c_double), ("t_start", C.c_double), ("t_done", C.c_double),
                ("first", Thermo), ("last", Thermo), ("errbits", C.c_uint), ("pad", C.c_uint),
                ("device_bytes", C.c_double)]


class SrvStats(C.Structure):
    _fields_ = [("queued", C.c_int), ("running", C.c_int), ("admitted", C.c_longlong),
                ("finished", C.c_longlong), ("failed", C.c_longlong), ("atom_steps", C.c_double),
                ("kernels", C.c_longlong), ("bytes_in_use", C.c_double), ("bytes_peak", C.c_double),
                ("pack_fblk", (C.c_int * 2) * 4), ("pack_chunks", (C.c_longlong * 2) * 4),
                ("pack_rebuilds", (C.c_longlong * 2) * 4)]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def bind(L):
    """A handle of the loaded libfmd with the fmdg_* prototypes declared
    (a separate ctypes object, so other bindings of the library keep their
    own argument types)."""
    L = C.CDLL(L._name)
    vp, i, d, sz = C.c_void_p, C.c_int, C.c_double, C.c_size_t
    P = C.POINTER
    protos = {
        "fmdg_create": ([P(vp), i], i), "fmdg_destroy": ([vp], None),
        "fmdg_set_box": ([vp, P(d), P(i), P(i), P(d)], i),
        "fmdg_set_kinds": ([vp, i, P(d), P(i)], i), "fmdg_set_pairs": ([vp, P(Pair)], i),
        "fmdg_set_eam": ([vp, i, i, d, i, d] + [P(d)] * 6, i), "fmdg_set_precision": ([vp, i], i),
        "fmdg_share_eam": ([vp, vp], i),
        "fmdg_upload": ([vp, i, P(i), P(d), P(d), P(C.c_uint), P(i), P(C.c_uint)], i),
        "fmdg_natoms": ([vp, P(i)], i),
        "fmdg_download": ([vp, P(i), P(d), P(d), P(d), P(d), P(C.c_uint), P(i), P(C.c_uint)], i),
        "fmdg_compute_forces": ([vp, i], i), "fmdg_thermo": ([vp, i, P(Thermo)], i),
        "fmdg_vv_steps": ([vp, i, d, i, i, d, d], i), "fmdg_get_thermo": ([vp, P(Thermo)], i),
        "fmdg_get_errors": ([vp, P(C.c_uint), i], i), "fmdg_sync": ([vp], i),
        "fmdg_last_error": ([], C.c_char_p),
        "fmdg_srv_create": ([P(vp), i, sz, i, i], i), "fmdg_srv_destroy": ([vp], None),
        "fmdg_srv_set_eam": ([vp, i, i, i, d, i, d] + [P(d)] * 6, i),
        "fmdg_srv_set_tuning": ([vp, i], i), "fmdg_srv_set_skin": ([vp, d], i),
        "fmdg_srv_set_list_capacity": ([vp, i], i), "fmdg_set_list_capacity": ([vp, i], i),
        "fmdg_set_build_lanes": ([vp, i], i),
        "fmdg_srv_submit": ([vp, P(JobDesc), P(C.c_longlong)], i),
        "fmdg_srv_progress": ([vp, i, P(i)], i), "fmdg_srv_result": ([vp, C.c_longlong, P(JobResult)], i),
        "fmdg_srv_state": ([vp, C.c_longlong, P(d), P(d), P(d), P(C.c_uint)], i),
        "fmdg_srv_release": ([vp, C.c_longlong], i), "fmdg_srv_now": ([vp, P(d)], i),
        "fmdg_srv_stats": ([vp, P(SrvStats)], i), "fmdg_srv_admit": ([vp], i),
        "fmdg_srv_run_resident": ([vp, i, P(C.c_float)], i),
        "fmdg_srv_profile_pack": ([vp, i, i, P(C.c_float), P(d), P(i)], i),
        "fmdg_measure_fma_peak": ([vp, i, P(d)], i),
        "fmdx_eam_tables": ([vp, P(i), P(i), P(d), P(i), P(d), P(d)] + [P(d)] * 6, i),
        "fmd_create": ([], vp), "fmd_free": ([vp], None),
        "fmd_pot_eam_alloy_load": ([vp, C.c_char_p], vp),
        "fmd_io_setShowErrorMessages": ([vp, C.c_bool], None),
    }
    for name, (at, rt) in protos.items():
        f = getattr(L, name)
        f.argtypes = at
        f.restype = rt
    return L


class EngineError(RuntimeError):
    pass


def check(L, rc, what):
    if rc != 0:
        raise EngineError("%s: status %d: %s" % (what, rc, L.fmdg_last_error().decode(errors="replace")))


# ------------------------------------------------------------------ potentials
MD_MASS_UNIT = workloads.MD_MASS_UNIT

# Serving defaults per potential: the Verlet skin (A) and the neighbour-list
# entries per atom (0: estimated from the job's initial density).  The
# analytic EAM collapses its copper crystals to ~2.4x their density over a
# few thousand steps (no equilibrium near a = 3.615 A), so its lists are
# sized for the collapsed density (an atom beyond its list's capacity scans
# its cell stencil directly, several times slower) and its skin is smaller
# (the dense lists cost more than the extra rebuilds): measured on the
# resident 2048-job fleet after 2000 steps, 1.05e9 -> 1.12e9 atom-steps/s.
POTENTIALS = {
    "lj": dict(cat=FMDG_POT_LJ, a=5.26, mass=39.948, dt=0.002, rc=8.5125,
               p=(4 * 0.0104, 3.405 ** 2, 8.5125 ** 2, 0.0), skin=0.8, list_capacity=0),
    "morse": dict(cat=FMDG_POT_MORSE, a=3.615, mass=63.546, dt=0.001, rc=8.0,
                  p=(0.3429, 1.3588, 2.866, 64.0), skin=0.8, list_capacity=0),
    "eam": dict(cat=FMDG_POT_EAM, a=3.615, mass=63.546, dt=0.001, rc=workloads.EAM_RC,
                p=(0.0, 0.0, workloads.EAM_RC ** 2, 0.0), skin=0.5, list_capacity=288),
}
POT_NAMES = ["lj", "morse", "eam"]

# Jobs that mix pair categories (the reference's hybrid tables,
# src/potential.h:26-32): a copper block on the analytic EAM beside an argon
# block on Lennard-Jones, copper-argon pairs Lennard-Jones (the parameters of
# the hybrid test case).  They form packs of their own (class 0).
HYBRID = {
    "cuar": dict(kinds=[("Cu", 63.546, 0), ("Ar", 39.948, -1)], dt=0.001, rc=8.5,
                 pairs={(0, 0): (FMDG_POT_EAM, (0.0, 0.0, workloads.EAM_RC ** 2, 0.0)),
                        (1, 1): (FMDG_POT_LJ, (4 * 0.0104, 3.4 ** 2, 8.5 ** 2, 0.0)),
                        (0, 1): (FMDG_POT_LJ, (4 * 0.0652, 2.87 ** 2, 7.175 ** 2, 0.0))}),
}


def job_table(pot):
    """Masses (internal units), EAM elements and the kind-pair table of a
    job type: one kind for the single-potential types, several for HYBRID."""
    if pot in HYBRID:
        H = HYBRID[pot]
        nk = len(H["kinds"])
        mass = np.array([m / MD_MASS_UNIT for _, m, _ in H["kinds"]])
        elem = np.array([e for _, _, e in H["kinds"]], np.int32)
        table = (Pair * (nk * nk))()
        for (a, b), (cat, p) in H["pairs"].items():
            for i, j in ((a, b), (b, a)):
                t = table[i * nk + j]
                t.cat = cat
                t.iloc, t.jloc = (int(elem[i]), int(elem[j])) if cat == FMDG_POT_EAM else (0, 0)
                for q in range(4):
                    t.p[q] = p[q]
        return mass, elem, table
    P = POTENTIALS[pot]
    mass = np.array([P["mass"] / MD_MASS_UNIT])
    elem = np.array([0 if P["cat"] == FMDG_POT_EAM else -1], np.int32)
    table = (Pair * 1)()
    table[0].cat = P["cat"]
    for q in range(4):
        table[0].p[q] = P["p"][q]
    return mass, elem, table


def job_rc(pot):
    return HYBRID[pot]["rc"] if pot in HYBRID else POTENTIALS[pot]["rc"]


def job_dt(pot):
    return HYBRID[pot]["dt"] if pot in HYBRID else POTENTIALS[pot]["dt"]


def hybrid_atoms(job):
    """A "cuar" job: an n^3-cell copper FCC block (a = 3.615 A) at the
    origin and an argon FCC block of m^3 cells (m = round(n a / 5.26), its
    lattice stretched to the copper block's width) 2 A beyond it along x;
    periodic box (2 n a + 4, n a, n a).  Returns x, v, kind, l[3]."""
    n = job["ncell"]
    lc = n * 3.615
    m = max(1, int(round(lc / 5.26)))
    aa = lc / m
    xc, vc = workloads.fcc_state(n, n, n, 3.615, job["T"], 63.546, seed=job["seed"])
    xa, va = workloads.fcc_state(m, m, m, aa, job["T"], 39.948, seed=job["seed"] + 1, origin=(lc + 2.0, 0.0, 0.0))
    x = np.concatenate([xc, xa])
    v = np.concatenate([vc, va])
    kind = np.concatenate([np.zeros(len(xc), np.uint32), np.ones(len(xa), np.uint32)])
    return x, v, kind, np.array([2.0 * lc + 4.0, lc, lc])


def eam_tables(L):
    """Tables of the analytic EAM as the setfl loader of libfmd builds them
    (src/eam.c:376-555 restated in fmd_pot.c)."""
    with tempfile.TemporaryDirectory() as work:
        path = workloads.write_analytic_eam(os.path.join(work, "analytic.eam.alloy"))
        md = L.fmd_create()
        L.fmd_io_setShowErrorMessages(md, False)
        pot = L.fmd_pot_eam_alloy_load(md, path.encode())
        if not pot:
            L.fmd_free(md)
            raise EngineError("EAM load failed")
        ne, nrho, nr2 = C.c_int(), C.c_int(), C.c_int()
        drho, dr2, rc2 = C.c_double(), C.c_double(), C.c_double()
        L.fmdx_eam_tables(pot, C.byref(ne), C.byref(nrho), C.byref(drho), C.byref(nr2), C.byref(dr2),
                          C.byref(rc2), None, None, None, None, None, None)
        t = dict(nelem=ne.value, Nrho=nrho.value, drho=drho.value, Nr2=nr2.value, dr2=dr2.value,
                 cutoff_sqr=rc2.value)
        F = np.zeros(ne.value * nrho.value)
        FDD = np.zeros_like(F)
        rho = np.zeros(ne.value * nr2.value)
        rhoDD = np.zeros_like(rho)
        phi = np.zeros(ne.value * ne.value * nr2.value)
        phiDD = np.zeros_like(phi)
        L.fmdx_eam_tables(pot, C.byref(ne), C.byref(nrho), C.byref(drho), C.byref(nr2), C.byref(dr2),
                          C.byref(rc2), _dp(F), _dp(FDD), _dp(rho), _dp(rhoDD), _dp(phi), _dp(phiDD))
        L.fmd_free(md)
    t.update(F=F, F_DD=FDD, rho=rho, rhoDD=rhoDD, phi=phi, phiDD=phiDD)
    return t


# ------------------------------------------------------------------ job stream
def served_stream(njobs=2048, seed=5, rate=50.0, nmin=500, nmax=200000, steps=(1000, 20000),
                  step_scale=1.0, pots=POT_NAMES):
    """Job descriptions of the served stream (no atoms yet: `job_atoms`).
    step_scale < 1 shortens every job and compresses the arrival times by
    the same factor, so the offered load relative to the device's capacity
    stays that of the full stream."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, njobs)) * step_scale
    N = np.exp(rng.uniform(math.log(nmin), math.log(nmax), njobs))
    pot = rng.integers(0, len(pots), njobs)
    T = rng.uniform(50.0, 1200.0, njobs)
    st = rng.integers(steps[0], steps[1] + 1, njobs)
    jobs = []
    for k in range(njobs):
        n = max(1, int(round((N[k] / 4.0) ** (1.0 / 3.0))))
        name = pots[pot[k]]
        jobs.append(dict(index=k, arrival=float(arrivals[k]), ncell=n, natoms=4 * n ** 3, pot=name,
                         T=float(T[k]), steps=max(1, int(round(st[k] * step_scale))),
                         dt=POTENTIALS[name]["dt"], seed=seed * 1000003 + k))
    return jobs


def job_atoms(job):
    """Positions (inside [0, l)) and velocities of a job's FCC cube."""
    P = POTENTIALS[job["pot"]]
    n = job["ncell"]
    x, v = workloads.fcc_state(n, n, n, P["a"], job["T"], P["mass"], seed=job["seed"])
    return x, v, n * P["a"]


class Server:
    """A served-mode instance on one device."""

    def __init__(self, L, device=0, budget_bytes=64 << 30, max_jobs=1024, chunk_steps=16, eam=None):
        self.L = L
        h = C.c_void_p()
        check(L, L.fmdg_srv_create(C.byref(h), device, budget_bytes, max_jobs, chunk_steps), "fmdg_srv_create")
        self.h = h
        self._keep = {}
        self._skin = None        # set_skin: every job's skin, else per potential
        self._capacity = None    # set_list_capacity: every job's, else per potential
        if eam is not None:
            self.set_eam(0, eam)

    def close(self):
        if self.h:
            self.L.fmdg_srv_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_eam(self, key, t):
        check(self.L, self.L.fmdg_srv_set_eam(self.h, key, t["nelem"], t["Nrho"], t["drho"], t["Nr2"], t["dr2"],
                                              _dp(t["F"]), _dp(t["F_DD"]), _dp(t["rho"]), _dp(t["rhoDD"]),
                                              _dp(t["phi"]), _dp(t["phiDD"])), "fmdg_srv_set_eam")

    def set_tuning(self, fblk):
        check(self.L, self.L.fmdg_srv_set_tuning(self.h, fblk), "fmdg_srv_set_tuning")

    def set_skin(self, skin):
        """Skin of every job submitted from now on (instead of the
        per-potential defaults)."""
        check(self.L, self.L.fmdg_srv_set_skin(self.h, skin), "fmdg_srv_set_skin")
        self._skin = skin

    def set_list_capacity(self, entries):
        """List capacity of every job submitted from now on (instead of the
        per-potential defaults; 0: estimated per job)."""
        check(self.L, self.L.fmdg_srv_set_list_capacity(self.h, entries), "fmdg_srv_set_list_capacity")
        self._capacity = entries

    def _job_list(self, pot):
        """Skin and list capacity for a job: what set_skin / set_list_capacity
        chose, else the potential's serving defaults (POTENTIALS; hybrid
        jobs: skin 0.8, estimated capacity)."""
        P = POTENTIALS.get(pot, {})
        skin = P.get("skin", 0.8) if self._skin is None else self._skin
        cap = P.get("list_capacity", 0) if self._capacity is None else self._capacity
        check(self.L, self.L.fmdg_srv_set_skin(self.h, skin), "fmdg_srv_set_skin")
        check(self.L, self.L.fmdg_srv_set_list_capacity(self.h, cap), "fmdg_srv_set_list_capacity")

    def submit(self, pot, x, v, l, steps, precision=PREC_MIXED, keep_state=False, dt=None, kind=None):
        """Queue a job of type `pot` (POTENTIALS or HYBRID); `l` a cube edge
        or three box lengths; `kind` per atom (default all 0)."""
        self._job_list(pot)
        x = np.ascontiguousarray(x, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        n = len(x)
        kind = np.zeros(n, np.uint32) if kind is None else np.ascontiguousarray(kind, np.uint32)
        mass, elem, pair = job_table(pot)
        l3 = np.broadcast_to(np.asarray(l, np.float64), (3,))
        d = JobDesc()
        for q in range(3):
            d.l[q] = l3[q]
            d.pbc[q] = 1
        d.nkinds = len(mass)
        d.mass = _dp(mass)
        d.eam_elem = elem.ctypes.data_as(C.POINTER(C.c_int))
        d.pairs = pair
        d.eam_key = 0
        d.n = n
        d.x = _dp(x)
        d.v = _dp(v)
        d.kind = kind.ctypes.data_as(C.POINTER(C.c_uint))
        d.steps = int(steps)
        d.dt = job_dt(pot) if dt is None else dt
        d.precision = precision
        d.keep_state = 1 if keep_state else 0
        jid = C.c_longlong()
        check(self.L, self.L.fmdg_srv_submit(self.h, C.byref(d), C.byref(jid)), "fmdg_srv_submit")
        return jid.value

    def progress(self, wait=True):
        a = C.c_int()
        check(self.L, self.L.fmdg_srv_progress(self.h, 1 if wait else 0, C.byref(a)), "fmdg_srv_progress")
        return a.value

    def now(self):
        t = C.c_double()
        self.L.fmdg_srv_now(self.h, C.byref(t))
        return t.value

    def result(self, jid):
        r = JobResult()
        check(self.L, self.L.fmdg_srv_result(self.h, jid, C.byref(r)), "fmdg_srv_result")
        return r

    def state(self, jid, n):
        x, v, F = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        ids = np.zeros(n, np.uint32)
        check(self.L, self.L.fmdg_srv_state(self.h, jid, _dp(x), _dp(v), _dp(F),
                                            ids.ctypes.data_as(C.POINTER(C.c_uint))), "fmdg_srv_state")
        return x, v, F, ids

    def release(self, jid):
        check(self.L, self.L.fmdg_srv_release(self.h, jid), "fmdg_srv_release")

    def stats(self):
        s = SrvStats()
        check(self.L, self.L.fmdg_srv_stats(self.h, C.byref(s)), "fmdg_srv_stats")
        return s

    def admit(self):
        check(self.L, self.L.fmdg_srv_admit(self.h), "fmdg_srv_admit")

    def run_resident(self, k):
        ms = C.c_float()
        check(self.L, self.L.fmdg_srv_run_resident(self.h, k, C.byref(ms)), "fmdg_srv_run_resident")
        return ms.value

    def profile_pack(self, pot, precision=PREC_MIXED):
        ms = (C.c_float * 4)()
        atoms, members = C.c_double(), C.c_int()
        cls = 0 if pot in HYBRID else POTENTIALS[pot]["cat"]
        check(self.L, self.L.fmdg_srv_profile_pack(self.h, cls, precision, ms, C.byref(atoms),
                                                   C.byref(members)), "fmdg_srv_profile_pack")
        return list(ms), atoms.value, members.value

    def drain(self):
        while self.progress(wait=True) > 0:
            pass


def host_binning3(x, l, rc):
    """Cell grid and upload order the served mode uses, per axis:
    nc = (int)(l/rc), cellh = l/nc (src/misc.c:41-50), atoms in input order
    inside a cell.  Returns nc[3], cellh[3], order, counts."""
    l = np.broadcast_to(np.asarray(l, np.float64), (3,))
    nc = np.maximum(1, (l / rc).astype(np.int64))
    cellh = l / nc
    ic = np.floor(x / cellh).astype(np.int64)
    flat = ic[:, 2] + nc[2] * (ic[:, 1] + nc[1] * ic[:, 0])
    order = np.argsort(flat, kind="stable")
    counts = np.bincount(flat, minlength=int(nc.prod())).astype(np.int32)
    return nc, cellh, order, counts


def host_binning(x, l, rc):
    """host_binning3 of a cube of edge l: (nc, cellh) as scalars."""
    nc, cellh, order, counts = host_binning3(x, l, rc)
    return int(nc[0]), float(cellh[0]), order, counts


class Single:
    """One job on the plain single-system path of the device engine (the
    path libfmd.so's fmd_dync_integrate drives): its own system, steps
    replayed from one captured graph, no packing."""

    def __init__(self, L, pot, x, v, l, precision=PREC_FP64, eam=None, device=0, kind=None, list_capacity=0,
                 build_lanes=0):
        self.L = L
        h = C.c_void_p()
        check(L, L.fmdg_create(C.byref(h), device), "fmdg_create")
        self.h = h
        nc, cellh, order, counts = host_binning3(x, l, job_rc(pot))
        l3 = np.broadcast_to(np.asarray(l, np.float64), (3,))
        lv = (C.c_double * 3)(*l3)
        pbc = (C.c_int * 3)(1, 1, 1)
        ncv = (C.c_int * 3)(*[int(c) for c in nc])
        ch = (C.c_double * 3)(*cellh)
        check(L, L.fmdg_set_box(h, lv, pbc, ncv, ch), "set_box")
        mass, elem, pair = job_table(pot)
        check(L, L.fmdg_set_kinds(h, len(mass), _dp(mass), elem.ctypes.data_as(C.POINTER(C.c_int))), "set_kinds")
        check(L, L.fmdg_set_pairs(h, pair), "set_pairs")
        if (elem >= 0).any():
            t = eam
            check(L, L.fmdg_set_eam(h, t["nelem"], t["Nrho"], t["drho"], t["Nr2"], t["dr2"], _dp(t["F"]),
                                    _dp(t["F_DD"]), _dp(t["rho"]), _dp(t["rhoDD"]), _dp(t["phi"]),
                                    _dp(t["phiDD"])), "set_eam")
        check(L, L.fmdg_set_precision(h, precision), "set_precision")
        check(L, L.fmdg_set_list_capacity(h, list_capacity), "set_list_capacity")
        check(L, L.fmdg_set_build_lanes(h, build_lanes), "set_build_lanes")
        n = len(x)
        xs = np.ascontiguousarray(x[order])
        vs = np.ascontiguousarray(v[order])
        kind = (np.zeros(n, np.uint32) if kind is None else np.asarray(kind, np.uint32))[order]
        kind = np.ascontiguousarray(kind)
        group = np.zeros(n, np.int32)
        ids = order.astype(np.uint32)
        check(L, L.fmdg_upload(h, n, counts.ctypes.data_as(C.POINTER(C.c_int)), _dp(xs), _dp(vs),
                               kind.ctypes.data_as(C.POINTER(C.c_uint)), group.ctypes.data_as(C.POINTER(C.c_int)),
                               ids.ctypes.data_as(C.POINTER(C.c_uint))), "upload")
        check(L, L.fmdg_compute_forces(h, -1), "forces")
        self.th0 = Thermo()
        check(L, L.fmdg_thermo(h, -1, C.byref(self.th0)), "thermo")
        self.n = n
        self.dt = job_dt(pot)

    def steps(self, k, dt=None):
        check(self.L, self.L.fmdg_vv_steps(self.h, k, self.dt if dt is None else dt, -1, 0, 1.0, 0.0), "vv_steps")

    def thermo(self):
        t = Thermo()
        check(self.L, self.L.fmdg_get_thermo(self.h, C.byref(t)), "get_thermo")
        return t

    def state(self):
        n = C.c_int()
        self.L.fmdg_natoms(self.h, C.byref(n))
        x, v, F = np.zeros((n.value, 3)), np.zeros((n.value, 3)), np.zeros((n.value, 3))
        ids = np.zeros(n.value, np.uint32)
        check(self.L, self.L.fmdg_download(self.h, None, _dp(x), _dp(v), _dp(F), None, None, None,
                                           ids.ctypes.data_as(C.POINTER(C.c_uint))), "download")
        return x, v, F, ids

    def close(self):
        if self.h:
            self.L.fmdg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
