"""ctypes wrapper of the CPU oracle (oracle/fmd_oracle.c) -- test
infrastructure: used by tests/, __graft_entry__.smoke() and bench.py's CPU
baseline only.  The oracle is built by `oracle/build.py` (build_oracle).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
MASS_UNIT = 9.6485332907e+03

P = C.c_void_p


class PairT(C.Structure):
    _fields_ = [("cat", C.c_int), ("iloc", C.c_int), ("jloc", C.c_int), ("pad", C.c_int), ("p", C.c_double * 4)]


class TtmParamsT(C.Structure):
    """oracle_ttm_params_t"""
    _fields_ = [("type", C.c_int), ("ratio", C.c_int), ("min_atoms", C.c_uint), ("nC", C.c_int), ("nG", C.c_int),
                ("C_gamma", C.c_double), ("K", C.c_double), ("G", C.c_double), ("dz2", C.c_double),
                ("frontsurf", C.c_double), ("laser_t0", C.c_double), ("laser_tdiff", C.c_double),
                ("laser_m_2sig2_inv", C.c_double), ("laser_m_absdepth_inv", C.c_double),
                ("laser_factor", C.c_double), ("Kzh_v2", C.c_double), ("Kzh_A", C.c_double), ("Kzh_B", C.c_double),
                ("T_C", P), ("Ct", P), ("C_DD", P), ("T_G", P), ("Gt", P), ("G_DD", P)]


class ThermoT(C.Structure):
    _fields_ = [("kinetic", C.c_double), ("temperature", C.c_double), ("momentum", C.c_double * 3),
                ("potential", C.c_double), ("count", C.c_double), ("virial", C.c_double)]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(P)


def _lib():
    if not os.path.exists(LIB):
        import importlib.util
        spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build.py"))
        ob = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(ob)
        ob.build_oracle()
    L = C.CDLL(LIB)
    L.oracle_create.restype = P
    for name, args in [("oracle_destroy", [P]), ("oracle_set_threads", [P, C.c_int]),
                       ("oracle_set_box", [P, P, P, P, P]), ("oracle_set_kinds", [P, C.c_int, P, P]),
                       ("oracle_set_pairs", [P, P]),
                       ("oracle_load_setfl", [P, C.c_char_p, C.c_char_p, C.c_int, P]),
                       ("oracle_eam_table", [P, C.c_int, C.c_int, P, P]),
                       ("oracle_upload", [P, C.c_int, P, P, P, P, P, P]), ("oracle_natoms", [P]),
                       ("oracle_download", [P, P, P, P, P, P, P, P, P]), ("oracle_set_state", [P, P, P]),
                       ("oracle_refresh", [P]), ("oracle_compute_forces", [P, C.c_int]),
                       ("oracle_thermo", [P, C.c_int, P]),
                       ("oracle_vv_steps", [P, C.c_int, C.c_double, C.c_int, C.c_int, C.c_double, C.c_double]),
                       ("oracle_get_thermo", [P, P]), ("oracle_errors", [P]),
                       ("oracle_ttm_setup", [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                             C.c_double, C.c_double, P, C.c_double]),
                       ("oracle_set_time", [P, C.c_double, C.c_double]), ("oracle_turi_update", [P]),
                       ("oracle_se_steps", [P, C.c_int, C.c_double, C.c_int]),
                       ("oracle_ttm_1d", [P, P, P, P, P, P])]:
        f = getattr(L, name)
        f.argtypes = args
        f.restype = C.c_uint if name == "oracle_errors" else (None if name == "oracle_destroy" else C.c_int)
    return L


class Oracle:
    """One system of the CPU restatement."""

    def __init__(self, threads: int = 1):
        self.L = _lib()
        self.o = C.c_void_p(self.L.oracle_create())
        self.L.oracle_set_threads(self.o, threads)

    def set_threads(self, threads: int):
        self.L.oracle_set_threads(self.o, threads)

    def close(self):
        if self.o:
            self.L.oracle_destroy(self.o)
            self.o = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setup(self, box, pbc, nc, cellh, kinds, pots, setfl=None):
        """kinds: [(name, mass_amu)]; pots: tuples as in tests/cases.py:
        ("lj", k1, k2, sigma, eps, rc), ("morse", k1, k2, D0, alpha, r0, rc),
        ("eam", k1, k2) (uses `setfl`)."""
        l = np.ascontiguousarray(box, dtype=np.float64)
        self.L.oracle_set_box(self.o, _ptr(l), _ptr(np.ascontiguousarray(pbc, dtype=np.int32)),
                              _ptr(np.ascontiguousarray(nc, dtype=np.int32)), _ptr(np.ascontiguousarray(cellh, dtype=np.float64)))
        nk = len(kinds)
        elem = -np.ones(nk, np.int32)
        enames = []
        eam_rc = None
        if setfl is not None:
            buf = C.create_string_buffer(1024)
            rc = C.c_double(0)
            ne = self.L.oracle_load_setfl(self.o, setfl.encode(), buf, 1024, C.byref(rc))
            assert ne > 0, ne
            enames = buf.value.decode().split()
            eam_rc = rc.value
        table = (PairT * (nk * nk))()
        for p in pots:
            k1, k2 = p[1], p[2]
            for a, b in ((k1, k2), (k2, k1)):
                t = table[a * nk + b]
                if p[0] == "lj":
                    t.cat = 1
                    t.p[0], t.p[1], t.p[2] = 4.0 * p[4], p[3] * p[3], p[5] * p[5]
                elif p[0] == "morse":
                    t.cat = 3
                    t.p[0], t.p[1], t.p[2], t.p[3] = p[3], p[4], p[5], p[6] * p[6]
                else:
                    t.cat = 2
                    t.p[2] = eam_rc * eam_rc
                    t.iloc = enames.index(kinds[a][0])
                    t.jloc = enames.index(kinds[b][0])
                    elem[a] = t.iloc
                    elem[b] = t.jloc
        mass = np.array([m / MASS_UNIT for _, m in kinds])
        self.L.oracle_set_kinds(self.o, nk, _ptr(mass), _ptr(elem))
        self.L.oracle_set_pairs(self.o, C.cast(table, P))

    def upload(self, cell, x, v, kind, group, atomid, ncell):
        counts = np.bincount(np.asarray(cell), minlength=ncell).astype(np.int32)
        x = np.ascontiguousarray(x, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        kind = np.ascontiguousarray(kind, np.uint32)
        group = np.ascontiguousarray(group, np.int32)
        atomid = np.ascontiguousarray(atomid, np.uint32)
        rc = self.L.oracle_upload(self.o, len(kind), _ptr(counts), _ptr(x), _ptr(v), _ptr(kind), _ptr(group),
                                  _ptr(atomid))
        assert rc == 0

    def dump(self):
        n = self.L.oracle_natoms(self.o)
        out = dict(cell=np.zeros(n, np.int32), id=np.zeros(n, np.uint32), kind=np.zeros(n, np.uint32),
                   group=np.zeros(n, np.int32), x=np.zeros((n, 3)), v=np.zeros((n, 3)), F=np.zeros((n, 3)),
                   vaream=np.zeros(n))
        self.L.oracle_download(self.o, _ptr(out["cell"]), _ptr(out["x"]), _ptr(out["v"]), _ptr(out["F"]),
                               _ptr(out["vaream"]), _ptr(out["kind"]), _ptr(out["group"]), _ptr(out["id"]))
        th = ThermoT()
        self.L.oracle_get_thermo(self.o, C.byref(th))
        out["pe"] = th.potential
        out["virial"] = th.virial
        return out

    def set_state(self, x=None, v=None):
        x = None if x is None else np.ascontiguousarray(x, np.float64)
        v = None if v is None else np.ascontiguousarray(v, np.float64)
        self.L.oracle_set_state(self.o, _ptr(x), _ptr(v))

    def refresh(self):
        return self.L.oracle_refresh(self.o)

    def forces(self, group=-1):
        self.L.oracle_compute_forces(self.o, group)

    def thermo(self, group=-1):
        th = ThermoT()
        self.L.oracle_thermo(self.o, group, C.byref(th))
        return th

    def get_thermo(self):
        th = ThermoT()
        self.L.oracle_get_thermo(self.o, C.byref(th))
        return th

    def vv(self, nsteps, dt, group=-1, thermostat=0, tau=1.0, T0=0.0):
        return self.L.oracle_vv_steps(self.o, nsteps, dt, group, thermostat, tau, T0)

    def errors(self):
        return self.L.oracle_errors(self.o)

    # ---- 1-D two-temperature model --------------------------------------
    def ttm_setup(self, pd, pk, Te_init, tables=None):
        """The reference's derived TTM parameters as a golden file records
        them (tests/golden/make_golden.py ttm_params): pd = C_gamma, K, G,
        dz2, frontsurf, laser_t0, laser_tdiff, laser_m_2sig2_inv,
        laser_m_absdepth_inv, laser_factor, Kzh v2, A, B, tcell_volume,
        starttime, stoptime, tcellh_z; pk = type, ratio, min_atoms, nC, nG,
        itc_start, itc_stop, nz, itc_glob_to_loc (z)."""
        q = TtmParamsT()
        q.type, q.ratio, q.min_atoms = int(pk[0]), int(pk[1]), int(pk[2])
        (q.C_gamma, q.K, q.G, q.dz2, q.frontsurf, q.laser_t0, q.laser_tdiff, q.laser_m_2sig2_inv,
         q.laser_m_absdepth_inv, q.laser_factor, q.Kzh_v2, q.Kzh_A, q.Kzh_B) = [float(v) for v in pd[:13]]
        keep = []
        if q.type == 2:
            q.nC, q.nG = int(pk[3]), int(pk[4])
            for name in ("T_C", "Ct", "C_DD", "T_G", "Gt", "G_DD"):
                a = np.ascontiguousarray(tables[name], dtype=np.float64)
                keep.append(a)
                setattr(q, name, _ptr(a))
        rc = self.L.oracle_ttm_setup(self.o, int(pk[7]), int(pk[8]), int(pk[5]), int(pk[6]), float(pd[16]),
                                     float(pd[13]), float(pd[14]), float(pd[15]), C.byref(q), float(Te_init))
        assert rc == 0, rc

    def set_time(self, time, dt):
        self.L.oracle_set_time(self.o, time, dt)

    def turi_update(self):
        self.L.oracle_turi_update(self.o)

    def se_steps(self, nsteps, dt, group=-1):
        assert self.L.oracle_se_steps(self.o, nsteps, dt, group) == 0

    def ttm_1d(self, nmax=4096):
        num = np.zeros(nmax, np.uint32)
        vcm = np.zeros((nmax, 3))
        Ti, Te, xi = np.zeros(nmax), np.zeros(nmax), np.zeros(nmax)
        n = self.L.oracle_ttm_1d(self.o, _ptr(num), _ptr(vcm), _ptr(Ti), _ptr(Te), _ptr(xi))
        assert n > 0, n
        return dict(num=num[:n].copy(), vcm=vcm[:n].copy(), Ti=Ti[:n].copy(), Te=Te[:n].copy(), xi=xi[:n].copy())


# unit factors of the reference (src/general.h:38-45)
_METER, _SECOND = 1e10, 1e12
_J_M3_K2, _W_M_K, _W_M2, _W_M3_K = 6.2415091259e-12, 6.2415091259e-4, 6.2415091259e-14, 6.2415091259e-24
_K_B = 8.6173303e-5


def ttm1_params(box, tdims_z, x, gamma, K, G, laser, frac, ratio, start=0.0, stop=-1.0):
    """The derived parameters of a 1-D type-1 TTM turi of tdims_z cells
    along z on a single domain, as the reference forms them from its
    fmd.h-level inputs, in the (pd, pk) layout of the golden files:
    turi geometry (src/turi.c:670-708: one margin cell each side, tcellh =
    l / tdims), heat capacity gamma Te, constant K and G
    (src/ttm.c setters, units src/general.h:38-45), the Gaussian pulse
    (src/ttm.c:794-816: laser = fluence, reflectance, t0, duration,
    absorption depth in SI units), and the front surface and activation
    threshold from the atoms' extent (src/ttm.c:63-80: frontsurf = lowest z,
    initial atoms per cell = N / V_extent * V_cell, threshold = that x
    frac)."""
    import math
    tcellh = [box[0] / 1, box[1] / 1, box[2] / tdims_z]
    vol_cell = tcellh[0] * tcellh[1] * tcellh[2]
    fluence, R, t0, duration, depth = laser
    Lp = depth * _METER
    I0 = math.sqrt(4 * math.log(2) / math.pi) * fluence / duration * _W_M2
    sigma = duration / math.sqrt(8 * math.log(2)) * _SECOND
    x = np.asarray(x, dtype=np.float64)
    ll, ul = x.min(axis=0), x.max(axis=0)
    vol = 1.0
    for d in range(3):
        vol *= ul[d] - ll[d]
    initial = int(len(x) / vol * vol_cell)
    pd = np.array([gamma * _J_M3_K2, K * _W_M_K, G * _W_M3_K, tcellh[2] * tcellh[2], ll[2], t0 * _SECOND,
                   4 * math.sqrt(2) * sigma, -0.5 / (sigma * sigma), -1. / Lp, I0 * (1 - R) / Lp, 0.0, 0.0, 0.0,
                   vol_cell, start, stop, tcellh[2]])
    pk = np.array([1, ratio, int(initial * frac), 0, 0, 1, 1 + tdims_z, tdims_z + 2, 1], dtype=np.int64)
    return pd, pk
