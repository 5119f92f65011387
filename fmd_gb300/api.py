"""ctypes binding of the FMD public C API (the `fmd.h` interface).

The same binding drives any shared library that exports the `fmd.h` symbols:
this package's GPU library (`libfmd.so`, the product) and, in tests only, the
reference library compiled as a CPU oracle.  Prototypes follow the reference
header src/fmd.h:157-263; TTM setters bind the `_fmd_ttm_*` targets of the
`_Generic` macros (src/fmd.h:240-255).

Library-specific white-box helpers (per-atom dumps) are bound by
`Lib.bind_dump()`; the product exports them as `fmdx_*` and the oracle as
`oref_*`, with identical signatures.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

D = C.c_double
P = C.c_void_p

FMD_GROUP_ALL = -1

# enum fmd_event_t (src/fmd.h:38-43)
FMD_EVENT_TIMER_TICK, FMD_EVENT_FIELD_UPDATE, FMD_EVENT_ERROR = 0, 1, 2
# enum fmd_turi_t (src/fmd.h:45-50)
FMD_TURI_CUSTOM, FMD_TURI_TTM_TYPE1, FMD_TURI_TTM_TYPE2 = 0, 1, 2
# enum fmd_field_t (src/fmd.h:52-61)
(FMD_FIELD_MASS, FMD_FIELD_VCM, FMD_FIELD_TEMPERATURE, FMD_FIELD_NUMBER,
 FMD_FIELD_NUMBER_DENSITY, FMD_FIELD_TTM_TE, FMD_FIELD_TTM_XI) = range(7)
# enum fmd_SaveConfigMode_t (src/fmd.h:30-36)
FMD_SCM_XYZ_ATOMSNUM, FMD_SCM_XYZ_SEPARATE, FMD_SCM_CSV, FMD_SCM_VTF = range(4)


class ErrorParams(C.Structure):
    """fmd_event_params_error_t (src/fmd.h:101-111)."""
    _fields_ = [("error", C.c_int), ("major", C.c_bool), ("source", C.c_char_p),
                ("func", C.c_char_p), ("line", C.c_int), ("p1", P), ("p2", P), ("p3", P)]


class TimerTickParams(C.Structure):
    _fields_ = [("timer", C.c_int)]


class FieldUpdateParams(C.Structure):
    _fields_ = [("turi", C.c_int), ("field", C.c_int)]


class HeatCapacityLinear(C.Structure):
    _fields_ = [("gamma", D)]


class HeatConductivityConstant(C.Structure):
    _fields_ = [("value", D)]


class HeatConductivityZhigilei(C.Structure):
    _fields_ = [("v", D), ("A", D), ("B", D)]


class CouplingFactorConstant(C.Structure):
    _fields_ = [("value", D)]


class LaserGaussian(C.Structure):
    _fields_ = [("fluence", D), ("reflectance", D), ("t0", D), ("duration", D),
                ("AbsorptionDepth", D)]


EventHandler = C.CFUNCTYPE(None, P, C.c_int, P, P)

_PROTOS = {
    "fmd_create": (P, []),
    "fmd_free": (None, [P]),
    "fmd_setEventHandler": (None, [P, P, EventHandler]),
    "fmd_box_setPBC": (None, [P, C.c_bool, C.c_bool, C.c_bool]),
    "fmd_box_setSize": (None, [P, D, D, D]),
    "fmd_box_setSubdomains": (C.c_bool, [P, C.c_int, C.c_int, C.c_int]),
    "fmd_matt_setAtomKinds": (None, [P, C.c_uint, P, P]),
    "fmd_matt_makeCuboidSC": (None, [P, D, D, D, C.c_int, C.c_int, C.c_int, D, C.c_uint, C.c_int, D]),
    "fmd_matt_makeCuboidBCC": (None, [P, D, D, D, C.c_int, C.c_int, C.c_int, D, C.c_uint, C.c_int, D]),
    "fmd_matt_makeCuboidFCC": (None, [P, D, D, D, C.c_int, C.c_int, C.c_int, D, C.c_uint, C.c_int, D]),
    "fmd_matt_makeCuboidSC_mix": (None, [P, D, D, D, C.c_int, C.c_int, C.c_int, D, P, C.c_int, D]),
    "fmd_matt_makeCuboidBCC_mix": (None, [P, D, D, D, C.c_int, C.c_int, C.c_int, D, P, C.c_int, D]),
    "fmd_matt_makeCuboidFCC_mix": (None, [P, D, D, D, C.c_int, C.c_int, C.c_int, D, P, C.c_int, D]),
    "fmd_matt_addVelocity": (None, [P, C.c_int, D, D, D]),
    "fmd_matt_translate": (None, [P, C.c_int, D, D, D]),
    "fmd_matt_saveConfiguration": (None, [P]),
    "fmd_matt_getKineticEnergy": (D, [P]),
    "fmd_matt_getTotalEnergy": (D, [P]),
    "fmd_matt_getTemperature": (D, [P]),
    "fmd_matt_getMomentum": (None, [P, P]),
    "fmd_matt_giveMaxwellDistribution": (None, [P, C.c_int, D]),
    "fmd_matt_findLimits": (None, [P, C.c_int, P, P]),
    "fmd_matt_changeGroupID": (None, [P, C.c_int, C.c_int]),
    "fmd_io_setSaveDirectory": (None, [P, C.c_char_p]),
    "fmd_io_setSaveConfigMode": (None, [P, C.c_int]),
    "fmd_io_loadState": (None, [P, C.c_char_p, C.c_bool]),
    "fmd_io_saveState": (None, [P, C.c_char_p]),
    "fmd_io_setShowErrorMessages": (None, [P, C.c_bool]),
    "fmd_pot_eam_alloy_load": (P, [P, C.c_char_p]),
    "fmd_pot_eam_getLatticeParameter": (D, [P, P, C.c_char_p]),
    "fmd_pot_eam_getCutoffRadius": (D, [P, P]),
    "fmd_pot_lj_apply": (P, [P, C.c_uint, C.c_uint, D, D, D]),
    "fmd_pot_morse_apply": (P, [P, C.c_uint, C.c_uint, D, D, D, D]),
    "fmd_pot_apply": (None, [P, C.c_uint, C.c_uint, P]),
    "fmd_timer_makeSimple": (C.c_int, [P, D, D, D]),
    "fmd_proc_getWallTime": (D, [P]),
    "fmd_proc_hasSubdomain": (C.c_bool, [P]),
    "fmd_proc_isRoot": (C.c_bool, [P]),
    "fmd_proc_setNumThreads": (None, [P, C.c_int]),
    "fmd_proc_getCellIncrement": (C.c_int, [P]),
    "fmd_proc_setCellIncrement": (None, [P, C.c_int]),
    "fmd_dync_getTimestep": (D, [P]),
    "fmd_dync_getTime": (D, [P]),
    "fmd_dync_equilibrate": (None, [P, C.c_int, D, D, D, D]),
    "fmd_dync_integrate": (None, [P, C.c_int, D, D]),
    "fmd_turi_add": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int, D, D]),
    "fmd_field_find": (C.c_int, [P, C.c_int, C.c_int]),
    "fmd_field_add": (C.c_int, [P, C.c_int, C.c_int, D]),
    "fmd_field_getArray": (P, [P, C.c_int, C.c_int, P, P]),
    "fmd_array3s_free": (None, [P]),
    "_fmd_ttm_setHeatCapacity_linear": (None, [P, C.c_int, HeatCapacityLinear]),
    "_fmd_ttm_setHeatCapacity_file": (None, [P, C.c_int, C.c_char_p]),
    "_fmd_ttm_setHeatConductivity_constant1": (None, [P, C.c_int, D]),
    "_fmd_ttm_setHeatConductivity_constant2": (None, [P, C.c_int, HeatConductivityConstant]),
    "_fmd_ttm_setHeatConductivity_zhigilei": (None, [P, C.c_int, HeatConductivityZhigilei]),
    "_fmd_ttm_setCouplingFactor_constant1": (None, [P, C.c_int, D]),
    "_fmd_ttm_setCouplingFactor_constant2": (None, [P, C.c_int, CouplingFactorConstant]),
    "_fmd_ttm_setCouplingFactor_file": (None, [P, C.c_int, C.c_char_p]),
    "fmd_ttm_setElectronTemperature": (None, [P, C.c_int, D]),
    "fmd_ttm_setTimestepRatio": (None, [P, C.c_int, C.c_int]),
    "fmd_ttm_setCellActivationFraction": (None, [P, C.c_int, D]),
    "_fmd_ttm_setLaserSource_gaussian": (None, [P, C.c_int, LaserGaussian]),
    "fmd_version_getMajor": (C.c_int, []),
    "fmd_version_getMinor": (C.c_int, []),
    "fmd_version_getRevision": (C.c_int, []),
    "fmd_version_getType": (C.c_char, []),
    "fmd_version_getString": (C.c_void_p, []),
}

# white-box per-atom helpers: (suffix, restype, argtypes)
_DUMP_PROTOS = {
    "natoms": (C.c_int, [P]),
    "dump": (C.c_int, [P, P, P, P, P, P, P, P, P]),
    "set_state": (None, [P, P, P]),
    "refresh": (None, [P]),
    "update_forces": (None, [P]),
    "potential_energy": (D, [P]),
    "virial": (D, [P]),
    "grid": (None, [P, P, P, P, P]),
    "ttm_1d": (C.c_int, [P, P, P, P, P, P]),
}


def _ptr(a):
    return None if a is None else a.ctypes.data_as(P)


class Lib:
    """A loaded library exporting the fmd.h API.  `prefix` selects the
    white-box helper family ('fmdx_' for the product, 'oref_' for the oracle)."""

    def __init__(self, path: str, prefix: str = "fmdx_"):
        self.path = os.path.abspath(path)
        self.L = C.CDLL(self.path)
        self.prefix = prefix
        for name, (res, args) in _PROTOS.items():
            f = getattr(self.L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        for suf, (res, args) in _DUMP_PROTOS.items():
            f = getattr(self.L, prefix + suf, None)
            if f is not None:
                f.restype = res
                f.argtypes = args

    def __getattr__(self, name):
        return getattr(self.L, name)

    def has(self, name: str) -> bool:
        return hasattr(self.L, name)

    # ---- white-box helpers --------------------------------------------------
    def wb(self, suf):
        return getattr(self.L, self.prefix + suf)

    def dump(self, md) -> dict:
        """Per-atom state in cell-storage order."""
        n = self.wb("natoms")(md)
        out = dict(cell=np.zeros(n, np.int32), id=np.zeros(n, np.uint32),
                   kind=np.zeros(n, np.uint32), group=np.zeros(n, np.int32),
                   x=np.zeros((n, 3)), v=np.zeros((n, 3)), F=np.zeros((n, 3)),
                   vaream=np.zeros(n))
        k = self.wb("dump")(md, _ptr(out["cell"]), _ptr(out["id"]), _ptr(out["kind"]),
                            _ptr(out["group"]), _ptr(out["x"]), _ptr(out["v"]),
                            _ptr(out["F"]), _ptr(out["vaream"]))
        assert k == n, (k, n)
        out["pe"] = self.wb("potential_energy")(md)
        if self.has(self.prefix + "virial"):
            out["virial"] = self.wb("virial")(md)
        return out

    def set_state(self, md, x=None, v=None):
        x = None if x is None else np.ascontiguousarray(x, dtype=np.float64)
        v = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        self.wb("set_state")(md, _ptr(x), _ptr(v))

    def grid(self, md):
        nc = np.zeros(3, np.int32)
        cellh = np.zeros(3)
        l = np.zeros(3)
        pbc = np.zeros(3, np.int32)
        self.wb("grid")(md, _ptr(nc), _ptr(cellh), _ptr(l), _ptr(pbc))
        return nc, cellh, l, pbc

    def ttm_1d(self, md, nmax=4096):
        num = np.zeros(nmax, np.uint32)
        vcm = np.zeros((nmax, 3))
        Ti = np.zeros(nmax)
        Te = np.zeros(nmax)
        xi = np.zeros(nmax)
        n = self.wb("ttm_1d")(md, _ptr(num), _ptr(vcm), _ptr(Ti), _ptr(Te), _ptr(xi))
        if n < 0:
            return None
        return dict(num=num[:n].copy(), vcm=vcm[:n].copy(), Ti=Ti[:n].copy(),
                    Te=Te[:n].copy(), xi=xi[:n].copy())


def set_atom_kinds(lib: Lib, md, names, masses):
    arr = (C.c_char_p * len(names))(*[n.encode() for n in names])
    m = (D * len(masses))(*masses)
    lib.fmd_matt_setAtomKinds(md, len(names), C.cast(arr, P), C.cast(m, P))


def write_state(path, time, l, pbc, names, kind, group, x, v):
    """State file in the reference's text format (src/misc.c:310-357):
    time, N, box, PBC flags, then per atom `name group` / x / v in %.16e."""
    with open(path, "w") as f:
        f.write("%.16e\n%u\n" % (time, len(kind)))
        f.write("%.16e\t%.16e\t%.16e\n" % tuple(l))
        f.write("%d %d %d\n" % tuple(int(b) for b in pbc))
        for i in range(len(kind)):
            f.write("%s %d\n" % (names[kind[i]], group[i]))
            f.write("%.16e\t%.16e\t%.16e\n" % tuple(x[i]))
            f.write("%.16e\t%.16e\t%.16e\n" % tuple(v[i]))
