"""Parity cases: small systems driven through the fmd.h API.

Each case is run identically through any library that exports fmd.h (the
reference oracle when golden vectors are generated, the GPU library in the
parity tests): create -> one subdomain -> box -> kinds -> potentials ->
`fmd_io_loadState` of a seeded state file -> integrate/equilibrate.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from fmd_gb300 import api, workloads

MASS = {"Ar": 39.948, "Cu": 63.546}


def _lj_state():
    x, v = workloads.fcc_state(10, 10, 10, 5.26, 100.0, MASS["Ar"], seed=1, disp=0.05)
    return dict(names=["Ar"], kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), x=x, v=v)


def _lj_small_state():
    x, v = workloads.fcc_state(4, 4, 4, 5.26, 80.0, MASS["Ar"], seed=11, disp=0.05)
    return dict(names=["Ar"], kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), x=x, v=v)


def _morse_state():
    rng = np.random.default_rng(3)
    x, v = workloads.fcc_state(6, 6, 4, 3.615, 300.0, MASS["Cu"], seed=3, origin=(0.0, 0.0, 10.0), disp=0.03)
    # escapers: atoms near the open faces moving outwards, and a fast projectile
    esc_x = np.array([[3.0, 4.0, 39.7], [15.0, 9.0, 39.8], [8.0, 18.0, 0.25], [19.0, 2.0, 0.3]])
    esc_v = np.array([[0.0, 0.0, 35.0], [1.0, -2.0, 30.0], [0.0, 0.0, -40.0], [3.0, 0.0, -33.0]])
    proj_x = workloads.fcc_sites(1, 1, 1, 3.615, origin=(9.0, 9.0, 28.0))
    proj_v = np.tile([0.0, 0.0, -60.0], (len(proj_x), 1)) + rng.standard_normal((len(proj_x), 3))
    # atoms that will cross the periodic x/y faces in the first steps
    cross_x = np.array([[0.05, 7.0, 20.0], [21.66, 12.0, 21.0], [11.0, 0.04, 19.5], [6.0, 21.67, 20.5]])
    cross_v = np.array([[-20.0, 0.0, 0.0], [25.0, 0.0, 0.0], [0.0, -22.0, 0.0], [0.0, 24.0, 0.0]])
    x = np.concatenate([x, esc_x, proj_x, cross_x])
    v = np.concatenate([v, esc_v, proj_v, cross_v])
    group = np.zeros(len(x), np.int32)
    return dict(names=["Cu"], kind=np.zeros(len(x), np.uint32), group=group, x=x, v=v)


def _eam_state():
    x, v = workloads.fcc_state(8, 8, 8, 3.615, 300.0, MASS["Cu"], seed=2, disp=0.04)
    return dict(names=["Cu"], kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), x=x, v=v)


def _hybrid_state():
    xc, vc = workloads.fcc_state(4, 4, 4, 3.615, 300.0, MASS["Cu"], seed=21, origin=(2.0, 8.0, 8.0), disp=0.03)
    xa, va = workloads.fcc_state(3, 3, 3, 5.26, 60.0, MASS["Ar"], seed=22, origin=(19.5, 8.0, 8.0), disp=0.03)
    va[:, 0] -= 5.0
    x = np.concatenate([xc, xa])
    v = np.concatenate([vc, va])
    kind = np.concatenate([np.zeros(len(xc), np.uint32), np.ones(len(xa), np.uint32)])
    group = np.concatenate([np.zeros(len(xc), np.int32), np.ones(len(xa), np.int32)])
    return dict(names=["Cu", "Ar"], kind=kind, group=group, x=x, v=v)


def _group_state():
    s = _lj_state()
    s["group"] = (np.arange(len(s["x"])) % 3 == 0).astype(np.int32)
    return s


def _ttm_state():
    x, v = workloads.fcc_state(6, 6, 16, 3.615, 300.0, MASS["Cu"], seed=41, origin=(0.0, 0.0, 8 * 3.615), disp=0.03)
    return dict(names=["Cu"], kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), x=x, v=v)


def _cu01_state():
    x, v = workloads.fcc_state(8, 8, 8, 3.615, 300.0, MASS["Cu"], seed=51, disp=0.04)
    return dict(names=["Cu"], kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), x=x, v=v)


LP_CU01 = 3.6316    # lattice parameter of the reference's type-2 TTM example (examples/04_ttm2.c:92)


def _ttm_cu_state():
    x, v = workloads.fcc_state(5, 5, 30, LP_CU01, 303.0, MASS["Cu"], seed=52, origin=(0.0, 0.0, 5 * LP_CU01),
                               disp=0.03)
    return dict(names=["Cu"], kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), x=x, v=v)


def _ttm_slab_state():
    x, v = workloads.fcc_state(4, 4, 100, 3.615, 300.0, MASS["Cu"], seed=4, origin=(0.0, 0.0, 20.0))
    return dict(names=["Cu"], kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), x=x, v=v)


def _ttm_slab_full_state():
    x, v = workloads.fcc_state(20, 20, 100, 3.615, 300.0, MASS["Cu"], seed=4, origin=(0.0, 0.0, 20.0))
    return dict(names=["Cu"], kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), x=x, v=v)


def _eam256k_state():
    x, v = workloads.fcc_state(40, 40, 40, 3.615, 300.0, MASS["Cu"], seed=2)
    return dict(names=["Cu"], kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), x=x, v=v)


def collision_atoms(seed=3):
    """The Morse collision configuration: an 80 x 80 x 20 FCC copper slab
    (300 K) and a projectile of the FCC sites within 20 A of a point 25 A
    above it, moving at -2 km/s along z; returns (box, x, v)."""
    a = 3.615
    lx = 80 * a
    x, v = workloads.fcc_state(80, 80, 20, a, 300.0, MASS["Cu"], seed=seed, origin=(0.0, 0.0, 2.0))
    top = 2.0 + 20 * a
    lz = 20 * a + 100.0
    c = np.array([lx / 2, lx / 2, top + 25.0])
    n = 13
    sph = workloads.fcc_sites(n, n, n, a, origin=tuple(c - n * a / 2))
    sph = sph[np.linalg.norm(sph - c, axis=1) <= 20.0]
    rng = np.random.default_rng(seed + 1)
    vs = workloads.maxwell_velocities(len(sph), MASS["Cu"], 300.0, rng)
    vs[:, 2] -= 20.0                      # -2 km/s (src/general.h:40: 1e-2 A/ps per m/s)
    return (lx, lx, lz), np.concatenate([x, sph]), np.concatenate([v, vs])


def _collision_state():
    _, x, v = collision_atoms()
    return dict(names=["Cu"], kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), x=x, v=v)


def _custom_state():
    x, v = workloads.fcc_state(8, 8, 8, 5.26, 90.0, MASS["Ar"], seed=42, disp=0.05)
    v[:, 2] += np.where(x[:, 0] < 21.04, 1.5, -1.5)
    return dict(names=["Ar"], kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), x=x, v=v)


def _fine_state():
    x, v = workloads.fcc_state(12, 12, 12, 5.26, 90.0, MASS["Ar"], seed=43, disp=0.05)
    v[:, 2] += np.where(x[:, 0] < 31.56, 1.5, -1.5)
    return dict(names=["Ar"], kind=np.zeros(len(x), np.uint32), group=np.zeros(len(x), np.int32), x=x, v=v)


def write_ttm_tables(work):
    """Synthetic type-2 tables (same two-column layout and units as the
    reference's table files: T in 1e4 K; C in 1e5 J/m^3K; G in 1e17 W/m^3K)."""
    T = np.linspace(0.0, 5.0, 201)                  # 0 .. 50 000 K
    C = 96.6 * (T * 1e4) / 1e5 * (1.0 / (1.0 + 0.05 * T))
    G = 1.0 + 0.3 * np.tanh(T - 1.0)
    pc = os.path.join(work, "Ce_syn.dat")
    pg = os.path.join(work, "G_syn.dat")
    np.savetxt(pc, np.stack([T, C], 1), fmt="%.10e")
    np.savetxt(pg, np.stack([T, G], 1), fmt="%.10e")
    return pc, pg


CASES = {
    "lj": dict(box=(52.6, 52.6, 52.6), pbc=(1, 1, 1), names=["Ar"],
               pots=[("lj", 0, 0, 3.405, 0.0104, 8.5125)], state=_lj_state,
               run=("integrate", -1, 0.002), steps=60, every=10),
    "lj_small": dict(box=(21.04, 21.04, 21.04), pbc=(1, 1, 1), names=["Ar"],
                     pots=[("lj", 0, 0, 3.405, 0.0104, 8.5125)], state=_lj_small_state,
                     run=("integrate", -1, 0.002), steps=60, every=10),
    "berendsen": dict(box=(52.6, 52.6, 52.6), pbc=(1, 1, 1), names=["Ar"],
                      pots=[("lj", 0, 0, 3.405, 0.0104, 8.5125)], state=_lj_state,
                      run=("equilibrate", -1, 0.002, 0.1, 150.0), steps=40, every=10),
    "group": dict(box=(52.6, 52.6, 52.6), pbc=(1, 1, 1), names=["Ar"],
                  pots=[("lj", 0, 0, 3.405, 0.0104, 8.5125)], state=_group_state,
                  run=("integrate", 1, 0.002), steps=40, every=10),
    "morse_open": dict(box=(21.69, 21.69, 40.0), pbc=(1, 1, 0), names=["Cu"],
                       pots=[("morse", 0, 0, 0.3429, 1.3588, 2.866, 8.0)], state=_morse_state,
                       run=("integrate", -1, 0.001), steps=60, every=10),
    "eam": dict(box=(28.92, 28.92, 28.92), pbc=(1, 1, 1), names=["Cu"],
                pots=[("eam_analytic", 0, 0)], state=_eam_state,
                run=("integrate", -1, 0.001), steps=60, every=10),
    "ttm1": dict(box=(21.69, 21.69, 144.6), pbc=(1, 1, 0), names=["Cu"], pots=[("eam_analytic", 0, 0)],
                 state=_ttm_state, run=("integrate", -1, 0.001), steps=30, every=10,
                 turi=dict(cat=1, dims=(1, 1, 20), gamma=96.6, K=400.0, G=1e17, Te=300.0, ratio=100, frac=0.1,
                           laser=(500.0, 0.0, 0.02e-12, 100e-15, 15e-9))),
    "ttm2": dict(box=(21.69, 21.69, 144.6), pbc=(1, 1, 0), names=["Cu"], pots=[("eam_analytic", 0, 0)],
                 state=_ttm_state, run=("integrate", -1, 0.001), steps=30, every=10,
                 turi=dict(cat=2, dims=(1, 1, 20), zhigilei=(1.57e6, 2.66e6, 2.41e11), Te=300.0, ratio=100,
                           frac=0.1, laser=(2000.0, 0.1, 0.02e-12, 100e-15, 15e-9))),
    "turi_custom": dict(box=(42.08, 42.08, 42.08), pbc=(1, 1, 1), names=["Ar"],
                        pots=[("lj", 0, 0, 3.405, 0.0104, 8.5125)], state=_custom_state,
                        run=("integrate", -1, 0.002), steps=20, every=10,
                        turi=dict(cat=0, dims=(2, 2, 3),
                                  fields=["TEMPERATURE", "NUMBER_DENSITY", "VCM", "MASS"])),
    # a custom turi of 11^3 = 1331 cells over 6912 atoms: more cells than
    # the per-block shared-memory bins hold, so the field passes add every
    # run total to the cell directly
    "turi_fine": dict(box=(63.12, 63.12, 63.12), pbc=(1, 1, 1), names=["Ar"],
                      pots=[("lj", 0, 0, 3.405, 0.0104, 8.5125)], state=_fine_state,
                      run=("integrate", -1, 0.002), steps=10, every=5,
                      turi=dict(cat=0, dims=(11, 11, 11),
                                fields=["TEMPERATURE", "NUMBER_DENSITY", "VCM", "MASS"])),
    # the reference's own data files (examples/data): the Mishin copper setfl
    # (as examples/02_collision.c:78 loads it) and the type-2 TTM tables of
    # examples/04_ttm2.c:116-160 (Ce_Cu.dat, G_Cu.dat, its Zhigilei K,
    # timestep ratio, activation fraction and laser; a shorter slab and an
    # earlier pulse so a short run crosses it)
    "eam_cu01": dict(box=(28.92, 28.92, 28.92), pbc=(1, 1, 1), names=["Cu"],
                     pots=[("eam_file", 0, 0, "Cu01.eam.alloy")], state=_cu01_state,
                     run=("integrate", -1, 0.001), steps=60, every=10, data=("Cu01.eam.alloy",)),
    "ttm2_cu": dict(box=(5 * LP_CU01, 5 * LP_CU01, 40 * LP_CU01), pbc=(1, 1, 0), names=["Cu"],
                    pots=[("eam_file", 0, 0, "Cu01.eam.alloy")], state=_ttm_cu_state,
                    run=("integrate", -1, 0.002), steps=30, every=10,
                    data=("Cu01.eam.alloy", "Ce_Cu.dat", "G_Cu.dat"),
                    turi=dict(cat=2, dims=(1, 1, 20), zhigilei=(1.57e6, 2.66e6, 2.41e11), Te=303.0, ratio=200,
                              frac=0.1, tables=("Ce_Cu.dat", "G_Cu.dat"),
                              laser=(2e4, 0.85, 0.02e-12, 100e-15, 14e-9))),
    # the laser-heated EAM slab of the TTM configuration (100 FCC cells along
    # z with 20 A of vacuum on either side, free z faces, a 50-cell 1-D
    # electron grid, gamma 96.6, K 400, G 1e17, 100 substeps of 0.01 fs,
    # 500 J/m^2 Gaussian pulse of 100 fs, 15 nm depth) on a 4 x 4 cell
    # cross-section instead of 20 x 20 (6400 atoms); the pulse at 0.06 ps,
    # crossed by the 200-step run
    "ttm_slab": dict(box=(4 * 3.615, 4 * 3.615, 100 * 3.615 + 40.0), pbc=(1, 1, 0), names=["Cu"],
                     pots=[("eam_analytic", 0, 0)], state=_ttm_slab_state, run=("integrate", -1, 0.001),
                     steps=200, every=40,
                     turi=dict(cat=1, dims=(1, 1, 50), gamma=96.6, K=400.0, G=1e17, Te=300.0, ratio=100,
                               frac=0.1, laser=(500.0, 0.0, 0.06e-12, 100e-15, 15e-9))),
    "hybrid": dict(box=(40.0, 30.0, 30.0), pbc=(1, 1, 1), names=["Cu", "Ar"],
                   pots=[("eam_analytic", 0, 0), ("lj", 1, 1, 3.4, 0.0104, 8.5),
                         ("lj", 0, 1, 2.87, 0.0652, 7.175)], state=_hybrid_state,
                   run=("integrate", -1, 0.001), steps=60, every=10),
}


# Full-size cases, kept out of CASES (the per-case golden tests store every
# atom's state; these goldens hold observables only: the thermo series, the
# turi fields, and the final state of the atoms with the `sample` lowest
# ids): the EAM configuration, and the TTM configuration's slab at its full
# 20 x 20 FCC-cell cross-section (160 000 atoms), 120 steps around the pulse
# at 0.06 ps.
FULL_CASES = {
    # the 256 000-atom EAM configuration (FCC 40^3, 300 K, seed 2), 100 steps
    "eam256k_full": dict(box=(40 * 3.615,) * 3, pbc=(1, 1, 1), names=["Cu"], pots=[("eam_analytic", 0, 0)],
                         state=_eam256k_state, run=("integrate", -1, 0.001), steps=100, every=25, sample=2048),
    # the Morse collision configuration (515 000 atoms, open z), 100 steps
    "morse_collision_full": dict(box=(80 * 3.615, 80 * 3.615, 20 * 3.615 + 100.0), pbc=(1, 1, 0), names=["Cu"],
                                 pots=[("morse", 0, 0, 0.3429, 1.3588, 2.866, 8.0)], state=_collision_state,
                                 run=("integrate", -1, 0.001), steps=100, every=25, sample=2048, spread=True),
    "ttm_slab_full": dict(box=(20 * 3.615, 20 * 3.615, 100 * 3.615 + 40.0), pbc=(1, 1, 0), names=["Cu"],
                          pots=[("eam_analytic", 0, 0)], state=_ttm_slab_full_state, run=("integrate", -1, 0.001),
                          steps=120, every=40,
                          turi=dict(cat=1, dims=(1, 1, 50), gamma=96.6, K=400.0, G=1e17, Te=300.0, ratio=100,
                                    frac=0.1, laser=(500.0, 0.0, 0.06e-12, 100e-15, 15e-9))),
}


def case_of(name: str) -> dict:
    return CASES[name] if name in CASES else FULL_CASES[name]


def write_data(workdir: str, data: dict):
    """Write data files (name -> bytes) into the work folder."""
    for fname, raw in data.items():
        with open(os.path.join(workdir, fname), "wb") as f:
            f.write(bytes(raw))


def golden_data(g: dict) -> dict:
    """The data files a golden .npz recorded (keys data:<file name>)."""
    return {k[5:]: np.asarray(v, np.uint8).tobytes() for k, v in g.items() if k.startswith("data:")}


def setup(lib: api.Lib, name: str, workdir: str, state: dict | None = None, data: dict | None = None):
    """Create an FMD instance for case `name` through the fmd.h API and load
    its seeded state.  `data`: the case's data files (name -> bytes), written
    into workdir first.  Returns (md, state)."""
    case = case_of(name)
    if state is None:
        state = case["state"]()
    if data:
        write_data(workdir, data)
    for fname in case.get("data", ()):
        if not os.path.exists(os.path.join(workdir, fname)):
            raise FileNotFoundError(f"case {name} needs the data file {fname}")
    md = C.c_void_p(lib.fmd_create())
    lib.fmd_io_setShowErrorMessages(md, False)
    lib.fmd_box_setSubdomains(md, 1, 1, 1)
    lib.fmd_box_setSize(md, *case["box"])
    lib.fmd_box_setPBC(md, *[bool(b) for b in case["pbc"]])
    api.set_atom_kinds(lib, md, case["names"], [MASS[n] for n in case["names"]])
    for p in case["pots"]:
        if p[0] == "lj":
            lib.fmd_pot_lj_apply(md, p[1], p[2], p[3], p[4], p[5])
        elif p[0] == "morse":
            lib.fmd_pot_morse_apply(md, p[1], p[2], p[3], p[4], p[5], p[6])
        elif p[0] == "eam_analytic":
            path = os.path.join(workdir, "analytic.eam.alloy")
            if not os.path.exists(path):
                workloads.write_analytic_eam(path)
            pot = lib.fmd_pot_eam_alloy_load(md, path.encode())
            lib.fmd_pot_apply(md, p[1], p[2], pot)
        elif p[0] == "eam_file":
            pot = lib.fmd_pot_eam_alloy_load(md, os.path.join(workdir, p[3]).encode())
            lib.fmd_pot_apply(md, p[1], p[2], pot)
    spath = os.path.join(workdir, name + ".stt")
    api.write_state(spath, 0.0, case["box"], case["pbc"], state["names"], state["kind"],
                    state["group"], state["x"], state["v"])
    lib.fmd_io_loadState(md, spath.encode(), False)
    if "turi" in case:
        # the TTM set-up reads the group's atom count (src/ttm.c:77), which
        # the reference only knows once a temperature has been computed
        lib.fmd_matt_getTemperature(md)
        # after the matter exists: the reference builds its local grid here
        setup_turi(lib, md, case["turi"], workdir)
    return md, state


def setup_turi(lib, md, tu, workdir):
    """Turi + TTM parameters through the fmd.h API; stores the handle."""
    import ctypes as C
    h = lib.fmd_turi_add(md, tu["cat"], *tu["dims"], 0.0, -1.0)
    tu["_handle"] = h
    if tu["cat"] == 0:
        for f in tu["fields"]:
            lib.fmd_field_add(md, h, getattr(api, "FMD_FIELD_" + f), 0.01)
        return
    if tu["cat"] == 1:
        lib._fmd_ttm_setHeatCapacity_linear(md, h, api.HeatCapacityLinear(tu["gamma"]))
        lib._fmd_ttm_setHeatConductivity_constant1(md, h, tu["K"])
        lib._fmd_ttm_setCouplingFactor_constant1(md, h, tu["G"])
    else:
        if "tables" in tu:
            pc, pg = (os.path.join(workdir, f) for f in tu["tables"])
        else:
            pc, pg = write_ttm_tables(workdir)
        lib._fmd_ttm_setHeatCapacity_file(md, h, pc.encode())
        v, A, B = tu["zhigilei"]
        lib._fmd_ttm_setHeatConductivity_zhigilei(md, h, api.HeatConductivityZhigilei(v, A, B))
        lib._fmd_ttm_setCouplingFactor_file(md, h, pg.encode())
    lib.fmd_ttm_setElectronTemperature(md, h, tu["Te"])
    lib.fmd_ttm_setTimestepRatio(md, h, tu["ratio"])
    lib.fmd_ttm_setCellActivationFraction(md, h, tu["frac"])
    f, R, t0, dur, depth = tu["laser"]
    lib._fmd_ttm_setLaserSource_gaussian(md, h, api.LaserGaussian(f, R, t0, dur, depth))


class Recorder:
    """Event handler recording (time, T, E_total, KE) at each timer tick and
    every error event."""

    def __init__(self, lib):
        self.lib = lib
        self.rows = []
        self.errors = []
        self.timer = None

        def handler(md, event, usp, params):
            if event == api.FMD_EVENT_TIMER_TICK:
                t = lib.fmd_dync_getTime(md)
                self.rows.append((t, lib.fmd_matt_getTemperature(md), lib.fmd_matt_getTotalEnergy(md),
                                  lib.fmd_matt_getKineticEnergy(md)))
            elif event == api.FMD_EVENT_ERROR:
                p = C.cast(params, C.POINTER(api.ErrorParams)).contents
                self.errors.append((p.error, bool(p.major)))

        self.cb = api.EventHandler(handler)
        self.fields = []       # (time, turi, field, values) at every field update event
        self.field_cats = {}

    def record_fields(self, md, turi):
        """also record every field-update event and the field's array"""
        import ctypes as C
        lib = self.lib
        self.turi = turi

        def handler(mdp, event, usp, params):
            if event == api.FMD_EVENT_TIMER_TICK:
                t = lib.fmd_dync_getTime(mdp)
                self.rows.append((t, lib.fmd_matt_getTemperature(mdp), lib.fmd_matt_getTotalEnergy(mdp),
                                  lib.fmd_matt_getKineticEnergy(mdp)))
            elif event == api.FMD_EVENT_ERROR:
                p = C.cast(params, C.POINTER(api.ErrorParams)).contents
                self.errors.append((p.error, bool(p.major)))
            elif event == api.FMD_EVENT_FIELD_UPDATE:
                p = C.cast(params, C.POINTER(api.FieldUpdateParams)).contents
                vals = None
                cat = self.field_cats.get(p.field)
                if cat is not None and cat != api.FMD_FIELD_TTM_XI:
                    arr = C.c_void_p()
                    dims = (C.c_uint * 3)()
                    a3s = lib.fmd_field_getArray(mdp, p.turi, p.field, C.byref(arr), dims)
                    if a3s:
                        vals = read_array3(arr, dims, cat)
                        lib.fmd_array3s_free(a3s)
                self.fields.append((lib.fmd_dync_getTime(mdp), p.turi, p.field, vals))

        self.cb = api.EventHandler(handler)
        for cat in range(7):
            fi = lib.fmd_field_find(md, turi, cat)
            if fi >= 0:
                self.field_cats[fi] = cat

    def attach(self, md, interval):
        self.lib.fmd_setEventHandler(md, None, self.cb)
        if self.timer is None:
            self.timer = self.lib.fmd_timer_makeSimple(md, 0.0, interval, -1.0)


def read_array3(arr, dims, cat):
    """Copy an fmd_array3_t (void***) of the given field category."""
    import ctypes as C
    n0, n1, n2 = dims[0], dims[1], dims[2]
    p0 = C.cast(arr, C.POINTER(C.POINTER(C.c_void_p)))
    if cat == api.FMD_FIELD_NUMBER:
        et, k = C.c_uint, 1
    elif cat == api.FMD_FIELD_VCM:
        et, k = C.c_double, 3
    else:
        et, k = C.c_double, 1
    out = np.zeros((n0, n1, n2, k))
    for i in range(n0):
        for j in range(n1):
            row = C.cast(p0[i][j], C.POINTER(et))
            out[i, j] = np.ctypeslib.as_array(row, shape=(n2 * k,)).reshape(n2, k)
    return out


def run(lib: api.Lib, name: str, md, rec: Recorder | None = None, steps=None):
    """Run the case's dynamics for `steps` time steps (default: the case's)."""
    case = case_of(name)
    r = case["run"]
    n = case["steps"] if steps is None else steps
    dt = r[2]
    duration = (n - 0.5) * dt
    if rec is not None:
        rec.attach(md, case["every"] * dt)
    if r[0] == "integrate":
        lib.fmd_dync_integrate(md, r[1], duration, dt)
    else:
        lib.fmd_dync_equilibrate(md, r[1], duration, dt, r[3], r[4])


def check_ttm_tables(tables, g):
    """Type-2 tables against the reference's: the knots exactly, the values
    (unit conversion of the file's numbers) to 1e-15 relative, and the
    spline second derivatives by their effect on the interpolated values
    (|dDD| h^2 / 6 within 1e-14 of the largest value): the tridiagonal
    solve rounds differently, and a nearly straight table has second
    derivatives at rounding level."""
    for key, arr in tables.items():
        ref = g["ttm_tab_" + key]
        if key.startswith("T_"):
            np.testing.assert_array_equal(arr, ref)
        elif key.endswith("_DD"):
            knots = g["ttm_tab_T_" + key[0]]
            vals = g["ttm_tab_" + key[0] + "t"]
            h = float(np.diff(knots).max())
            assert np.abs(arr - ref).max() * h * h / 6.0 <= 1e-14 * np.abs(vals).max(), key
        else:
            np.testing.assert_allclose(arr, ref, rtol=1e-15, atol=0)
