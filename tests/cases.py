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
    "hybrid": dict(box=(40.0, 30.0, 30.0), pbc=(1, 1, 1), names=["Cu", "Ar"],
                   pots=[("eam_analytic", 0, 0), ("lj", 1, 1, 3.4, 0.0104, 8.5),
                         ("lj", 0, 1, 2.87, 0.0652, 7.175)], state=_hybrid_state,
                   run=("integrate", -1, 0.001), steps=60, every=10),
}


def setup(lib: api.Lib, name: str, workdir: str, state: dict | None = None):
    """Create an FMD instance for case `name` through the fmd.h API and load
    its seeded state.  Returns (md, state)."""
    case = CASES[name]
    if state is None:
        state = case["state"]()
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
    spath = os.path.join(workdir, name + ".stt")
    api.write_state(spath, 0.0, case["box"], case["pbc"], state["names"], state["kind"],
                    state["group"], state["x"], state["v"])
    lib.fmd_io_loadState(md, spath.encode(), False)
    return md, state


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

    def attach(self, md, interval):
        self.lib.fmd_setEventHandler(md, None, self.cb)
        self.timer = self.lib.fmd_timer_makeSimple(md, 0.0, interval, -1.0)


def run(lib: api.Lib, name: str, md, rec: Recorder | None = None, steps=None):
    """Run the case's dynamics for `steps` time steps (default: the case's)."""
    case = CASES[name]
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
