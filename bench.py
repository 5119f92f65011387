"""Benchmark: atom-steps/s of FMD's per-timestep hot path on one GB300.

Workload (default): the 256 000-atom EAM system -- FCC 40x40x40 cells,
a = 3.615 A, Cu mass, periodic, analytic EAM tabulated on 10 000 r and
10 000 rho points, 300 K Maxwell velocities from seed 2, dt = 1 fs,
NVE velocity Verlet.  Synthetic inputs built through the fmd.h API
(no dataset involved).  One "step" = one MD time step of the whole system
(refresh, EAM density + embedding, forces, both half-kicks, reductions).

    python bench.py [--steps K] [--warmup W] [--precision fp64|mixed]
    python bench.py --impl reference     # CPU oracle port on the host cores

Timing: device time with CUDA events on the engine's stream, one event
pair per step, L2 flushed (256 MB write) before every timed step; the
working set (~30 MB) is smaller than L2, so flushing is the rule used.
`e2e` drives the same steps through the C-ABI with host buffers: every
step uploads positions+velocities from pinned host memory, runs the step
and reads positions, velocities and the thermo record back.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOAD = dict(name="eam256k", cells=(40, 40, 40), a=3.615, T=300.0, seed=2, dt=0.001, mass=63.546)
# algorithmic work per atom-step: unique pairs inside rc (half shell) for the
# analytic EAM at a = 3.615 A, rc = 5.5 A: 4/3 pi rc^3 n / 2 = 29.5 pairs;
# flops per pair from the reference's formulas (density 26, force 68) plus
# 26 per atom for the embedding (src/eam.h:177-406, src/cspline.h:26-27)
PAIRS_PER_ATOM = 29.5
FLOP_DENSITY = 26.0 * PAIRS_PER_ATOM + 26.0
FLOP_FORCE = 68.0 * PAIRS_PER_ATOM


def clocks_sampler(stop, out):
    cmd = ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
           "--format=csv,noheader,nounits", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]]
    while not stop.is_set():
        try:
            r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=5)
            if r.returncode == 0 and r.stdout.strip():
                out.append([p.strip() for p in r.stdout.strip().split(",")])
        except Exception:
            pass
        stop.wait(0.2)


def summarize_clocks(samples):
    if not samples:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    sm = sorted(float(s[0]) for s in samples if s[0].replace(".", "").isdigit())
    mx = max(float(s[1]) for s in samples if s[1].replace(".", "").isdigit()) if sm else None
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    reasons = set()
    for s in samples:
        for k, n in enumerate(names):
            if len(s) > 3 + k and s[3 + k].lower().startswith("active"):
                reasons.add(n)
    return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
            "samples": len(samples)}


def make_system(lib, api, work, precision):
    from fmd_gb300 import workloads
    w = WORKLOAD
    md = C.c_void_p(lib.fmd_create())
    lib.fmd_io_setShowErrorMessages(md, True)
    lib.fmd_box_setSubdomains(md, 1, 1, 1)
    L = [c * w["a"] for c in w["cells"]]
    lib.fmd_box_setSize(md, *L)
    lib.fmd_box_setPBC(md, True, True, True)
    api.set_atom_kinds(lib, md, ["Cu"], [w["mass"]])
    path = os.path.join(work, "analytic.eam.alloy")
    workloads.write_analytic_eam(path)
    pot = lib.fmd_pot_eam_alloy_load(md, path.encode())
    lib.fmd_pot_apply(md, 0, 0, pot)
    lib.L.fmdx_set_seed.argtypes = [C.c_void_p, C.c_ulonglong]
    lib.L.fmdx_set_seed(md, w["seed"])
    lib.L.fmdx_set_precision.argtypes = [C.c_void_p, C.c_int]
    lib.L.fmdx_set_precision(md, 1 if precision == "mixed" else 0)
    lib.fmd_matt_makeCuboidFCC(md, 0.0, 0.0, 0.0, *w["cells"], w["a"], 0, 0, w["T"])
    lib.fmd_dync_integrate(md, -1, 0.0, w["dt"])     # distribute + initial forces
    return md


def run_ours(args):
    import fmd_gb300
    from fmd_gb300 import api
    lib = fmd_gb300.load()
    L = lib.L
    L.fmdx_device.restype = C.c_void_p
    L.fmdx_device.argtypes = [C.c_void_p]
    for name, at in [("fmdg_vv_steps", [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_int, C.c_double, C.c_double]),
                     ("fmdg_timer_start", [C.c_void_p]), ("fmdg_timer_stop", [C.c_void_p, C.POINTER(C.c_float)]),
                     ("fmdg_flush_l2", [C.c_void_p]), ("fmdg_sync", [C.c_void_p]),
                     ("fmdg_set_profiling", [C.c_void_p, C.c_int]),
                     ("fmdg_get_profile", [C.c_void_p, C.c_char_p, C.POINTER(C.c_float), C.POINTER(C.c_int)]),
                     ("fmdg_measure_fma_peak", [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
                     ("fmdg_launch_count", [C.c_void_p, C.POINTER(C.c_longlong)]),
                     ("fmdg_natoms", [C.c_void_p, C.POINTER(C.c_int)]),
                     ("fmdg_get_errors", [C.c_void_p, C.POINTER(C.c_uint), C.c_int])]:
        getattr(L, name).argtypes = at
        getattr(L, name).restype = C.c_int
    w = WORKLOAD
    dt = w["dt"]
    with tempfile.TemporaryDirectory() as work:
        md = make_system(lib, api, work, args.precision)
        dev = C.c_void_p(L.fmdx_device(md))
        n = C.c_int(0)
        L.fmdg_natoms(dev, C.byref(n))
        natoms = n.value

        def ck(rc, what):
            if rc != 0:
                L.fmdg_last_error.restype = C.c_char_p
                raise RuntimeError(f"{what}: {L.fmdg_last_error().decode()}")

        ck(L.fmdg_vv_steps(dev, args.warmup, dt, -1, 0, 1.0, 0.0), "warmup")
        ck(L.fmdg_sync(dev), "sync")
        stop = threading.Event()
        samples = []
        th = threading.Thread(target=clocks_sampler, args=(stop, samples), daemon=True)
        th.start()
        lc0 = C.c_longlong(0)
        L.fmdg_launch_count(dev, C.byref(lc0))
        total_ms = 0.0
        ms = C.c_float(0.0)
        for _ in range(args.steps):
            ck(L.fmdg_flush_l2(dev), "flush")
            ck(L.fmdg_timer_start(dev), "timer")
            ck(L.fmdg_vv_steps(dev, 1, dt, -1, 0, 1.0, 0.0), "step")
            ck(L.fmdg_timer_stop(dev, C.byref(ms)), "timer")
            total_ms += ms.value
        lc1 = C.c_longlong(0)
        L.fmdg_launch_count(dev, C.byref(lc1))
        stop.set()
        th.join(timeout=5)
        clocks = summarize_clocks(samples)
        # per-phase device time (separate launches between events)
        ck(L.fmdg_set_profiling(dev, 1), "prof")
        nprof = max(3, min(10, args.steps))
        ck(L.fmdg_vv_steps(dev, nprof, dt, -1, 0, 1.0, 0.0), "profile")
        phases = {}
        for ph in ("bin", "nlist", "density", "force", "reduce"):
            pms, pn = C.c_float(0.0), C.c_int(0)
            L.fmdg_get_profile(dev, ph.encode(), C.byref(pms), C.byref(pn))
            phases[ph] = pms.value / max(pn.value, 1)
        ck(L.fmdg_set_profiling(dev, 0), "prof")
        peak64, peak32 = C.c_double(0), C.c_double(0)
        ck(L.fmdg_measure_fma_peak(dev, 1, C.byref(peak64)), "peak")
        ck(L.fmdg_measure_fma_peak(dev, 0, C.byref(peak32)), "peak")
        errs = C.c_uint(0)
        L.fmdg_get_errors(dev, C.byref(errs), 0)
        lib.fmd_free(md)

    ms_per_step = total_ms / args.steps
    value = natoms / (ms_per_step * 1e-3)
    force_ms = phases["force"]
    achieved = natoms * FLOP_FORCE / (force_ms * 1e-3) / 1e12
    peak = peak64.value if args.precision == "fp64" else peak32.value
    out = {
        "metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32-compute/f64-accumulate",
        "data": "synthetic",
        "config": {"workload": "EAM FCC 40x40x40 (256000 atoms), analytic EAM on 10000-point splines, "
                               "300 K, dt 1 fs, NVE", "atoms": natoms, "precision": args.precision,
                   "l2": "flushed before every timed step (working set < L2)"},
        "gpu_launches": int(lc1.value - lc0.value),
        "phases_ms": phases,
        "roofline": {"bound": "fp64-issue" if args.precision == "fp64" else "fp32-issue",
                     "kernel": "k_force (EAM pair forces + finish step)",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "peak_source": "measured FMA-chain microkernel (no CUDA-core peak in MEASURED_PEAKS.json)",
                     "traffic": None},
        "clocks": clocks,
        "device_errors": errs.value,
    }
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        print(json.dumps({"impl": "reference", "unavailable": "CPU oracle port not built yet"}))
        return
    out = run_ours(args)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
