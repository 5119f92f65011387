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


def numpy_state_cell_order(nc, cellh):
    """The workload's atoms binned the way the reference distributes them:
    cell = floor(x/cellh), insertion order kept inside each cell."""
    from fmd_gb300 import workloads
    w = WORKLOAD
    x, v = workloads.fcc_state(*w["cells"], w["a"], w["T"], w["mass"], seed=w["seed"])
    ic = np.floor(x / np.asarray(cellh)).astype(np.int64)
    cell = ic[:, 2] + nc[2] * (ic[:, 1] + nc[1] * ic[:, 0])
    order = np.argsort(cell, kind="stable")
    n = len(x)
    return (cell[order].astype(np.int32), x[order], v[order], np.zeros(n, np.uint32), np.zeros(n, np.int32),
            order.astype(np.uint32))


def eam_geometry():
    w = WORKLOAD
    box = [c * w["a"] for c in w["cells"]]
    from fmd_gb300 import workloads
    nc = [int(b / workloads.EAM_RC) for b in box]
    cellh = [b / n for b, n in zip(box, nc)]
    return box, nc, cellh


def cpu_port_run(threads, target_s=12.0, max_steps=20):
    """Time the CPU oracle port (restated reference algorithm, OpenMP with
    per-thread buffers) on the same workload; returns (atom-steps/s, steps)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from fmd_gb300 import workloads
    w = WORKLOAD
    box, nc, cellh = eam_geometry()
    with tempfile.TemporaryDirectory() as work:
        setfl = workloads.write_analytic_eam(os.path.join(work, "analytic.eam.alloy"))
        o = pyoracle.Oracle(threads=threads)
        o.setup(box, [1, 1, 1], nc, cellh, [("Cu", w["mass"])], [("eam", 0, 0)], setfl)
    cell, x, v, kind, group, ids = numpy_state_cell_order(nc, cellh)
    o.upload(cell, x, v, kind, group, ids, int(np.prod(nc)))
    o.forces(-1)
    t0 = time.perf_counter()
    o.vv(1, w["dt"])
    t1 = time.perf_counter()
    k = int(max(1, min(max_steps, target_s / max(t1 - t0, 1e-6))))
    t2 = time.perf_counter()
    o.vv(k, w["dt"])
    t3 = time.perf_counter()
    o.close()
    return len(x) * k / (t3 - t2), k


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
        for ph in ("bin", "nlist", "density", "force", "turi"):
            pms, pn = C.c_float(0.0), C.c_int(0)
            L.fmdg_get_profile(dev, ph.encode(), C.byref(pms), C.byref(pn))
            phases[ph] = pms.value / max(pn.value, 1)
        ck(L.fmdg_set_profiling(dev, 0), "prof")
        peak64, peak32 = C.c_double(0), C.c_double(0)
        ck(L.fmdg_measure_fma_peak(dev, 1, C.byref(peak64)), "peak")
        ck(L.fmdg_measure_fma_peak(dev, 0, C.byref(peak32)), "peak")
        errs = C.c_uint(0)
        L.fmdg_get_errors(dev, C.byref(errs), 0)
        # end to end through the C-ABI with pinned host buffers
        L.fmdg_host_alloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        L.fmdg_host_free.argtypes = [C.c_void_p]
        L.fmdg_run_host.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int] + [C.c_void_p] * 6
        nb = 3 * natoms * 8
        bufs = [C.c_void_p() for _ in range(5)]
        for k, b in enumerate(bufs):
            ck(L.fmdg_host_alloc(C.byref(b), nb if k < 4 else natoms * 4), "pinned alloc")
        th = (C.c_double * 8)()
        ck(L.fmdg_run_host(dev, 0, dt, -1, None, None, bufs[0], bufs[1], bufs[4], th), "e2e prime")
        xin, vin, xout, vout = bufs[0], bufs[1], bufs[2], bufs[3]
        e2e_steps = max(3, args.steps)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ck(L.fmdg_run_host(dev, 1, dt, -1, xin, vin, xout, vout, bufs[4], th), "e2e step")
            xin, xout = xout, xin
            vin, vout = vout, vin
        t1 = time.perf_counter()
        e2e_value = natoms * e2e_steps / (t1 - t0)
        for b in bufs:
            L.fmdg_host_free(b)
        lib.fmd_free(md)
    cores = os.cpu_count() or 1
    if args.skip_cpu:
        cpu_value, cpu_steps = None, 0
    else:
        cpu_value, cpu_steps = cpu_port_run(cores)

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
        "e2e": {"value": e2e_value, "unit": "atom-steps/s", "h2d_bytes_per_step": 2 * 3 * natoms * 8,
                "d2h_bytes_per_step": 2 * 3 * natoms * 8 + natoms * 4 + 64,
                "how": "fmdg_run_host: positions+velocities in from pinned host memory, one step, "
                       "positions+velocities+atom ids+thermo record out; wall clock"},
        "cpu_baseline": {"value": cpu_value, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{cpu_steps} velocity-Verlet steps of the same 256000-atom EAM system "
                                   "(restated reference algorithm, OpenMP, per-thread force buffers)"},
    }
    return out


def run_reference(args):
    """The reference's CPU implementation of the path on the host cores: the
    oracle port (the reference's own sources are not present on the GPU
    host), all threads, same workload, metric and unit."""
    cores = os.cpu_count() or 1
    vals = []
    for _ in range(max(1, min(args.steps, 3))):
        v, k = cpu_port_run(cores, target_s=8.0, max_steps=10)
        vals.append(v)
    value = float(np.median(vals))
    w = WORKLOAD
    out = {"impl": "reference", "metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": 0,
           "steps": len(vals), "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic",
           "config": {"workload": "EAM FCC 40x40x40 (256000 atoms), analytic EAM on 10000-point splines, "
                                  "300 K, dt 1 fs, NVE", "atoms": int(np.prod(w["cells"])) * 4},
           "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                            "sample": f"median of {len(vals)} timed samples of up to 10 steps each"},
           "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU baseline (profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        run_reference(args)
        return
    out = run_ours(args)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
