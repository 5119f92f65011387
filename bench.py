"""Benchmark: atom-steps/s of FMD's per-timestep hot path on one GB300.

Workloads
  served (default)  the served job stream: 2048 independent FCC cubes (500
                    to 200 000 atoms, log-uniform), potential uniform over
                    the argon LJ / copper Morse / analytic copper EAM,
                    50-1200 K, step counts uniform in [1000, 20000], Poisson
                    arrivals at 50 jobs/s (seed 5).  Mixed precision
                    (binary32 pair arithmetic, binary64 sums), packed per
                    potential, chunks of steps replayed as CUDA graphs.
                    --jobs / --step-scale shorten it (first jobs; step
                    counts and arrival times scaled together) for quick runs.
  eam256k           one 256 000-atom EAM system (FCC 40x40x40, a = 3.615 A,
                    300 K, seed 2, dt 1 fs), the single-system drop-in path.
  ttm               the laser-heated EAM slab with the 1-D two-temperature
                    model (800 000 atoms, 50 electron cells), the fmd.h path;
                    roofline of the HBM-bound turi field passes.

    python bench.py [--steps K] [--warmup W] [--workload served|eam256k|ttm]
    python bench.py --impl reference     # CPU oracle port on the host cores

served: `value` = every job of the stream resident in HBM at once, K fleet
steps (each: FLEET_CHUNK velocity-Verlet steps of every job, all packs'
graphs replayed concurrently) between CUDA events on a join stream; the
fleet's working set (tens of GB) is larger than L2.  `e2e` = the stream
through the request loop (fmdg_srv_* C-ABI) from host arrays: arrivals,
admission by HBM budget, upload, steps, results; wall clock from the first
arrival to the last completion; p50/p99 job latency.  `plain_fp64` = jobs
one at a time through the plain single-system binary64 path (the path
libfmd.so's fmd_dync_integrate drives): every PLAIN_EVERY-th job timed
(set-up + first step, then PLAIN_STEPS steps) and extrapolated to its step
count; `served_over_plain_fp64` = e2e / plain_fp64.
eam256k: device time with CUDA events per step, L2 flushed (256 MB write)
before every timed step; `e2e` drives the same steps through the C-ABI
with pinned host buffers.
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
# The served fleet runs dozens of packs on their own streams: more hardware
# work queues (the default is 8) keep unrelated streams from queueing behind
# one another.  Read when the CUDA context is created, so set before it.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

import numpy as np  # noqa: E402

WORKLOAD = dict(name="eam256k", cells=(40, 40, 40), a=3.615, T=300.0, seed=2, dt=0.001, mass=63.546)
# algorithmic work per atom-step: unique pairs inside rc (half shell) for the
# analytic EAM at a = 3.615 A, rc = 5.5 A: 4/3 pi rc^3 n / 2 = 29.5 pairs;
# flops per pair from the reference's formulas (density 26, force 68) plus
# 26 per atom for the embedding (src/eam.h:177-406, src/cspline.h:26-27)
PAIRS_PER_ATOM = 29.5
FLOP_DENSITY = 26.0 * PAIRS_PER_ATOM + 26.0
FLOP_FORCE = 68.0 * PAIRS_PER_ATOM
# served stream: algorithmic flops of the pair-force kernel per atom-step
# (unique pairs inside rc x flops per pair of the reference's formulas):
# LJ 35.5 x 31 (src/lj.h:35-56), Morse 91 x 31 (src/morse.h:35-56),
# EAM 29.5 x 68 (src/eam.h:186-226)
SERVED_FORCE_FLOP = {"lj": 35.5 * 31.0, "morse": 91.0 * 31.0, "eam": 29.5 * 68.0}
# DRAM bytes (read + write) per atom of one pair-force launch, from ncu
# captures of the same kernels (dram__bytes_read.sum + dram__bytes_write.sum
# divided by the atoms of the launch): packed Morse on a 149616-atom pack,
# single-system mixed EAM on the 256000-atom system (both skin lists); the traffic
# grows with the atoms (the neighbour list dominates it)
FORCE_DRAM_BYTES_PER_ATOM = {"morse_pack": 144.87e6 / 149616, "eam_single": 101.07e6 / 256000}


class ClockSampler:
    """nvidia-smi clock and throttle readings around a timed region: one
    query after another (~50 ms apart) from before the region starts until
    it ends; a reading counts when its query overlapped the region."""

    QUERY = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.readings = []          # (t_query_start, t_query_end, fields)
        self.stop_ev = threading.Event()
        self.first = threading.Event()
        self.t0 = self.t1 = None
        self.th = None

    def _loop(self):
        cmd = ["nvidia-smi", "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
               "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]]
        while not self.stop_ev.is_set():
            ta = time.monotonic()
            try:
                r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=5)
                if r.returncode == 0 and r.stdout.strip():
                    self.readings.append((ta, time.monotonic(), [p.strip() for p in r.stdout.strip().split(",")]))
                    self.first.set()
            except Exception:
                self.first.set()
                return
            self.stop_ev.wait(0.05)

    def start(self):
        """Start sampling; returns once the first reading is in (at most 10 s)."""
        import shutil
        if shutil.which("nvidia-smi"):
            self.th = threading.Thread(target=self._loop, daemon=True)
            self.th.start()
            self.first.wait(timeout=10)
        self.t0 = time.monotonic()

    def stop(self):
        self.t1 = time.monotonic()
        self.stop_ev.set()
        if self.th is not None:
            self.th.join(timeout=6)
        return self.summary()

    def summary(self):
        inside = [f for a, b, f in self.readings if b >= self.t0 and a <= self.t1]
        if not inside and self.readings:     # region shorter than one query: the nearest reading
            inside = [min(self.readings, key=lambda r: abs(r[1] - self.t1))[2]]
        out = summarize_clocks(inside)
        out["region_s"] = round(self.t1 - self.t0, 3)
        return out


def hbm_peak_gbs():
    """The measured HBM copy bandwidth (MEASURED_PEAKS.json beside this
    file), else the fallback figure; returns (GB/s, source)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except Exception:
        return 6800.0, "fallback (6.8 TB/s)"


def hbm_side(traffic_bytes, kernel_ms):
    """The same kernel against the HBM roof: its DRAM bytes per launch
    (ncu) over its event-timed duration, as a fraction of the copy peak."""
    if not traffic_bytes or not kernel_ms:
        return {}
    peak, src = hbm_peak_gbs()
    gbs = traffic_bytes / (kernel_ms * 1e-3) / 1e9
    return {"dram_gbs": gbs, "frac_of_hbm": gbs / peak, "hbm_peak_gbs": peak, "hbm_peak_source": src}


def summarize_clocks(samples):
    if not samples:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    sm = sorted(float(s[0]) for s in samples if len(s) > 0 and s[0].replace(".", "").isdigit())
    mxs = [float(s[1]) for s in samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
    mx = max(mxs) if mxs else None
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


def cpu_port_ttm(threads, target_s=12.0, max_steps=20):
    """Time the CPU oracle port on the TTM slab: the full symplectic-Euler
    step (kick-drift, refresh, turi fields, TTM solver, EAM forces with the
    friction term), OpenMP pair loops on `threads` threads, the slab's
    seeded initial state at the pulse (time 0.95 ps: the source active) and
    the type-1 parameters the reference derives from the workload's inputs
    (pyoracle.ttm1_params); returns (atom-steps/s, steps)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from fmd_gb300 import workloads
    w = TTM
    nx, ny, nz = w["cells"]
    a = w["a"]
    box = (nx * a, ny * a, nz * a + 2 * w["vacuum"])
    x, v = workloads.fcc_state(nx, ny, nz, a, w["T"], w["mass"], seed=w["seed"], origin=(0.0, 0.0, w["vacuum"]))
    ncell = [int(b / workloads.EAM_RC) for b in box]
    cellh = [b / q for b, q in zip(box, ncell)]
    ic = np.floor(x / np.asarray(cellh)).astype(np.int64)
    cell = ic[:, 2] + ncell[2] * (ic[:, 1] + ncell[1] * ic[:, 0])
    order = np.argsort(cell, kind="stable")
    n = len(x)
    with tempfile.TemporaryDirectory() as work:
        setfl = workloads.write_analytic_eam(os.path.join(work, "analytic.eam.alloy"))
        o = pyoracle.Oracle(threads=threads)
        o.setup(box, [1, 1, 0], ncell, cellh, [("Cu", w["mass"])], [("eam", 0, 0)], setfl)
    o.upload(cell[order].astype(np.int32), x[order], v[order], np.zeros(n, np.uint32), np.zeros(n, np.int32),
             order.astype(np.uint32), int(np.prod(ncell)))
    pd, pk = pyoracle.ttm1_params(box, w["dims"][2], x, w["gamma"], w["K"], w["G"], w["laser"], w["frac"],
                                  w["ratio"])
    o.ttm_setup(pd, pk, w["Te"])
    o.set_time(w["t_start"], w["dt"])
    o.turi_update()
    o.forces(-1)
    t0 = time.perf_counter()
    o.se_steps(1, w["dt"])
    t1 = time.perf_counter()
    k = int(max(1, min(max_steps, target_s / max(t1 - t0, 1e-6))))
    t2 = time.perf_counter()
    o.se_steps(k, w["dt"])
    t3 = time.perf_counter()
    o.close()
    return n * k / (t3 - t2), k


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
        sampler = ClockSampler()
        sampler.start()
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
        clocks = sampler.stop()
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
    # both modes issue on the binary32 pipe: binary64 mode evaluates EAM
    # pairs in double-float arithmetic (fmdg_df.cuh), binary64 accuracy
    peak = peak32.value
    out = {
        "metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": ("double-float pairs (two binary32, ~48 bits), binary64 integration" if args.precision == "fp64"
                  else "f32-compute/f64-accumulate"),
        "data": "synthetic",
        "config": {"workload": "EAM FCC 40x40x40 (256000 atoms), analytic EAM on 10000-point splines, "
                               "300 K, dt 1 fs, NVE", "atoms": natoms, "precision": args.precision,
                   "l2": "flushed before every timed step (working set < L2)"},
        "gpu_launches": int(lc1.value - lc0.value),
        "phases_ms": phases,
        "roofline": {"bound": "fp32-issue",
                     "kernel": ("k_force (EAM pair forces + finish step, double-float binary64 arithmetic)"
                                if args.precision == "fp64" else "k_force (EAM pair forces + finish step)"),
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "frac_of_fp64_fma_peak": achieved / peak64.value,
                     "peak_source": "measured FMA-chain microkernel (no CUDA-core peak in MEASURED_PEAKS.json)",
                     "traffic": (FORCE_DRAM_BYTES_PER_ATOM["eam_single"] * natoms if args.precision == "mixed"
                                 else None),
                     **hbm_side(FORCE_DRAM_BYTES_PER_ATOM["eam_single"] * natoms if args.precision == "mixed"
                                else None, phases["force"])},
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


# ---------------------------------------------------------------- TTM slab
TTM = dict(cells=(40, 50, 100), a=3.615, T=300.0, seed=4, mass=63.546, dt=0.001, vacuum=20.0,
           dims=(1, 1, 50), gamma=96.6, K=400.0, G=1e17, Te=300.0, ratio=100, frac=0.1,
           laser=(500.0, 0.0, 1e-12, 100e-15, 15e-9), t_start=0.95)
# algorithmic HBM bytes per atom-step of the memory-bound TTM kernels
# (binary64 state): the two turi field passes each read x, v (48 B) and the
# kind (4 B) of every atom (src/turi.c:959-1335); the kick-drift reads x, v,
# F and the kind, writes x, v (124 B, src/integrators.c:129-179)
TTM_FIELD_BYTES = 2 * (48 + 4)
SE_KICK_BYTES = 72 + 4 + 48


def ttm_config():
    w = TTM
    return {"workload": "laser-heated EAM copper slab with a 1-D two-temperature model: FCC %dx%dx%d cells "
                        "(%d atoms; a = 3.615 A, 300 K seed 4), periodic x, y, %.0f A vacuum on both free z "
                        "faces, analytic EAM; electron grid of %d cells along z, gamma 96.6 J/m^3K^2, K 400 W/mK, "
                        "G 1e17 W/m^3K, 100 explicit substeps of 0.01 fs per 1 fs step; 500 J/m^2 Gaussian pulse "
                        "(FWHM 100 fs at 1 ps, 15 nm depth); timed steps start at %.2f ps (through the pulse)"
                        % (*w["cells"], 4 * int(np.prod(w["cells"])), w["vacuum"], w["dims"][2], w["t_start"]),
            "atoms": 4 * int(np.prod(w["cells"])), "precision": "mixed forces, binary64 electron temperatures",
            "step": "one symplectic-Euler step: kick-drift, cell refresh, turi field passes, TTM solver, "
                    "neighbour list, EAM density, pair forces + friction term",
            "l2": "working set (~0.5 GB) larger than L2, no flush needed"}


def make_ttm_system(lib, api, work):
    from fmd_gb300 import workloads
    w = TTM
    nx, ny, nz = w["cells"]
    a = w["a"]
    box = (nx * a, ny * a, nz * a + 2 * w["vacuum"])
    x, v = workloads.fcc_state(nx, ny, nz, a, w["T"], w["mass"], seed=w["seed"], origin=(0.0, 0.0, w["vacuum"]))
    n = len(x)
    md = C.c_void_p(lib.fmd_create())
    lib.fmd_io_setShowErrorMessages(md, True)
    lib.fmd_box_setSubdomains(md, 1, 1, 1)
    lib.fmd_box_setSize(md, *box)
    lib.fmd_box_setPBC(md, True, True, False)
    api.set_atom_kinds(lib, md, ["Cu"], [w["mass"]])
    path = workloads.write_analytic_eam(os.path.join(work, "analytic.eam.alloy"))
    pot = lib.fmd_pot_eam_alloy_load(md, path.encode())
    lib.fmd_pot_apply(md, 0, 0, pot)
    spath = os.path.join(work, "slab.stt")
    api.write_state(spath, 0.0, box, (1, 1, 0), ["Cu"], np.zeros(n, np.uint32), np.zeros(n, np.int32), x, v)
    lib.fmd_io_loadState(md, spath.encode(), False)
    lib.L.fmdx_set_precision.argtypes = [C.c_void_p, C.c_int]
    lib.L.fmdx_set_precision(md, 1)
    lib.fmd_matt_getTemperature(md)          # the TTM set-up reads the group's atom count
    h = lib.fmd_turi_add(md, 1, *w["dims"], 0.0, -1.0)
    lib._fmd_ttm_setHeatCapacity_linear(md, h, api.HeatCapacityLinear(w["gamma"]))
    lib._fmd_ttm_setHeatConductivity_constant1(md, h, w["K"])
    lib._fmd_ttm_setCouplingFactor_constant1(md, h, w["G"])
    lib.fmd_ttm_setElectronTemperature(md, h, w["Te"])
    lib.fmd_ttm_setTimestepRatio(md, h, w["ratio"])
    lib.fmd_ttm_setCellActivationFraction(md, h, w["frac"])
    lib._fmd_ttm_setLaserSource_gaussian(md, h, api.LaserGaussian(*w["laser"]))
    return md, h, n


def run_ttm(args):
    import fmd_gb300
    from fmd_gb300 import api
    lib = fmd_gb300.load()
    L = lib.L
    L.fmdx_device.restype = C.c_void_p
    L.fmdx_device.argtypes = [C.c_void_p]
    for name, at in [("fmdg_se_steps", [C.c_void_p, C.c_int, C.c_double, C.c_int]),
                     ("fmdg_timer_start", [C.c_void_p]), ("fmdg_timer_stop", [C.c_void_p, C.POINTER(C.c_float)]),
                     ("fmdg_sync", [C.c_void_p]), ("fmdg_set_profiling", [C.c_void_p, C.c_int]),
                     ("fmdg_get_profile", [C.c_void_p, C.c_char_p, C.POINTER(C.c_float), C.POINTER(C.c_int)]),
                     ("fmdg_measure_fma_peak", [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
                     ("fmdg_launch_count", [C.c_void_p, C.POINTER(C.c_longlong)]),
                     ("fmdg_get_errors", [C.c_void_p, C.POINTER(C.c_uint), C.c_int])]:
        getattr(L, name).argtypes = at
        getattr(L, name).restype = C.c_int
    w = TTM
    dt = w["dt"]

    def ck(rc, what):
        if rc != 0:
            L.fmdg_last_error.restype = C.c_char_p
            raise RuntimeError(f"{what}: {L.fmdg_last_error().decode()}")

    with tempfile.TemporaryDirectory() as work:
        md, h, natoms = make_ttm_system(lib, api, work)
        # to the window before the pulse (warm-up included)
        n_pre = max(1, int(round(args.ttm_start / dt)) - args.steps)
        lib.fmd_dync_integrate(md, -1, (n_pre - 0.5) * dt, dt)
        field_te = lib.fmd_field_find(md, h, api.FMD_FIELD_TTM_TE)
        dev = C.c_void_p(L.fmdx_device(md))
        # e2e: one fmd_dync_integrate call over the K steps, as the
        # reference's TTM examples run it, with an event handler that reads
        # the electron-temperature field array back at every field update
        # (every step)
        arr = C.c_void_p()
        dims = (C.c_uint * 3)()
        reads = [0, 0]

        def on_event(mdp, event, usp, params):
            if event == api.FMD_EVENT_FIELD_UPDATE:
                fp = C.cast(params, C.POINTER(api.FieldUpdateParams)).contents
                if fp.turi == h and fp.field == field_te:
                    a3s = lib.fmd_field_getArray(md, h, field_te, C.byref(arr), dims)
                    lib.fmd_array3s_free(a3s)
                    reads[0] += 1
                    reads[1] += 8 * dims[0] * dims[1] * dims[2]

        handler = api.EventHandler(on_event)
        lib.fmd_setEventHandler(md, None, handler)
        t0 = time.perf_counter()
        lib.fmd_dync_integrate(md, -1, (args.steps - 0.5) * dt, dt)
        t1 = time.perf_counter()
        lib.fmd_setEventHandler(md, None, api.EventHandler())
        e2e_value = natoms * args.steps / (t1 - t0)
        te_bytes = int(round(reads[1] / max(args.steps, 1)))
        # device time: K steps replayed from the captured step graph
        ck(L.fmdg_se_steps(dev, args.warmup, dt, -1), "warm-up")
        ck(L.fmdg_sync(dev), "sync")
        sampler = ClockSampler()
        sampler.start()
        lc0, lc1 = C.c_longlong(0), C.c_longlong(0)
        L.fmdg_launch_count(dev, C.byref(lc0))
        ms = C.c_float(0.0)
        ck(L.fmdg_timer_start(dev), "timer")
        ck(L.fmdg_se_steps(dev, args.steps, dt, -1), "steps")
        ck(L.fmdg_timer_stop(dev, C.byref(ms)), "timer")
        L.fmdg_launch_count(dev, C.byref(lc1))
        clocks = sampler.stop()
        ck(L.fmdg_set_profiling(dev, 1), "prof")
        nprof = max(3, min(10, args.steps))
        ck(L.fmdg_se_steps(dev, nprof, dt, -1), "profile")
        phases = {}
        for ph in ("bin", "turi", "ttm", "force"):
            pms, pn = C.c_float(0.0), C.c_int(0)
            L.fmdg_get_profile(dev, ph.encode(), C.byref(pms), C.byref(pn))
            phases[ph] = pms.value / max(pn.value, 1)
        ck(L.fmdg_set_profiling(dev, 0), "prof")
        peak32 = C.c_double(0)
        ck(L.fmdg_measure_fma_peak(dev, 0, C.byref(peak32)), "peak")
        errs = C.c_uint(0)
        L.fmdg_get_errors(dev, C.byref(errs), 0)
        ttm = lib.ttm_1d(md)
        lib.fmd_free(md)
    te = np.asarray(ttm["Te"])
    peak, src = hbm_peak_gbs()
    ms_per_step = ms.value / args.steps
    field_gbs = TTM_FIELD_BYTES * natoms / (phases["turi"] * 1e-3) / 1e9
    kick_gbs = SE_KICK_BYTES * natoms / (phases["bin"] * 1e-3) / 1e9
    force_tf = natoms * (FLOP_DENSITY + FLOP_FORCE) / (phases["force"] * 1e-3) / 1e12
    cores = os.cpu_count() or 1
    if args.skip_cpu:
        cpu_value, cpu_steps = None, 0
    else:
        cpu_value, cpu_steps = cpu_port_ttm(cores)
    return {
        "metric": "atom-steps/s", "value": natoms / (ms_per_step * 1e-3), "unit": "atom-steps/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-compute/f64-accumulate (Te f64)", "data": "synthetic",
        "config": dict(ttm_config(), t_start_ps=args.ttm_start), "gpu_launches": int(lc1.value - lc0.value),
        "phases_ms": phases,
        "roofline": {"bound": "hbm", "kernel": "k_turi_pass_a + k_turi_pass_b (turi field passes; with the "
                                              "cell clears and finishes of the phase)",
                     "achieved": field_gbs, "peak": peak, "unit": "GB/s", "frac": field_gbs / peak,
                     "peak_source": src, "algorithmic_bytes_per_atom": TTM_FIELD_BYTES, "traffic": None},
        "hbm_kernels": {"kick_drift_refresh": {"achieved_gbs": kick_gbs, "frac": kick_gbs / peak,
                                               "algorithmic_bytes_per_atom": SE_KICK_BYTES,
                                               "note": "k_bin_classify (kick-drift) + the reference-order "
                                                       "refresh kernels; bytes of the kick-drift only"},
                        "ttm_solver_ms": phases["ttm"]},
        "roofline_force": {"bound": "fp32-issue", "kernel": "neighbour list + EAM density + pair forces",
                           "achieved": force_tf, "peak": peak32.value, "unit": "TFLOP/s",
                           "frac": force_tf / peak32.value},
        "clocks": clocks, "device_errors": errs.value,
        "te_max_k": float(te[te >= 0].max()) if (te >= 0).any() else None,
        "e2e": {"value": e2e_value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": te_bytes,
                "how": "one fmd_dync_integrate call over the K steps through the fmd.h API (the state stays "
                       "resident), an event handler reading the electron-temperature field array back at every "
                       "field update (every step); wall clock",
                "te_reads": reads[0]},
        "cpu_baseline": {"value": cpu_value, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{cpu_steps} velocity-Verlet steps of the 256000-atom EAM system (the "
                                   "oracle port has no TTM solver: the EAM part of the step)"},
    }


# ---------------------------------------------------------------- served stream
METRIC = "atom-steps/s on 1 GB300, batched-served vs plain at ≤1e-5 force err; p50/p99"
SERVED_JOBS = 2048
SERVED_STEP_SCALE = 1.0
FLEET_CHUNK = 8      # velocity-Verlet steps of every resident job per timed fleet step
PLAIN_EVERY = 16     # plain arm: every 16th job of the stream
PLAIN_STEPS = 200    # plain arm: steps timed per sampled job after its first
REF_EVERY = 16       # reference arm and cpu_baseline: every 16th job of the stream


def served_config(args):
    scale = "" if args.step_scale == 1.0 else f"; step counts and arrival times x {args.step_scale}"
    return {"workload": f"served job stream, {args.jobs} jobs (seed 5): FCC cubes 500-200000 atoms log-uniform, "
                        "LJ argon / Morse copper / analytic-EAM copper, 50-1200 K, 1000-20000 steps, "
                        "Poisson arrivals at 50/s" + scale,
            "jobs": args.jobs, "step_scale": args.step_scale, "precision": "mixed",
            "step": f"value: {FLEET_CHUNK} velocity-Verlet steps of every job of the stream, all resident "
                    "(no job reaches its last step, so the timed steps form no thermo record); "
                    "e2e: the whole stream",
            "l2": "fleet working set (tens of GB) larger than L2, no flush needed"}


def served_jobs(args, atoms=True, every=1):
    """The stream's job descriptions (every `every`-th job), with their
    atoms unless atoms=False."""
    from fmd_gb300 import serve
    jobs = serve.served_stream(args.jobs, seed=5, step_scale=args.step_scale)[::every]
    if atoms:
        for j in jobs:
            j["x"], j["v"], j["l"] = serve.job_atoms(j)
    return jobs


def cpu_port_job(j, threads, setfl, max_atom_steps=4.0e6, max_steps=10):
    """The CPU oracle port (restated reference algorithm, OpenMP, per-thread
    buffers) on one job of the stream: set-up and initial forces untimed,
    then k velocity-Verlet steps timed (k bounded by max_atom_steps);
    returns (atom-steps, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from fmd_gb300 import serve
    if "x" not in j:
        j["x"], j["v"], j["l"] = serve.job_atoms(j)
    P = serve.POTENTIALS[j["pot"]]
    nc, cellh, order, counts = serve.host_binning(j["x"], j["l"], P["rc"])
    if j["pot"] == "lj":
        pots = [("lj", 0, 0, 3.405, 0.0104, 8.5125)]
    elif j["pot"] == "morse":
        pots = [("morse", 0, 0, 0.3429, 1.3588, 2.866, 8.0)]
    else:
        pots = [("eam", 0, 0)]
    o = pyoracle.Oracle(threads=threads)
    o.setup([j["l"]] * 3, [1, 1, 1], [nc] * 3, [cellh] * 3, [("Cu", P["mass"])], pots,
            setfl if j["pot"] == "eam" else None)
    n = len(order)
    cell = np.repeat(np.arange(nc ** 3, dtype=np.int32), counts)
    o.upload(cell, j["x"][order], j["v"][order], np.zeros(n, np.uint32), np.zeros(n, np.int32),
             order.astype(np.uint32), nc ** 3)
    o.forces(-1)
    k = int(max(1, min(max_steps, j["steps"], max_atom_steps // n)))
    t0 = time.perf_counter()
    o.vv(k, P["dt"])
    dt = time.perf_counter() - t0
    o.close()
    return float(n * k), dt


def cpu_port_jobs(jobs, threads, budget_s=12.0):
    """cpu_port_job over the given jobs, one at a time, until budget_s of
    timed CPU work; returns (atom-steps/s, one-line description)."""
    from fmd_gb300 import workloads
    done_as, spent, used = 0.0, 0.0, {}
    with tempfile.TemporaryDirectory() as work:
        setfl = workloads.write_analytic_eam(os.path.join(work, "analytic.eam.alloy"))
        for j in jobs:
            if spent >= budget_s:
                break
            a, t = cpu_port_job(j, threads, setfl)
            done_as += a
            spent += t
            used[j["pot"]] = used.get(j["pot"], 0) + 1
    desc = (f"{sum(used.values())} jobs of the stream (every {REF_EVERY}th; "
            + ", ".join(f"{v} {k}" for k, v in sorted(used.items()))
            + f"), one at a time, up to 10 steps or 4e6 atom-steps each, {threads} threads")
    return done_as / spent, desc


def plain_sample(L, eam, jobs, every=PLAIN_EVERY, nsteps=PLAIN_STEPS):
    """The plain arm: jobs of the stream one at a time through the plain
    single-system binary64 path (the path libfmd.so's fmd_dync_integrate
    drives).  Every `every`-th job: set-up plus its first step timed as a
    fixed cost, then up to `nsteps` steps timed; the job's time is the fixed
    cost plus the per-step time times its remaining steps (the plain path
    rebuilds its exact neighbour list every step, so a step costs the same
    all along).  Returns (atom-steps/s, details)."""
    from fmd_gb300 import serve
    t_total, as_total, timed_s = 0.0, 0.0, 0.0
    drifts = []
    for j in jobs[::every]:
        t0 = time.perf_counter()
        one = serve.Single(L, j["pot"], j["x"], j["v"], j["l"], precision=serve.PREC_FP64, eam=eam)
        one.steps(1)
        one.thermo()                        # synchronises
        t1 = time.perf_counter()
        k = min(nsteps, j["steps"] - 1)
        if k > 0:
            one.steps(k)
            t = one.thermo()
        else:
            t = one.thermo()
        t2 = time.perf_counter()
        e0 = one.th0.kinetic + one.th0.potential
        drifts.append(abs(t.kinetic + t.potential - e0) / abs(e0))
        one.close()
        t_total += (t1 - t0) + ((t2 - t1) * (j["steps"] - 1) / k if k > 0 else 0.0)
        as_total += float(len(j["x"])) * j["steps"]
        timed_s += t2 - t0
    return as_total / t_total, {"jobs": len(jobs[::every]), "every": every, "steps_timed_per_job": nsteps,
                                "seconds_timed": timed_s, "seconds_extrapolated": t_total,
                                "median_rel_energy_drift": float(np.median(drifts))}


def served_force_errors(L, eam, jobs, per_pot=3, max_atoms=40000):
    """Max relative force error of the served (packed, mixed-precision)
    kernels against the binary64 path at identical positions: per
    potential the coldest jobs of the stream up to max_atoms atoms (cold
    crystals have the smallest net forces, the largest relative errors)
    and the first job; each runs 24 packed steps, then the binary64
    single-system path evaluates the forces at the job's final positions.
    Returns {potential: max error}."""
    from fmd_gb300 import serve
    out = {}
    for p in serve.POT_NAMES:
        mine = [j for j in jobs if j["pot"] == p and len(j["x"]) <= max_atoms]
        pick = sorted(mine, key=lambda j: j["T"])[:per_pot] + [next(j for j in jobs if j["pot"] == p)]
        worst = 0.0
        for j in pick:
            srv = serve.Server(L, chunk_steps=8, eam=eam)
            jid = srv.submit(p, j["x"], j["v"], j["l"], 24, precision=serve.PREC_MIXED, keep_state=True)
            srv.drain()
            xp, vp, Fp, _ = srv.state(jid, len(j["x"]))
            srv.close()
            # the binary64 forces at the same positions: Single numbers the
            # atoms by their row in xp
            one = serve.Single(L, p, xp, vp, j["l"], precision=serve.PREC_FP64, eam=eam)
            _, _, F64, rows = one.state()
            one.close()
            Fb = np.zeros_like(F64)
            Fb[rows] = F64
            worst = max(worst, float(np.abs(Fp - Fb).max() / np.abs(Fb).max()))
        out[p] = worst
    return out


def run_served(args):
    import fmd_gb300
    from fmd_gb300 import serve
    L = serve.bind(fmd_gb300.load())
    eam = serve.eam_tables(L)
    jobs = served_jobs(args)
    n_atoms = sum(len(j["x"]) for j in jobs)
    K, W = args.steps, args.warmup

    # --- value: the whole stream resident in HBM, K fleet steps of
    # FLEET_CHUNK velocity-Verlet steps of every job --------------------
    fleet = serve.Server(L, budget_bytes=240 << 30, max_jobs=len(jobs) + 1, chunk_steps=FLEET_CHUNK, eam=eam)
    for j in jobs:
        fleet.submit(j["pot"], j["x"], j["v"], j["l"], (W + K + 2) * FLEET_CHUNK, precision=serve.PREC_MIXED)
    fleet.admit()
    st = fleet.stats()
    assert st.running == len(jobs), "the stream does not fit the fleet budget"
    fleet_bytes = st.bytes_in_use
    for _ in range(W):              # warm-up; the autotuner picks block sizes here
        fleet.run_resident(1)
    sampler = ClockSampler()
    sampler.start()
    k0 = fleet.stats().kernels
    ms = fleet.run_resident(K)
    k1 = fleet.stats().kernels
    clocks = sampler.stop()
    tuned = {p: fleet.stats().pack_fblk[serve.POTENTIALS[p]["cat"]][1] for p in serve.POT_NAMES}
    phases = {}
    for p in serve.POT_NAMES:
        pm, atoms, members = fleet.profile_pack(p)
        phases[p] = {"bin_ms": pm[0], "nlist_ms": pm[1], "density_ms": pm[2], "force_ms": pm[3],
                     "atoms": atoms, "jobs": members, "threads_per_block": tuned[p]}
    fleet.close()
    value = n_atoms * K * FLEET_CHUNK / (ms * 1e-3)
    if args.only == "fleet":
        return {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": 1, "steps": K,
                "warmup": W, "ms_per_step": ms / K, "config": served_config(args), "gpu_launches": int(k1 - k0),
                "phases": phases, "clocks": clocks, "note": "resident fleet only (--only fleet)"}
    # peak of the binary32 FMA pipe (measured microkernel)
    h = C.c_void_p()
    serve.check(L, L.fmdg_create(C.byref(h), 0), "create")
    peak32 = C.c_double()
    serve.check(L, L.fmdg_measure_fma_peak(h, 0, C.byref(peak32)), "peak")
    L.fmdg_destroy(h)
    dom = max(serve.POT_NAMES, key=lambda p: phases[p]["force_ms"])
    fl = SERVED_FORCE_FLOP[dom] * phases[dom]["atoms"]
    achieved = fl / (phases[dom]["force_ms"] * 1e-3) / 1e12

    # --- e2e: the stream through the request loop ------------------------
    srv = serve.Server(L, budget_bytes=64 << 30, max_jobs=1024, chunk_steps=32, eam=eam)
    ids = [None] * len(jobs)
    nxt = 0
    sampler_e2e = ClockSampler()
    sampler_e2e.start()
    t0 = srv.now()
    active = 0
    while nxt < len(jobs) or active > 0:
        now = srv.now() - t0
        while nxt < len(jobs) and jobs[nxt]["arrival"] <= now:
            j = jobs[nxt]
            ids[nxt] = srv.submit(j["pot"], j["x"], j["v"], j["l"], j["steps"], precision=serve.PREC_MIXED)
            nxt += 1
        if active == 0 and nxt < len(jobs) and srv.stats().queued == 0:
            wait_s = jobs[nxt]["arrival"] - (srv.now() - t0)
            if wait_s > 0:
                time.sleep(min(wait_s, 0.01))
        active = srv.progress(wait=(nxt >= len(jobs)))
    clocks_e2e = sampler_e2e.stop()
    res = [srv.result(i) for i in ids]
    sst = srv.stats()
    srv.close()
    assert all(r.state == 2 for r in res), "a served job failed"
    errbits = int(np.bitwise_or.reduce([r.errbits for r in res]))
    job_as = np.array([r.n * r.steps for r in res], dtype=np.float64)
    arr = np.array([j["arrival"] for j in jobs]) + 0.0
    done = np.array([r.t_done for r in res]) - t0
    lat = done - arr
    span = done.max() - arr.min()
    e2e_value = job_as.sum() / span
    total_steps = sum(j["steps"] for j in jobs)
    h2d = sum(len(j["x"]) * (6 * 8 + 4) for j in jobs)
    d2h = len(jobs) * 2 * 64

    def drift(r):
        e0 = r.first.kinetic + r.first.potential
        e1 = r.last.kinetic + r.last.potential
        return abs(e1 - e0) / abs(e0)

    # jobs whose run raised a device error bit (the configured analytic EAM
    # collapses the crystal; a job that runs long enough drives its density
    # past the F(rho) table, as the reference's run would) leave the drift
    # statistic and are counted per potential
    bad_jobs = {p: 0 for p in serve.POT_NAMES}
    drifts = []
    for j, r in zip(jobs, res):
        if r.errbits:
            bad_jobs[j["pot"]] += 1
        else:
            drifts.append(drift(r))
    drifts = [d for d in drifts if np.isfinite(d)]
    served_drift = float(np.median(drifts)) if drifts else None

    # --- plain: jobs one at a time, binary64 single-system path ------------
    plain_value, plain = plain_sample(L, eam, jobs)

    ferr = served_force_errors(L, eam, jobs)

    cores = os.cpu_count() or 1
    if args.skip_cpu:
        cpu_value, cpu_sample = None, "skipped"
    else:
        cpu_value, cpu_sample = cpu_port_jobs(jobs[::REF_EVERY], cores)
    out = {
        "metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": 1,
        "steps": K, "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-compute/f64-accumulate", "data": "synthetic",
        "served_over_plain_fp64": e2e_value / plain_value,
        "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
        "max_rel_force_err_mixed_vs_fp64": max(ferr.values()),
        "median_rel_energy_drift": served_drift,
        "jobs_with_device_errors": int(sum(bad_jobs.values())),
        "e2e": {"value": e2e_value, "unit": "atom-steps/s",
                "h2d_bytes_per_step": h2d / total_steps, "d2h_bytes_per_step": d2h / total_steps,
                "how": "fmdg_srv_* request loop, jobs submitted from host arrays at their arrival times; "
                       "wall clock first arrival to last completion; bytes per job-step"},
        "plain_fp64": {"value": plain_value, "unit": "atom-steps/s", **plain},
        "config": served_config(args),
        "gpu_launches": int(k1 - k0),
        "roofline": {"bound": "fp32-issue", "kernel": f"k_force_skin<LocPack> ({dom} packs: pair forces + finish step)",
                     "achieved": achieved, "peak": peak32.value, "unit": "TFLOP/s",
                     "frac": achieved / peak32.value,
                     "peak_source": "measured FMA-chain microkernel (MEASURED_PEAKS.json has no CUDA-core peak)",
                     "traffic": (FORCE_DRAM_BYTES_PER_ATOM["morse_pack"] * phases[dom]["atoms"] if dom == "morse"
                                 else None),
                     **hbm_side(FORCE_DRAM_BYTES_PER_ATOM["morse_pack"] * phases[dom]["atoms"] if dom == "morse"
                                else None, phases[dom]["force_ms"])},
        "cpu_baseline": {"value": cpu_value, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                         "sample": cpu_sample},
        "clocks": clocks,
        "served": {"jobs": len(jobs), "atoms": n_atoms, "fleet_bytes": fleet_bytes,
                   "makespan_s": float(span), "force_err": ferr, "device_error_bits": errbits,
                   "jobs_with_device_errors": bad_jobs,
                   "drift_note": "median over the jobs without device error bits",
                   "e2e_bytes_peak": sst.bytes_peak, "threads_per_block": tuned, "clocks_e2e": clocks_e2e,
                   "graph_rebuilds": int(sum(sst.pack_rebuilds[c][m] for c in range(4) for m in range(2)))},
        "phases": phases,
    }
    return out


def run_reference(args):
    """The reference's CPU implementation of the path on the host cores: the
    oracle port (the reference's own sources are not present on the GPU
    host), all threads, same workload, metric and unit.  Each step is a
    bounded sample: one job of the stream (every REF_EVERY-th, in turn) for
    up to 10 velocity-Verlet steps (served), or up to 10 steps of the
    256 000-atom EAM system (eam256k)."""
    cores = os.cpu_count() or 1
    if args.workload == "served":
        from fmd_gb300 import workloads
        jobs = served_jobs(args, atoms=False, every=REF_EVERY)
        done_as, spent = 0.0, 0.0
        with tempfile.TemporaryDirectory() as work:
            setfl = workloads.write_analytic_eam(os.path.join(work, "analytic.eam.alloy"))
            for s in range(args.warmup + args.steps):
                j = jobs[s % len(jobs)]
                a, t = cpu_port_job(j, cores, setfl)
                if s >= args.warmup:
                    done_as += a
                    spent += t
                j.pop("x", None)
                j.pop("v", None)
        value = done_as / spent
        out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "atom-steps/s",
               "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": spent / args.steps * 1e3,
               "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": served_config(args),
               "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                                "sample": f"each step one job of the stream (every {REF_EVERY}th, in turn), "
                                          "up to 10 steps or 4e6 atom-steps"},
               "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return
    ttm = args.workload == "ttm"
    port = cpu_port_ttm if ttm else cpu_port_run
    for _ in range(args.warmup):                # untimed, short
        port(cores, target_s=1.0, max_steps=1)
    done_as, spent = 0.0, 0.0
    w = TTM if ttm else WORKLOAD
    natoms = int(np.prod(w["cells"])) * 4
    for _ in range(args.steps):
        v, k = port(cores, target_s=8.0, max_steps=10)
        done_as += natoms * k
        spent += natoms * k / v
    value = done_as / spent
    out = {"impl": "reference", "metric": "atom-steps/s", "value": value, "unit": "atom-steps/s", "n_gpus": 0,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": spent / args.steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic",
           "config": (ttm_config() if args.workload == "ttm" else
                      {"workload": "EAM FCC 40x40x40 (256000 atoms), analytic EAM on 10000-point splines, "
                                   "300 K, dt 1 fs, NVE", "atoms": natoms}),
           "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                            "sample": ("each step up to 10 symplectic-Euler steps of the 800000-atom TTM slab "
                                       "(turi fields, TTM solver, friction term included)" if ttm else
                                       "each step up to 10 velocity-Verlet steps of the 256000-atom EAM system")},
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
    ap.add_argument("--workload", default="served", choices=["served", "eam256k", "ttm"])
    ap.add_argument("--ttm-start", type=float, default=TTM["t_start"],
                    help="ttm: simulation time (ps) at which the timed steps start")
    ap.add_argument("--only", default="all", choices=["all", "fleet"],
                    help="served: 'fleet' times the resident fleet only (profiling runs)")
    ap.add_argument("--jobs", type=int, default=SERVED_JOBS, help="served: jobs of the stream (its first jobs)")
    ap.add_argument("--step-scale", type=float, default=SERVED_STEP_SCALE,
                    help="served: factor on step counts and arrival times")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    # Under torchrun (N > 1) rank 0 alone runs and prints; the engine uses
    # one GPU (multi-GPU serving is not built), and its line says n_gpus 1
    if int(os.environ.get("RANK", "0")) != 0:
        return
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload == "served":
        out = run_served(args)
    elif args.workload == "ttm":
        out = run_ttm(args)
    else:
        out = run_ours(args)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
