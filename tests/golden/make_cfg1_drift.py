"""The oracle's NVE energy drift on the full-size EAM configuration, for
tests/test_full_configs_gpu.py::test_eam256k_full_size.

256 000 copper atoms (FCC 40 x 40 x 40 cells, a = 3.615 A, periodic),
the analytic EAM on 10 000-point splines, Maxwell velocities at 300 K from
seed 2 (fmd_gb300.workloads.fcc_state), dt = 1 fs, up to 5000
velocity-Verlet steps, total energy sampled every 250 steps; the drift is
taken over the first 2000 steps (the potential collapses the crystal and
the run stops before step 5000, for the reference as here).  Run by the CPU oracle
(oracle/fmd_oracle.c, binary64, OpenMP with per-thread buffers): ten
minutes or so of host time, so the result is recorded here instead of
being recomputed by every GPU test run.

    python tests/golden/make_cfg1_drift.py      # writes tests/golden/cfg1_drift.json
"""
import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from fmd_gb300 import workloads  # noqa: E402
import pyoracle  # noqa: E402

CELLS, A, T, SEED, MASS, DT = 40, 3.615, 300.0, 2, 63.546, 0.001
STEPS, EVERY = 5000, 250
# The analytic EAM has no equilibrium near 3.615 A: the crystal collapses
# locally after ~1000 steps and the run turns violent (the oracle's run
# stops with an atom beyond its neighbouring cell before step 5000); the
# drift is compared over the first WINDOW steps, and the whole record is kept
WINDOW = 2000


def main():
    x, v = workloads.fcc_state(CELLS, CELLS, CELLS, A, T, MASS, seed=SEED)
    l = CELLS * A
    nc = int(l / workloads.EAM_RC)
    cellh = l / nc
    ic = np.floor(x / cellh).astype(np.int64)
    cell = ic[:, 2] + nc * (ic[:, 1] + nc * ic[:, 0])
    order = np.argsort(cell, kind="stable")
    n = len(x)
    t0 = time.time()
    with tempfile.TemporaryDirectory() as work:
        setfl = workloads.write_analytic_eam(os.path.join(work, "a.eam.alloy"))
        o = pyoracle.Oracle(threads=os.cpu_count() or 1)
        o.setup([l] * 3, [1, 1, 1], [nc] * 3, [cellh] * 3, [("Cu", MASS)], [("eam", 0, 0)], setfl)
    o.upload(cell[order].astype(np.int32), x[order], v[order], np.zeros(n, np.uint32), np.zeros(n, np.int32),
             order.astype(np.uint32), nc ** 3)
    o.forces(-1)
    th = o.thermo(-1)
    es, temps = [th.kinetic + th.potential], [th.temperature]
    failed_at = None
    for k in range(STEPS // EVERY):
        if o.vv(EVERY, DT) != 0:
            failed_at = (k + 1) * EVERY     # a refresh found an atom beyond its neighbouring cell
            break
        th = o.get_thermo()
        es.append(th.kinetic + th.potential)
        temps.append(th.temperature)
        print((k + 1) * EVERY, es[-1], th.temperature, flush=True)
    o.close()
    e = np.array(es[:WINDOW // EVERY + 1])
    drift = float(np.abs(e - e[0]).max() / abs(e[0]))
    out = dict(config="EAM 256000 atoms (FCC 40^3, a 3.615 A, 300 K seed 2, dt 1 fs), NVE",
               steps=WINDOW, every=EVERY, energies=es, temperatures=temps, drift=drift,
               run_steps=STEPS, failed_at_step=failed_at, seconds=time.time() - t0, threads=os.cpu_count())
    with open(os.path.join(HERE, "cfg1_drift.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({k: out[k] for k in ("drift", "seconds", "threads")}))


if __name__ == "__main__":
    main()
