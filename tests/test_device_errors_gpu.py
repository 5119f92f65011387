"""Device-side error detection turned into the reference's error events,
without any GPU fault: the kernels test their inputs, record sticky error
bits, skip the offending access and carry on; the host reads the bits after
a batch of steps and raises FMD_EVENT_ERROR (src/error.c) with the
reference's error codes.

* an atom placed beyond the neighbouring cells -> FMD_ERR_UNEXPECTED_POSITION
  (src/misc.c:286-290);
* an EAM density beyond the F(rho) table -> FMD_ERR_OUTSIDE_REAL_INTERVAL
  (src/eam.c:168-171);
* the same EAM fault in a served job: the job completes and reports the bit.
"""
import tempfile

import numpy as np
import pytest

import cases
from fmd_gb300 import api, serve

pytestmark = pytest.mark.gpu

FMD_ERR_UNEXPECTED_POSITION = 1        # enum fmd_error_t (src/fmd.h)
FMD_ERR_OUTSIDE_REAL_INTERVAL = 5


def _errors_after(lib, name, edit, duration):
    with tempfile.TemporaryDirectory() as work:
        md, _ = cases.setup(lib, name, work)
        rec = cases.Recorder(lib)
        lib.fmd_setEventHandler(md, None, rec.cb)
        dt = cases.CASES[name]["run"][2]
        lib.fmd_dync_integrate(md, -1, 0.0, dt)
        assert rec.errors == []
        d = lib.dump(md)
        x = d["x"].copy()
        edit(x, lib.grid(md))
        lib.set_state(md, x, None)
        lib.fmd_dync_integrate(md, -1, duration, dt)
        errs = list(rec.errors)
        # the engine stays usable after the event
        lib.fmd_dync_integrate(md, -1, duration, dt)
        lib.fmd_free(md)
    return errs


def test_position_error_event(gpu_lib):
    def edit(x, grid):
        nc, cellh, l, pbc = grid
        x[0, 0] = -3.0 * cellh[0]
    errs = _errors_after(gpu_lib, "lj", edit, 0.0019)
    assert (FMD_ERR_UNEXPECTED_POSITION, True) in errs, errs


# five atoms moved to within 0.02 A of atom 0: its density gains ~26 per
# such neighbour (f(r) -> e^3.3 as r -> 0), ~132 in all, and leaves the
# 0-120 F(rho) table
CLUSTER = np.array([[0.02, 0.0, 0.0], [0.0, 0.02, 0.0], [0.0, 0.0, 0.02], [-0.02, 0.0, 0.0], [0.0, -0.02, 0.0]])


def test_eam_density_range_error_event(gpu_lib):
    def edit(x, grid):
        x[1:6] = x[0] + CLUSTER
    errs = _errors_after(gpu_lib, "eam", edit, 0.00095)
    assert (FMD_ERR_OUTSIDE_REAL_INTERVAL, True) in errs, errs


def test_served_job_reports_device_errors(gpu_lib):
    L = serve.bind(gpu_lib.L)
    eam = serve.eam_tables(L)
    j = dict(pot="eam", ncell=6, T=300.0, seed=91)
    x, v, l = serve.job_atoms(j)
    x = x.copy()
    x[1:6] = x[0] + CLUSTER
    srv = serve.Server(L, chunk_steps=4, eam=eam)
    bad = srv.submit("eam", x, v, l, 4)
    xg, vg, lg = serve.job_atoms(dict(j, seed=92))
    good = srv.submit("eam", xg, vg, lg, 4)
    srv.drain()
    rb, rg = srv.result(bad), srv.result(good)
    assert rb.state == 2 and (rb.errbits & 0x2)
    assert rg.state == 2 and rg.errbits == 0
    srv.close()
