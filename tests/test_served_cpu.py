"""Host-side parts of the served mode that run without a GPU: the job
stream's distributions and the EAM tables handed to the server."""
import math

import numpy as np

from fmd_gb300 import serve, workloads


def test_stream_distribution():
    jobs = serve.served_stream(2048, seed=5)
    assert len(jobs) == 2048
    n = np.array([j["natoms"] for j in jobs])
    assert n.min() >= 500 and n.max() <= 4 * 37 ** 3
    # log-uniform sizes: median near sqrt(500*200000)
    assert 5e3 < np.median(n) < 2e4
    arr = np.array([j["arrival"] for j in jobs])
    assert np.all(np.diff(arr) > 0)
    assert abs(2048 / arr[-1] - 50.0) < 5.0
    pots = [j["pot"] for j in jobs]
    for p in serve.POT_NAMES:
        assert 0.28 < pots.count(p) / 2048 < 0.39
    for j in jobs:
        P = serve.POTENTIALS[j["pot"]]
        assert j["ncell"] * P["a"] > 2 * P["rc"]
        assert 1000 <= j["steps"] <= 20000
        assert 50.0 <= j["T"] <= 1200.0
        assert j["dt"] == P["dt"]


def test_stream_scaling_keeps_order():
    a = serve.served_stream(64, seed=5)
    b = serve.served_stream(64, seed=5, step_scale=0.05)
    for x, y in zip(a, b):
        assert x["natoms"] == y["natoms"] and x["pot"] == y["pot"]
        assert math.isclose(y["arrival"], 0.05 * x["arrival"])
        assert y["steps"] == max(1, round(0.05 * x["steps"]))


def test_job_atoms_inside_box():
    for j in serve.served_stream(30, seed=7):
        x, v, l = serve.job_atoms(j)
        assert len(x) == j["natoms"]
        assert x.min() >= 0.0 and x.max() < l
        m = serve.POTENTIALS[j["pot"]]["mass"]
        assert np.abs((v * m).sum(axis=0)).max() < 1e-9 * np.abs(v * m).sum()


def test_hybrid_job_geometry_and_table():
    """A "cuar" job: both blocks inside the periodic box, no two atoms
    closer than 3.5 A across the interfaces or the periodic faces, every
    periodic length above twice the largest cutoff, and a symmetric
    two-kind pair table with EAM only between copper atoms."""
    for n in (5, 6, 9):
        x, v, kind, l = serve.hybrid_atoms(dict(ncell=n, T=300.0, seed=3))
        assert x.min() >= 0.0 and np.all(x.max(axis=0) < l)
        assert np.all(l > 2 * serve.job_rc("cuar"))
        assert (kind == 0).sum() == 4 * n ** 3
        cu, ar = x[kind == 0], x[kind == 1]
        d = cu[:, None, :] - ar[None, :, :]
        d -= l * np.round(d / l)
        assert np.sqrt((d * d).sum(-1)).min() > 3.5
    mass, elem, table = serve.job_table("cuar")
    assert list(elem) == [0, -1]
    cats = [[table[a * 2 + b].cat for b in range(2)] for a in range(2)]
    assert cats == [[serve.FMDG_POT_EAM, serve.FMDG_POT_LJ], [serve.FMDG_POT_LJ, serve.FMDG_POT_LJ]]
    assert list(table[1].p) == list(table[2].p)
    assert abs(table[0].p[2] - workloads.EAM_RC ** 2) < 1e-12


def test_host_binning_order():
    j = dict(pot="morse", ncell=5, T=300.0, seed=3)
    x, v, l = serve.job_atoms(j)
    nc, cellh, order, counts = serve.host_binning(x, l, 8.0)
    assert nc == 2 and counts.sum() == len(x)
    ic = np.floor(x[order] / cellh).astype(int)
    flat = ic[:, 2] + nc * (ic[:, 1] + nc * ic[:, 0])
    assert np.all(np.diff(flat) >= 0)


def test_eam_tables_from_host_library(lib):
    L = serve.bind(lib.L)
    t = serve.eam_tables(L)
    assert t["nelem"] == 1 and t["Nrho"] == workloads.EAM_NRHO
    assert t["Nr2"] == workloads.EAM_NR + 2
    assert abs(t["cutoff_sqr"] - workloads.EAM_RC ** 2) < 1e-9
    f, phi, F = workloads.analytic_eam_functions()
    rho = np.arange(t["Nrho"]) * t["drho"]
    assert np.allclose(t["F"], F(rho), rtol=1e-12, atol=1e-12)
