"""Synthetic workload builders shared by the benchmark and the tests.

* `write_analytic_eam` writes the analytic EAM of the 256 000-atom EAM
  workload as a DYNAMO setfl (eam/alloy) file, the only EAM input format the
  FMD API accepts (`fmd_pot_eam_alloy_load`, reference src/eam.c:376-555).
* `fcc_state` builds an FCC cuboid with the lattice convention of the
  reference's lattice builder (src/structure.c:53-136: site = origin +
  (cell + 0.25 + basis) * a, cells in x-major / z-fastest order) and seeded
  Maxwell-Boltzmann velocities with the net momentum removed
  (src/structure.c:33-51).  The reference seeds its generator from the wall
  clock, so seeded states are produced here and loaded through
  `fmd_io_loadState` by every implementation under test.
"""
from __future__ import annotations

import numpy as np

K_BOLTZMANN = 8.6173303e-5        # eV/K            (src/general.h:47)
MD_MASS_UNIT = 9.6485332907e+03   # Da per internal mass unit (src/general.h:37)

# analytic EAM of the 256 000-atom workload (Cu-like, a = 3.615 A)
EAM_R_E = 2.556
EAM_BETA = 3.3
EAM_D = 0.35
EAM_ALPHA = 1.36
EAM_F0 = 1.1
EAM_RC = 5.5
EAM_TAPER_START = 5.0     # cubic switching function on [5.0, 5.5] A for phi and f
EAM_NR = 10000
EAM_NRHO = 10000
# rho grid 0 .. 119.988.  The lattice value at a = 3.615 A is ~16, but this
# potential has no equilibrium near 3.615 A: its energy per atom falls
# monotonically as the lattice contracts, down to a ~ 2.7 A (rho ~ 49), so a
# periodic crystal at 3.615 A is under ~ -74 GPa and collapses locally after
# ~10^3 steps, densities reaching 45-50; the table covers them with margin
EAM_DRHO = 0.012


def _taper(r):
    t = np.clip((r - EAM_TAPER_START) / (EAM_RC - EAM_TAPER_START), 0.0, 1.0)
    return 1.0 - 3.0 * t * t + 2.0 * t * t * t


def analytic_eam_functions():
    """(f(r), phi(r), F(rho)) of the analytic EAM as numpy callables."""
    def f(r):
        return np.exp(-EAM_BETA * (r / EAM_R_E - 1.0)) * _taper(r)

    def phi(r):
        e = np.exp(-EAM_ALPHA * (r - EAM_R_E))
        return EAM_D * (e * e - 2.0 * e) * _taper(r)

    def F(rho):
        return -EAM_F0 * np.sqrt(np.maximum(rho, 0.0))

    return f, phi, F


def write_analytic_eam(path, element="Cu", mass=63.546, lattice=3.615):
    """Write the analytic EAM as a single-element setfl file.

    r grid: Nr = 10000 points, dr = 5.5/9999 (the loader pads Nr by 2 and
    needs (Nr+1)*dr > cutoff, src/eam.c:412-415); rho grid: Nrho = 10000,
    drho = 0.012.  The pair block stores r*phi(r) as the format requires.
    """
    f, phi, F = analytic_eam_functions()
    dr = EAM_RC / (EAM_NR - 1)
    r = np.arange(EAM_NR) * dr
    rho = np.arange(EAM_NRHO) * EAM_DRHO
    with open(path, "w") as fp:
        fp.write("analytic EAM: f=exp(-3.3(r/2.556-1)), phi=0.35[exp(-2.72(r-2.556))-2exp(-1.36(r-2.556))],\n")
        fp.write("F=-1.1 sqrt(rho); f and phi multiplied by a cubic switch on [5.0, 5.5] A\n")
        fp.write("generated by fmd_gb300.workloads\n")
        fp.write("1 %s\n" % element)
        fp.write("%d %.16e %d %.16e %.16e\n" % (EAM_NRHO, EAM_DRHO, EAM_NR, dr, EAM_RC))
        fp.write("29 %.6f %.6f fcc\n" % (mass, lattice))
        for block in (F(rho), f(r), r * phi(r)):
            for i in range(0, len(block), 5):
                fp.write(" ".join("%.16e" % v for v in block[i:i + 5]) + "\n")
    return path


FCC_BASIS = np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])


def fcc_sites(nx, ny, nz, a, origin=(0.0, 0.0, 0.0)):
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    cells = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1).astype(np.float64)
    x = (cells[:, None, :] + 0.25 + FCC_BASIS[None, :, :]) * a + np.asarray(origin, dtype=np.float64)
    return x.reshape(-1, 3)


def maxwell_velocities(n, mass_amu, T, rng):
    m = mass_amu / MD_MASS_UNIT
    v = rng.standard_normal((n, 3)) * np.sqrt(K_BOLTZMANN * T / m)
    v -= v.mean(axis=0)
    return v


def fcc_state(nx, ny, nz, a, T, mass_amu, seed, origin=(0.0, 0.0, 0.0), disp=0.0):
    """Positions and velocities of an FCC cuboid; `disp` adds a seeded
    Gaussian displacement (A) so step-0 forces are not all zero."""
    rng = np.random.default_rng(seed)
    x = fcc_sites(nx, ny, nz, a, origin)
    v = maxwell_velocities(len(x), mass_amu, T, rng)
    if disp > 0.0:
        x = x + rng.standard_normal(x.shape) * disp
    return x, v
