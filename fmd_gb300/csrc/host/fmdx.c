/*
 * fmdx_*: extensions exported by libfmd.so beyond fmd.h -- per-atom state
 * in cell order for parity tests, the device handle for kernel-level
 * benchmarks, precision mode and seeding.  They have no counterpart in the
 * reference's public header; the per-atom dump mirrors what a white-box
 * walk of the reference's cells (src/cell.h:40-58) shows.
 */
#include <stdlib.h>
#include <string.h>
#include "fmd_private.h"

int fmdx_natoms(fmd_t *md)
{
    if (!md->ParticlesDistributed) return -1;
    int n = 0;
    if (fmdg_natoms(md->dev, &n)) return -1;
    return n;
}

void fmdx_grid(fmd_t *md, int *nc, double *cellh, double *l, int *pbc)
{
    for (int d = 0; d < 3; d++)
    {
        nc[d] = md->nc[d];
        cellh[d] = md->cellh[d];
        l[d] = md->l[d];
        pbc[d] = md->PBC[d];
    }
}

int fmdx_dump(fmd_t *md, int *cell, unsigned *atomid, unsigned *kind, int *group,
              double *x, double *v, double *F, double *vaream)
{
    if (!md->ParticlesDistributed) return -1;
    int n = 0;
    if (fmdg_natoms(md->dev, &n)) return -1;
    if (fmdg_download(md->dev, cell, x, v, F, vaream, kind, group, atomid)) return -1;
    return n;
}

void fmdx_set_state(fmd_t *md, const double *x, const double *v)
{
    if (!md->ParticlesDistributed) return;
    _fmdh_dev_ok(md, fmdg_set_state(md->dev, x, v), "fmdg_set_state");
    md->KineticEnergyUpdated = false;
}

void fmdx_refresh(fmd_t *md)
{
    if (!md->ParticlesDistributed) return;
    _fmdh_dev_ok(md, fmdg_refresh(md->dev), "fmdg_refresh");
}

void fmdx_update_forces(fmd_t *md)
{
    if (!md->ParticlesDistributed) return;
    if (_fmdh_dev_ok(md, fmdg_compute_forces(md->dev, md->ActiveGroup), "fmdg_compute_forces"))
        md->thermo_pending = true;
}

double fmdx_potential_energy(fmd_t *md)
{
    if (md->thermo_pending) _fmdh_thermo_from_device(md);
    return md->GroupPotentialEnergy;
}

/* pair virial sum r_ij . F_ij of the last force evaluation (eV; no
   counterpart in the reference) */
double fmdx_virial(fmd_t *md)
{
    if (md->thermo_pending) _fmdh_thermo_from_device(md);
    return md->GroupVirial;
}

int fmdx_time_iteration(fmd_t *md) { return md->time_iteration; }

fmdg_sys_t *fmdx_device(fmd_t *md) { return md->dev; }

/* FMDG_PREC_FP64 (0) or FMDG_PREC_MIXED (1); takes effect at the next run */
void fmdx_set_precision(fmd_t *md, int mode)
{
    md->precision = mode;
    md->dev_tables_ok = false;
}

/* distribute the atoms to the device without running (first half of
   fmd_dync_integrate) */
int fmdx_distribute(fmd_t *md) { return _fmdh_distribute(md) ? 0 : -1; }

/* Tables of an EAM potential loaded with fmd_pot_eam_alloy_load in the
   layout of fmdg_set_eam (for callers that drive the device engine or the
   served mode directly).  Sizes only when F is NULL.  Returns 0, or -1
   when pot is not an EAM potential. */
int fmdx_eam_tables(fmd_pot_t *pot, int *nelem, int *Nrho, double *drho, int *Nr2, double *dr2,
                    double *cutoff_sqr, double *F, double *F_DD, double *rho, double *rhoDD, double *phi,
                    double *phiDD)
{
    if (pot == NULL || pot->cat != POTCAT_EAM) return -1;
    const eam_t *e = (const eam_t *)pot->data;
    *nelem = e->nelem;
    *Nrho = e->Nrho;
    *drho = e->drho;
    *Nr2 = e->Nr2;
    *dr2 = e->dr2;
    *cutoff_sqr = e->cutoff_sqr;
    if (F != NULL) _fmdh_eam_flatten(e, F, F_DD, rho, rhoDD, phi, phiDD);
    return 0;
}
