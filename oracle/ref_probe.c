/*
 * White-box accessors for the reference FMD library compiled as a CPU oracle
 * (test infrastructure only; built into oracle/_ref/libfmdref.so by
 * oracle/Makefile.ref, never linked into the product).
 *
 * The reference keeps its atoms in per-cell arrays inside the private
 * `struct _fmd` (src/fmd-private.h:57-114, cell layout src/cell.h:40-58).
 * These helpers walk the interior cells of the single-rank local grid in
 * storage order (src/subdomain.c:201-222: interior cells first, LOOP3D
 * order, z fastest) and copy out per-atom state, so golden vectors can be
 * produced and the restated oracle can be pinned against the reference.
 */
#include "fmd-private.h"
#include "cell.h"
#include "turi.h"
#include "ttm.h"
#include "eam.h"
#include <string.h>

void _fmd_refreshGrid(fmd_t *md);                      /* src/misc.c:268 */
void _fmd_dync_updateForces(fmd_t *md);                /* src/forces.c:332 */
void _fmd_matt_distribute(fmd_t *md);                  /* src/matter.c:399 */
void _fmd_pot_update_and_process_potcats(fmd_t *md);   /* src/potential.c:216 */

int oref_natoms(fmd_t *md)
{
    if (!md->ParticlesDistributed) return -1;
    int n = 0;
    for (unsigned ic = 0; ic < md->subd.nc; ic++) n += md->subd.grid[ic].parts_num;
    return n;
}

void oref_grid(fmd_t *md, int *nc, double *cellh, double *l, int *pbc)
{
    for (int d = 0; d < 3; d++)
    {
        nc[d] = md->nc[d];
        cellh[d] = md->cellh[d];
        l[d] = md->l[d];
        pbc[d] = md->PBC[d];
    }
}

/* per-atom dump in storage order; any output pointer may be NULL */
int oref_dump(fmd_t *md, int *cell, unsigned *atomid, unsigned *kind, int *group,
              double *x, double *v, double *F, double *vaream)
{
    int k = 0;
    for (unsigned ic = 0; ic < md->subd.nc; ic++)
    {
        cell_t *c = md->subd.grid + ic;
        for (unsigned i = 0; i < c->parts_num; i++, k++)
        {
            if (cell) cell[k] = (int)ic;
            if (atomid) atomid[k] = c->AtomID[i];
            if (kind) kind[k] = c->atomkind[i];
            if (group) group[k] = c->GroupID[i];
            for (int d = 0; d < 3; d++)
            {
                if (x) x[3 * k + d] = c->x[3 * i + d];
                if (v) v[3 * k + d] = c->v[3 * i + d];
                if (F) F[3 * k + d] = (c->F != NULL) ? c->F[3 * i + d] : 0.0;
            }
            if (vaream) vaream[k] = (c->vaream != NULL) ? c->vaream[i] : 0.0;
        }
    }
    return k;
}

/* overwrite positions/velocities of the atoms in storage order */
void oref_set_state(fmd_t *md, const double *x, const double *v)
{
    int k = 0;
    for (unsigned ic = 0; ic < md->subd.nc; ic++)
    {
        cell_t *c = md->subd.grid + ic;
        for (unsigned i = 0; i < c->parts_num; i++, k++)
            for (int d = 0; d < 3; d++)
            {
                if (x) c->x[3 * i + d] = x[3 * k + d];
                if (v) c->v[3 * i + d] = v[3 * k + d];
            }
    }
    md->KineticEnergyUpdated = false;
}

void oref_refresh(fmd_t *md) { _fmd_refreshGrid(md); }

/* distribute + process potentials + allocate force arrays, as the first
   call of fmd_dync_integrate does (src/integrators.c:287-291), without
   computing forces */
void oref_prepare(fmd_t *md)
{
    fmd_dync_integrate(md, FMD_GROUP_ALL, -1.0, 1e-3);
}

void oref_update_forces(fmd_t *md) { _fmd_dync_updateForces(md); }

double oref_potential_energy(fmd_t *md) { return md->GroupPotentialEnergy; }

int oref_time_iteration(fmd_t *md) { return md->time_iteration; }

/* 1-D TTM fields of the active TTM turi (src/ttm.h:35-90), local indexes
   including the turi margin; returns the local length or -1 */
int oref_ttm_1d(fmd_t *md, unsigned *num, double *vcm, double *Ti, double *Te, double *xi)
{
    turi_t *t = md->active_ttm_turi;
    if (t == NULL || t->ttm == NULL || t->ttm->dim != 1) return -1;
    ttm_t *ttm = t->ttm;
    int n = (int)t->tdims_local[2];
    for (int i = 0; i < n; i++)
    {
        if (num) num[i] = ttm->num_1d[i];
        if (Ti) Ti[i] = ttm->Ti_1d[i];
        if (Te) Te[i] = ttm->Te_1d[i];
        if (xi) xi[i] = ttm->xi_1d[i];
        if (vcm) for (int d = 0; d < 3; d++) vcm[3 * i + d] = ttm->vcm_1d[i][d];
    }
    return n;
}

void oref_ttm_geom(fmd_t *md, int *tdims_local, int *itc_start, int *itc_glob_to_loc, double *tcellh)
{
    turi_t *t = md->active_ttm_turi;
    for (int d = 0; d < 3; d++)
    {
        tdims_local[d] = t->tdims_local[d];
        itc_start[d] = t->itc_start[d];
        itc_glob_to_loc[d] = t->itc_glob_to_loc[d];
        tcellh[d] = t->tcellh[d];
    }
}

/* The active TTM turi's derived parameters (src/ttm.h:41-100, set by the
   fmd_ttm_set* calls and _fmd_ttm_getReady, src/ttm.c:63-80): d[] = C_gamma,
   K, G, dz2, frontsurf, laser_t0, laser_tdiff, laser_m_2sig2_inv,
   laser_m_absdepth_inv, laser_factor_constant, Kzh.v2, Kzh.A, Kzh.B,
   tcell_volume, starttime, stoptime, tcellh[2]; k[] = type (1, 2),
   timestep_ratio, min_atoms_num, nC, nG, itc_start_owned[2], itc_stop[2],
   tdims_local[2], itc_glob_to_loc[2].  Returns -1 without a 1-D TTM. */
int oref_ttm_params(fmd_t *md, double *d, int *k)
{
    turi_t *t = md->active_ttm_turi;
    if (t == NULL || t->ttm == NULL || t->ttm->dim != 1) return -1;
    ttm_t *ttm = t->ttm;
    const double dv[17] = {ttm->C_gamma, ttm->K, ttm->G, ttm->dz2, ttm->frontsurf, ttm->laser_t0,
                           ttm->laser_tdiff, ttm->laser_m_2sig2_inv, ttm->laser_m_absdepth_inv,
                           ttm->laser_factor_constant, ttm->Kzh.v2, ttm->Kzh.A, ttm->Kzh.B, t->tcell_volume,
                           t->starttime, t->stoptime, t->tcellh[2]};
    const int kv[9] = {t->cat == FMD_TURI_TTM_TYPE1 ? 1 : 2, (int)ttm->timestep_ratio, (int)ttm->min_atoms_num,
                       ttm->nC, ttm->nG, t->itc_start_owned[2], t->itc_stop[2], (int)t->tdims_local[2],
                       t->itc_glob_to_loc[2]};
    memcpy(d, dv, sizeof dv);
    memcpy(k, kv, sizeof kv);
    return 0;
}

/* a type-2 TTM table (which: 0 T_C, 1 Ct, 2 C_DD, 3 T_G, 4 Gt, 5 G_DD) */
int oref_ttm_table(fmd_t *md, int which, double *out)
{
    turi_t *t = md->active_ttm_turi;
    if (t == NULL || t->ttm == NULL) return -1;
    ttm_t *ttm = t->ttm;
    const double *src[6] = {ttm->T_C, ttm->Ct, ttm->C_DD, ttm->T_G, ttm->Gt, ttm->G_DD};
    const int n = which < 3 ? ttm->nC : ttm->nG;
    if (which < 0 || which > 5 || src[which] == NULL) return -1;
    memcpy(out, src[which], sizeof(double) * n);
    return n;
}

/* EAM tables after load (src/eam.h:408-430): copies element `el`'s arrays */
int oref_eam_tables(fmd_pot_t *pot, int el, int *Nrho, int *Nr2, double *drho, double *dr2,
                    double *cutoff_sqr, double *F, double *F_DD, double *rho, double *rhoDD,
                    double *phi, double *phiDD)
{
    eam_t *eam = (eam_t *)pot->data;
    *Nrho = eam->Nrho; *Nr2 = eam->Nr2; *drho = eam->drho; *dr2 = eam->dr2;
    *cutoff_sqr = eam->cutoff_sqr;
    eam_element_t *e = eam->elements + el;
    if (F) memcpy(F, e->F, eam->Nrho * sizeof(double));
    if (F_DD) memcpy(F_DD, e->F_DD, eam->Nrho * sizeof(double));
    if (rho) memcpy(rho, e->rho, eam->Nr2 * sizeof(double));
    if (rhoDD) memcpy(rhoDD, e->rhoDD, eam->Nr2 * sizeof(double));
    if (phi) memcpy(phi, e->phi[el], eam->Nr2 * sizeof(double));
    if (phiDD) memcpy(phiDD, e->phiDD[el], eam->Nr2 * sizeof(double));
    return eam->ElementsNo;
}
