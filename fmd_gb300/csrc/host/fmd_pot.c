/*
 * Atom kinds, potential set-up and the device potential tables.
 *
 * Semantics follow the reference: kinds and masses (src/potential.c:32-54),
 * LJ / Morse parameter records (src/lj.c:92-113, src/morse.c:94-114),
 * pair table and potential categories (src/potential.c:135-249), largest
 * cutoff (src/potential.c:251-291), DYNAMO setfl loading with resampling of
 * f(r) and r*phi(r)/r onto a uniform r^2 grid (src/eam.c:324-555), and the
 * natural cubic spline preparation (src/cspline.c:24-74, the tridiagonal
 * sweep of the classic natural-spline algorithm).  The arithmetic is kept
 * in the same order so the tables are bit-identical to the reference's.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "fmd_private.h"

void fmd_matt_setAtomKinds(fmd_t *md, unsigned number, const fmd_string_t names[], const fmd_real_t masses[])
{
    if (number == 0 || number > FMD_MAX_KINDS)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "number of atomkinds %u (1..%d supported)",
                number, FMD_MAX_KINDS);
        return;
    }
    md->nkinds = number;
    for (unsigned i = 0; i < number; i++)
    {
        md->kinds[i].mass = masses[i] / FMD_MASS_UNIT;
        snprintf(md->kinds[i].name, sizeof md->kinds[i].name, "%s", names[i]);
        md->kinds[i].eam_elem = -1;
    }
    md->pottable_made = false;
    md->dev_tables_ok = false;
}

static fmd_pot_t *new_pot(fmd_t *md, potcat_t cat, void *data)
{
    fmd_pot_t *pot = (fmd_pot_t *)calloc(1, sizeof(fmd_pot_t));
    if (pot == NULL) { FMD_ERR(md, FMD_ERR_UNABLE_ALLOCATE_MEM, false, "potential"); return NULL; }
    pot->cat = cat;
    pot->data = data;
    pot->next = md->potlist;
    md->potlist = pot;
    return pot;
}

fmd_pot_t *fmd_pot_lj_apply(fmd_t *md, unsigned atomkind1, unsigned atomkind2,
                            fmd_real_t sigma, fmd_real_t epsilon, fmd_real_t cutoff)
{
    lj_t *lj = (lj_t *)malloc(sizeof(lj_t));
    if (lj == NULL) { FMD_ERR(md, FMD_ERR_UNABLE_ALLOCATE_MEM, false, "LJ"); return NULL; }
    lj->sig = sigma;
    lj->sig_sqr = sigma * sigma;
    lj->eps = epsilon;
    lj->eps4 = 4. * epsilon;
    lj->cutoff_sqr = cutoff * cutoff;
    fmd_pot_t *pot = new_pot(md, POTCAT_LJ, lj);
    if (pot) fmd_pot_apply(md, atomkind1, atomkind2, pot);
    return pot;
}

fmd_pot_t *fmd_pot_morse_apply(fmd_t *md, unsigned atomkind1, unsigned atomkind2,
                               fmd_real_t D0, fmd_real_t alpha, fmd_real_t r0, fmd_real_t cutoff)
{
    morse_t *m = (morse_t *)malloc(sizeof(morse_t));
    if (m == NULL) { FMD_ERR(md, FMD_ERR_UNABLE_ALLOCATE_MEM, false, "Morse"); return NULL; }
    m->D0 = D0;
    m->alpha = alpha;
    m->r0 = r0;
    m->cutoff_sqr = cutoff * cutoff;
    fmd_pot_t *pot = new_pot(md, POTCAT_MORSE, m);
    if (pot) fmd_pot_apply(md, atomkind1, atomkind2, pot);
    return pot;
}

/* ---- natural cubic splines ---- */

/* uniform grid x_i = i*h; natural end conditions (src/cspline.c:50-74) */
void _fmdh_spline_prepare(double h, const double *y, int n, double *yDD)
{
    double *u = (double *)malloc((size_t)(n > 1 ? n - 1 : 1) * sizeof(double));
    const double sig = 0.5;
    yDD[0] = u[0] = 0.0;
    for (int i = 1; i <= n - 2; i++)
    {
        const double p = sig * yDD[i - 1] + 2.0;
        yDD[i] = (sig - 1.0) / p;
        u[i] = (y[i + 1] - 2 * y[i] + y[i - 1]) / h;
        u[i] = (3.0 * u[i] / h - sig * u[i - 1]) / p;
    }
    yDD[n - 1] = 0.0;
    for (int k = n - 2; k >= 0; k--) yDD[k] = yDD[k] * yDD[k + 1] + u[k];
    free(u);
}

/* arbitrary increasing abscissae (src/cspline.c:24-48) */
void _fmdh_spline_prepare_adv(const double *x, const double *y, int n, double *yDD)
{
    double *u = (double *)malloc((size_t)(n > 1 ? n - 1 : 1) * sizeof(double));
    yDD[0] = u[0] = 0.0;
    for (int i = 1; i <= n - 2; i++)
    {
        const double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
        const double p = sig * yDD[i - 1] + 2.0;
        yDD[i] = (sig - 1.0) / p;
        u[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]);
        u[i] = (6.0 * u[i] / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p;
    }
    yDD[n - 1] = 0.0;
    for (int k = n - 2; k >= 0; k--) yDD[k] = yDD[k] * yDD[k + 1] + u[k];
    free(u);
}

static double spline_val_uniform(double h, const double *y, const double *ydd, int n, double x)
{
    int lo = (int)(x / h);
    /* the last sample of a resampled table lands on the final knot */
    if (lo > n - 2) lo = n - 2;
    const int hi = lo + 1;
    const double a = hi - x / h;
    const double b = 1 - a;
    return a * y[lo] + b * y[hi] + ((a * a * a - a) * ydd[lo] + (b * b * b - b) * ydd[hi]) * (h * h) / 6.0;
}

/* f2(r^2) = f1(r): resample a table on r_i = i*dr onto s_j = j*dr2
   (src/eam.c:324-341) */
static void convert_r_to_r2(const eam_t *eam, const double *src, double *dst)
{
    double *dd = (double *)malloc(eam->Nr * sizeof(double));
    _fmdh_spline_prepare(eam->dr, src, eam->Nr, dd);
    for (int i = 0; i < eam->Nr2; i++)
        dst[i] = spline_val_uniform(eam->dr, src, dd, eam->Nr, sqrt(i * eam->dr2));
    free(dd);
}

static void eam_free(eam_t *eam)
{
    if (eam == NULL) return;
    for (int i = 0; i < eam->nelem; i++)
    {
        free(eam->el[i].F); free(eam->el[i].F_DD);
        free(eam->el[i].rho); free(eam->el[i].rhoDD);
        for (int j = 0; j <= i; j++)
        {
            free(eam->phi[i * eam->nelem + j]);
            free(eam->phiDD[i * eam->nelem + j]);
        }
    }
    free(eam->el);
    free(eam->phi);
    free(eam->phiDD);
    free(eam);
}

static bool read_doubles(FILE *fp, double *out, int n)
{
    for (int i = 0; i < n; i++)
        if (fscanf(fp, "%lf", &out[i]) != 1) return false;
    return true;
}

/* DYNAMO multi-element setfl reader (src/eam.c:376-480) */
static eam_t *load_setfl(fmd_t *md, const char *path)
{
    const char *ftype = "DYNAMO multi-element setfl (eam/alloy)";
    FILE *fp = fopen(path, "r");
    if (fp == NULL) { FMD_ERR(md, FMD_ERR_UNABLE_OPEN_FILE, false, "%s", path); return NULL; }
    eam_t *eam = (eam_t *)calloc(1, sizeof(eam_t));
    char str[1024];
    double *tmp = NULL;
    for (int i = 0; i < 3; i++)
        if (fgets(str, sizeof str, fp) == NULL) goto corrupted;
    if (fscanf(fp, "%d", &eam->nelem) != 1 || eam->nelem < 1 || eam->nelem > 16) goto corrupted;
    eam->el = (eam_element_t *)calloc(eam->nelem, sizeof(eam_element_t));
    eam->phi = (double **)calloc((size_t)eam->nelem * eam->nelem, sizeof(double *));
    eam->phiDD = (double **)calloc((size_t)eam->nelem * eam->nelem, sizeof(double *));
    for (int i = 0; i < eam->nelem; i++)
    {
        if (fscanf(fp, "%63s", eam->el[i].name) != 1) goto corrupted;
    }
    double cutoff;
    if (fscanf(fp, "%d%lf%d%lf%lf", &eam->Nrho, &eam->drho, &eam->Nr, &eam->dr, &cutoff) != 5) goto corrupted;
    if (eam->Nrho < 3 || eam->Nr < 2) goto corrupted;
    eam->Nr2 = (eam->Nr += 2);
    if ((eam->Nr - 1) * eam->dr <= cutoff) goto corrupted;
    eam->cutoff_sqr = cutoff * cutoff;
    eam->dr2 = ((eam->Nr - 1) * eam->dr) * ((eam->Nr - 1) * eam->dr) / (eam->Nr2 - 1);
    tmp = (double *)malloc(eam->Nr * sizeof(double));
    for (int i = 0; i < eam->nelem; i++)
    {
        eam_element_t *e = &eam->el[i];
        char z[64], lat[64];
        if (fscanf(fp, "%63s%lf%lf%63s", z, &e->mass, &e->lattice, lat) != 4) goto corrupted;
        e->mass /= FMD_MASS_UNIT;
        e->F = (double *)malloc(eam->Nrho * sizeof(double));
        e->F_DD = (double *)malloc(eam->Nrho * sizeof(double));
        if (!read_doubles(fp, e->F, eam->Nrho)) goto corrupted;
        if (!read_doubles(fp, tmp, eam->Nr - 2)) goto corrupted;
        tmp[eam->Nr - 1] = tmp[eam->Nr - 2] = 0.;
        e->rho = (double *)malloc(eam->Nr2 * sizeof(double));
        e->rhoDD = (double *)malloc(eam->Nr2 * sizeof(double));
        convert_r_to_r2(eam, tmp, e->rho);
        _fmdh_spline_prepare(eam->drho, e->F, eam->Nrho, e->F_DD);
        _fmdh_spline_prepare(eam->dr2, e->rho, eam->Nr2, e->rhoDD);
    }
    for (int i = 0; i < eam->nelem; i++)
        for (int j = 0; j <= i; j++)
        {
            for (int k = 0; k < eam->Nr - 2; k++)
            {
                if (fscanf(fp, "%lf", &tmp[k]) != 1) goto corrupted;
                if (k == 0) tmp[k] = FLT_MAX;
                else tmp[k] /= k * eam->dr;
            }
            tmp[eam->Nr - 1] = tmp[eam->Nr - 2] = 0.;
            double *ph = (double *)malloc(eam->Nr2 * sizeof(double));
            double *phdd = (double *)malloc(eam->Nr2 * sizeof(double));
            convert_r_to_r2(eam, tmp, ph);
            _fmdh_spline_prepare(eam->dr2, ph, eam->Nr2, phdd);
            eam->phi[i * eam->nelem + j] = eam->phi[j * eam->nelem + i] = ph;
            eam->phiDD[i * eam->nelem + j] = eam->phiDD[j * eam->nelem + i] = phdd;
        }
    free(tmp);
    fclose(fp);
    return eam;
corrupted:
    FMD_ERR(md, FMD_ERR_FILE_CORRUPTED, true, "%s file %s", ftype, path);
    free(tmp);
    fclose(fp);
    /* release what was read: elements whose arrays exist */
    if (eam->el)
        for (int i = 0; i < eam->nelem; i++)
        {
            free(eam->el[i].F); free(eam->el[i].F_DD); free(eam->el[i].rho); free(eam->el[i].rhoDD);
        }
    if (eam->phi)
        for (int i = 0; i < eam->nelem; i++)
            for (int j = 0; j <= i; j++)
            {
                free(eam->phi[i * eam->nelem + j]);
                free(eam->phiDD[i * eam->nelem + j]);
            }
    free(eam->el); free(eam->phi); free(eam->phiDD); free(eam);
    return NULL;
}

fmd_pot_t *fmd_pot_eam_alloy_load(fmd_t *md, fmd_string_t path)
{
    eam_t *eam = load_setfl(md, path);
    if (eam == NULL) return NULL;
    return new_pot(md, POTCAT_EAM, eam);
}

fmd_real_t fmd_pot_eam_getLatticeParameter(fmd_t *md, fmd_pot_t *pot, fmd_string_t element)
{
    if (pot == NULL || pot->cat != POTCAT_EAM)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "potential category %d", pot ? (int)pot->cat : -1);
        return 0.;
    }
    eam_t *eam = (eam_t *)pot->data;
    for (int i = 0; i < eam->nelem; i++)
        if (strcmp(element, eam->el[i].name) == 0) return eam->el[i].lattice;
    FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "element %s is not in the EAM potential", element);
    return 0.;
}

fmd_real_t fmd_pot_eam_getCutoffRadius(fmd_t *md, fmd_pot_t *pot)
{
    if (pot == NULL || pot->cat != POTCAT_EAM)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "potential category %d", pot ? (int)pot->cat : -1);
        return 0.;
    }
    return sqrt(((eam_t *)pot->data)->cutoff_sqr);
}

static int eam_find(const eam_t *eam, const char *name)
{
    for (int i = 0; i < eam->nelem; i++)
        if (strcmp(name, eam->el[i].name) == 0) return i;
    return -1;
}

void fmd_pot_apply(fmd_t *md, unsigned atomkind1, unsigned atomkind2, fmd_pot_t *pot)
{
    if (pot == NULL) return;
    if (atomkind1 >= md->nkinds || atomkind2 >= md->nkinds)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "atom kind %u/%u", atomkind1, atomkind2);
        return;
    }
    if (!md->pottable_made)
    {
        memset(md->pottable, 0, sizeof md->pottable);
        md->pottable_made = true;
    }
    int loc1 = -1, loc2 = -1;
    if (pot->cat == POTCAT_EAM)
    {
        eam_t *eam = (eam_t *)pot->data;
        loc1 = eam_find(eam, md->kinds[atomkind1].name);
        loc2 = eam_find(eam, md->kinds[atomkind2].name);
        if (loc1 < 0 || loc2 < 0)
        {
            FMD_ERR(md, FMD_ERR_WRONG_POTENTIAL, false, "EAM for atom kinds %u and %u", atomkind1, atomkind2);
            return;
        }
        if (md->applied_eam != NULL && md->applied_eam != eam)
        {
            FMD_ERR(md, FMD_ERR_NOT_SUPPORTED_YET, false, "one EAM potential per instance");
            return;
        }
        md->applied_eam = eam;
        md->kinds[atomkind1].eam_elem = loc1;
        md->kinds[atomkind2].eam_elem = loc2;
    }
    potpair_t *a = &md->pottable[atomkind1][atomkind2], *b = &md->pottable[atomkind2][atomkind1];
    a->cat = b->cat = pot->cat;
    a->pot = b->pot = pot;
    a->iloc = loc1; a->jloc = loc2;
    b->iloc = loc2; b->jloc = loc1;
    md->dev_tables_ok = false;
}

static double pair_cutoff_sqr(const potpair_t *p)
{
    switch (p->cat)
    {
        case POTCAT_LJ: return ((lj_t *)p->pot->data)->cutoff_sqr;
        case POTCAT_MORSE: return ((morse_t *)p->pot->data)->cutoff_sqr;
        case POTCAT_EAM: return ((eam_t *)p->pot->data)->cutoff_sqr;
        default: return -1.0;
    }
}

double _fmdh_largest_cutoff(fmd_t *md)
{
    if (!md->pottable_made)
    {
        FMD_ERR(md, FMD_ERR_UNPREPARED, false, "potential table");
        return 0.;
    }
    double max = 0.0;
    for (unsigned i = 0; i < md->nkinds; i++)
        for (unsigned j = 0; j <= i; j++)
        {
            const double r = pair_cutoff_sqr(&md->pottable[i][j]);
            if (r < 0)
            {
                FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "pair potential category %d",
                        (int)md->pottable[i][j].cat);
                return 0.;
            }
            if (r > max) max = r;
        }
    return sqrt(max);
}

bool _fmdh_pots_ready(fmd_t *md)
{
    if (!md->pottable_made)
    {
        FMD_ERR(md, FMD_ERR_UNPREPARED, false, "potential table");
        return false;
    }
    for (unsigned i = 0; i < md->nkinds; i++)
        for (unsigned j = 0; j <= i; j++)
            if (md->pottable[i][j].cat == POTCAT_NONE)
            {
                FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "pair potential category %d", 0);
                return false;
            }
    return true;
}

/* Pair table, masses and EAM tables to the device (replaces the per-pair
   pointer chasing of the reference's pottable). */
/* EAM tables of all elements as contiguous arrays in the device engine's
   layout: F, F_DD [nelem*Nrho]; rho, rhoDD [nelem*Nr2]; phi, phiDD
   [nelem*nelem*Nr2] */
void _fmdh_eam_flatten(const eam_t *e, double *F, double *FDD, double *rho, double *rhoDD, double *phi,
                       double *phiDD)
{
    const int ne = e->nelem;
    for (int i = 0; i < ne; i++)
    {
        memcpy(F + (size_t)i * e->Nrho, e->el[i].F, sizeof(double) * e->Nrho);
        memcpy(FDD + (size_t)i * e->Nrho, e->el[i].F_DD, sizeof(double) * e->Nrho);
        memcpy(rho + (size_t)i * e->Nr2, e->el[i].rho, sizeof(double) * e->Nr2);
        memcpy(rhoDD + (size_t)i * e->Nr2, e->el[i].rhoDD, sizeof(double) * e->Nr2);
        for (int j = 0; j < ne; j++)
        {
            memcpy(phi + ((size_t)i * ne + j) * e->Nr2, e->phi[i * ne + j], sizeof(double) * e->Nr2);
            memcpy(phiDD + ((size_t)i * ne + j) * e->Nr2, e->phiDD[i * ne + j], sizeof(double) * e->Nr2);
        }
    }
}

int _fmdh_upload_tables(fmd_t *md)
{
    if (md->dev_tables_ok) return FMDG_OK;
    const int nk = (int)md->nkinds;
    double mass[FMD_MAX_KINDS] = {0};
    int elem[FMD_MAX_KINDS] = {0};
    for (int k = 0; k < nk; k++)
    {
        mass[k] = md->kinds[k].mass;
        elem[k] = md->kinds[k].eam_elem;
    }
    int rc = fmdg_set_kinds(md->dev, nk, mass, elem);
    if (rc) return rc;
    fmdg_pair_t table[FMD_MAX_KINDS * FMD_MAX_KINDS];
    memset(table, 0, sizeof table);
    for (int i = 0; i < nk; i++)
        for (int j = 0; j < nk; j++)
        {
            const potpair_t *p = &md->pottable[i][j];
            fmdg_pair_t *t = &table[i * nk + j];
            t->cat = (int)p->cat;
            if (p->cat == POTCAT_LJ)
            {
                const lj_t *lj = (const lj_t *)p->pot->data;
                t->p[0] = lj->eps4; t->p[1] = lj->sig_sqr; t->p[2] = lj->cutoff_sqr;
            }
            else if (p->cat == POTCAT_MORSE)
            {
                const morse_t *m = (const morse_t *)p->pot->data;
                t->p[0] = m->D0; t->p[1] = m->alpha; t->p[2] = m->r0; t->p[3] = m->cutoff_sqr;
            }
            else if (p->cat == POTCAT_EAM)
            {
                t->p[2] = ((const eam_t *)p->pot->data)->cutoff_sqr;
                t->iloc = p->iloc;
                t->jloc = p->jloc;
            }
        }
    if ((rc = fmdg_set_pairs(md->dev, table))) return rc;
    if (md->applied_eam != NULL)
    {
        const eam_t *e = md->applied_eam;
        const int ne = e->nelem;
        double *F = (double *)malloc(sizeof(double) * ne * e->Nrho);
        double *FDD = (double *)malloc(sizeof(double) * ne * e->Nrho);
        double *rho = (double *)malloc(sizeof(double) * ne * e->Nr2);
        double *rhoDD = (double *)malloc(sizeof(double) * ne * e->Nr2);
        double *phi = (double *)malloc(sizeof(double) * ne * ne * e->Nr2);
        double *phiDD = (double *)malloc(sizeof(double) * ne * ne * e->Nr2);
        _fmdh_eam_flatten(e, F, FDD, rho, rhoDD, phi, phiDD);
        rc = fmdg_set_eam(md->dev, ne, e->Nrho, e->drho, e->Nr2, e->dr2, F, FDD, rho, rhoDD, phi, phiDD);
        free(F); free(FDD); free(rho); free(rhoDD); free(phi); free(phiDD);
        if (rc) return rc;
    }
    if ((rc = fmdg_set_precision(md->dev, md->precision))) return rc;
    md->dev_tables_ok = true;
    return FMDG_OK;
}

void _fmdh_pots_free(fmd_t *md)
{
    fmd_pot_t *p = md->potlist;
    while (p != NULL)
    {
        fmd_pot_t *next = p->next;
        if (p->cat == POTCAT_EAM) eam_free((eam_t *)p->data);
        else free(p->data);
        free(p);
        p = next;
    }
    md->potlist = NULL;
    md->applied_eam = NULL;
}
