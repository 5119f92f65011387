/*
 * CPU restatement of FMD 0.4.0's per-timestep hot path -- TEST
 * INFRASTRUCTURE ONLY (see fmd_oracle.h).  Parity pinned against golden
 * vectors produced by the reference compiled from its own sources.
 *
 * Correspondence with the reference (paths inside the reference project):
 *   cell lists, append / swap-remove ..... src/cell.h:84-95, src/cell.c:151-160
 *   refresh (re-binning) ................. src/misc.c:268-308
 *   periodic migration / open-face loss .. src/md-ghost.c:827-869, :109-143, :41-61
 *   ghost images ......................... src/md-ghost.c:85-107, :750-786
 *   half-shell neighbour cells ........... src/subdomain.c:76-199 (cnb1: codes 14..26)
 *   LJ pair update ....................... src/lj.h:26-58, loop src/lj.c:28-90
 *   Morse pair update .................... src/morse.h:26-58, loop src/morse.c:30-92
 *   EAM density / embedding / force ...... src/eam.h:176-406, src/eam.c:29-322
 *   hybrid category switch ............... src/forces.c:33-290
 *   velocity Verlet + Berendsen .......... src/integrators.c:40-126
 *   group thermodynamics ................. src/matter.c:31-68
 *   natural cubic spline ................. src/cspline.h:26-27, src/cspline.c:50-74
 *   setfl loading, r -> r^2 resampling ... src/eam.c:324-480
 *   turi fields (number, mass, vcm, T) .. src/turi.c:959-1335
 *   TTM activation, types 1 and 2, xi .... src/ttm.c:154-383, src/turi.c:1337-1373
 *   TTM friction term .................... src/forces.c:292-330, :376-378
 *   symplectic Euler ..................... src/integrators.c:129-225
 * Ghost cells are not materialised: a neighbour cell across a periodic face
 * is the interior cell on the far side with its positions shifted by +/- l,
 * and the partial force of that image is added to its owner directly (the
 * reference adds it after the loop, src/md-ghost.c:788-825; the sum is the
 * same up to binary64 reordering).  OpenMP runs use per-thread accumulation
 * buffers, so results do not depend on scheduling.
 */
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "fmd_oracle.h"

#define K_B 8.6173303e-5
#define MASS_UNIT 9.6485332907e+03
#define MAXK 8

typedef struct
{
    int n, cap;
    double *x, *v, *F, *va;
    int *group;
    unsigned *kind, *id;
} ocell_t;

/* a 1-D TTM turi (one cell across x and y) */
typedef struct
{
    int on;
    oracle_ttm_params_t p;
    double *tabs;              /* owned copies of the type-2 tables */
    int nz, g2l, lo, hi;       /* local cells incl. margins; itc = (int)(z/h) + g2l; interior [lo, hi) */
    double tcellh, vol, start, stop;
    unsigned *num;
    double *mass, *vcm, *Ti, *Te, *Te2, *xi, *Ke, *Ce, *Gc;
} ottm_t;

struct oracle_sys
{
    double l[3], cellh[3];
    int pbc[3], nc[3];
    int ncell;                 /* interior cells */
    int ng[3], ngrid;          /* local grid incl. one ghost layer: nc+2 */
    ocell_t *grid;             /* ngrid cells, local coords (z fastest) */
    int nkinds;
    double mass[MAXK];
    int eam_elem[MAXK];
    oracle_pair_t pairs[MAXK * MAXK];
    int cats;
    /* EAM tables on the r^2 grid */
    int nelem, Nrho, Nr, Nr2;
    double drho, dr, dr2, eam_rc2;
    double *F, *FDD, *rho, *rhoDD, *phi, *phiDD;
    double elem_mass[16], elem_lat[16];
    oracle_thermo_t th;
    double lambda;
    unsigned err;
    int nthreads;
    /* flat indexing for accumulation buffers */
    int *start;
    double time, dt;           /* simulation time and step of the TTM runs */
    ottm_t ttm;
};

/* ------------------------------------------------------------ cells */

static int gidx(const oracle_sys_t *o, int x, int y, int z) { return z + o->ng[2] * (y + o->ng[1] * x); }
static int is_interior(const oracle_sys_t *o, const int c[3])
{
    for (int d = 0; d < 3; d++)
        if (c[d] < 1 || c[d] > o->nc[d]) return 0;
    return 1;
}

static void cell_reserve(ocell_t *c, int n)
{
    if (n <= c->cap) return;
    int cap = c->cap ? c->cap : 4;
    while (cap < n) cap *= 2;
    c->x = (double *)realloc(c->x, sizeof(double) * 3 * cap);
    c->v = (double *)realloc(c->v, sizeof(double) * 3 * cap);
    c->F = (double *)realloc(c->F, sizeof(double) * 3 * cap);
    c->va = (double *)realloc(c->va, sizeof(double) * cap);
    c->group = (int *)realloc(c->group, sizeof(int) * cap);
    c->kind = (unsigned *)realloc(c->kind, sizeof(unsigned) * cap);
    c->id = (unsigned *)realloc(c->id, sizeof(unsigned) * cap);
    c->cap = cap;
}

static void cell_copy(ocell_t *from, int i, ocell_t *to, int j)
{
    memcpy(to->x + 3 * j, from->x + 3 * i, 3 * sizeof(double));
    memcpy(to->v + 3 * j, from->v + 3 * i, 3 * sizeof(double));
    memcpy(to->F + 3 * j, from->F + 3 * i, 3 * sizeof(double));
    to->va[j] = from->va[i];
    to->group[j] = from->group[i];
    to->kind[j] = from->kind[i];
    to->id[j] = from->id[i];
}

static int cell_append(ocell_t *c)
{
    cell_reserve(c, c->n + 1);
    return c->n++;
}

/* swap-with-last removal (src/cell.c:151-160) */
static void cell_remove(ocell_t *c, int i)
{
    c->n--;
    if (c->n != i) cell_copy(c, c->n, c, i);
}

static void free_grid(oracle_sys_t *o)
{
    if (!o->grid) return;
    for (int c = 0; c < o->ngrid; c++)
    {
        ocell_t *g = &o->grid[c];
        free(g->x); free(g->v); free(g->F); free(g->va); free(g->group); free(g->kind); free(g->id);
    }
    free(o->grid);
    o->grid = NULL;
    free(o->start);
    o->start = NULL;
}

/* interior cell c (storage order) -> local grid cell */
static ocell_t *icell(oracle_sys_t *o, int c)
{
    const int x = c / (o->nc[1] * o->nc[2]), y = (c / o->nc[2]) % o->nc[1], z = c % o->nc[2];
    return &o->grid[gidx(o, x + 1, y + 1, z + 1)];
}

/* ---------------------------------------------------------- lifetime */

oracle_sys_t *oracle_create(void)
{
    oracle_sys_t *o = (oracle_sys_t *)calloc(1, sizeof(oracle_sys_t));
    o->nthreads = 1;
    o->lambda = 1.0;
    return o;
}

static void free_ttm(ottm_t *t)
{
    free(t->tabs); free(t->num); free(t->mass); free(t->vcm); free(t->Ti); free(t->Te); free(t->Te2);
    free(t->xi); free(t->Ke); free(t->Ce); free(t->Gc);
    memset(t, 0, sizeof *t);
}

void oracle_destroy(oracle_sys_t *o)
{
    if (!o) return;
    free_grid(o);
    free_ttm(&o->ttm);
    free(o->F); free(o->FDD); free(o->rho); free(o->rhoDD); free(o->phi); free(o->phiDD);
    free(o);
}

int oracle_set_threads(oracle_sys_t *o, int nthreads)
{
    o->nthreads = nthreads > 0 ? nthreads : 1;
    return 0;
}

int oracle_set_box(oracle_sys_t *o, const double l[3], const int pbc[3], const int nc[3], const double cellh[3])
{
    free_grid(o);
    for (int d = 0; d < 3; d++)
    {
        o->l[d] = l[d];
        o->pbc[d] = pbc[d] != 0;
        o->nc[d] = nc[d];
        o->cellh[d] = cellh[d];
        o->ng[d] = nc[d] + 2;
    }
    o->ncell = nc[0] * nc[1] * nc[2];
    o->ngrid = o->ng[0] * o->ng[1] * o->ng[2];
    o->grid = (ocell_t *)calloc(o->ngrid, sizeof(ocell_t));
    o->start = (int *)calloc(o->ncell + 1, sizeof(int));
    return 0;
}

int oracle_set_kinds(oracle_sys_t *o, int nkinds, const double *mass, const int *eam_elem)
{
    if (nkinds < 1 || nkinds > MAXK) return -1;
    o->nkinds = nkinds;
    for (int k = 0; k < nkinds; k++)
    {
        o->mass[k] = mass[k];
        o->eam_elem[k] = eam_elem ? eam_elem[k] : -1;
    }
    return 0;
}

int oracle_set_pairs(oracle_sys_t *o, const oracle_pair_t *table)
{
    o->cats = 0;
    for (int k = 0; k < o->nkinds * o->nkinds; k++)
    {
        o->pairs[k] = table[k];
        o->cats |= 1 << table[k].cat;
    }
    return 0;
}

int oracle_set_eam(oracle_sys_t *o, int nelem, int Nrho, double drho, int Nr2, double dr2,
                   const double *F, const double *F_DD, const double *rho, const double *rhoDD,
                   const double *phi, const double *phiDD)
{
    free(o->F); free(o->FDD); free(o->rho); free(o->rhoDD); free(o->phi); free(o->phiDD);
    o->nelem = nelem; o->Nrho = Nrho; o->drho = drho; o->Nr2 = Nr2; o->dr2 = dr2;
    const size_t nF = (size_t)nelem * Nrho, nR = (size_t)nelem * Nr2, nP = (size_t)nelem * nelem * Nr2;
    o->F = (double *)malloc(nF * 8); memcpy(o->F, F, nF * 8);
    o->FDD = (double *)malloc(nF * 8); memcpy(o->FDD, F_DD, nF * 8);
    o->rho = (double *)malloc(nR * 8); memcpy(o->rho, rho, nR * 8);
    o->rhoDD = (double *)malloc(nR * 8); memcpy(o->rhoDD, rhoDD, nR * 8);
    o->phi = (double *)malloc(nP * 8); memcpy(o->phi, phi, nP * 8);
    o->phiDD = (double *)malloc(nP * 8); memcpy(o->phiDD, phiDD, nP * 8);
    return 0;
}

/* ---------------------------------------------------- splines, setfl */

/* uniform natural spline second derivatives (src/cspline.c:50-74) */
static void spline_prepare(double h, const double *y, int n, double *ydd)
{
    double *u = (double *)malloc(sizeof(double) * (n > 1 ? n : 2));
    const double sig = 0.5;
    ydd[0] = u[0] = 0.0;
    for (int i = 1; i <= n - 2; i++)
    {
        const double p = sig * ydd[i - 1] + 2.0;
        ydd[i] = (sig - 1.0) / p;
        u[i] = (y[i + 1] - 2 * y[i] + y[i - 1]) / h;
        u[i] = (3.0 * u[i] / h - sig * u[i - 1]) / p;
    }
    ydd[n - 1] = 0.0;
    for (int k = n - 2; k >= 0; k--) ydd[k] = ydd[k] * ydd[k + 1] + u[k];
    free(u);
}

#define SVAL(a, b, y, lo, hi, ydd, h) \
    ((a) * (y)[lo] + (b) * (y)[hi] + (((a) * (a) * (a) - (a)) * (ydd)[lo] + ((b) * (b) * (b) - (b)) * (ydd)[hi]) * ((h) * (h)) / 6.0)
#define SDER(a, b, y, lo, hi, ydd, h) \
    (((y)[hi] - (y)[lo]) / (h) + ((3 * (b) * (b) - 1) * (ydd)[hi] - (3 * (a) * (a) - 1) * (ydd)[lo]) * (h) / 6.0)

static double spline_at(double h, const double *y, const double *ydd, int n, double x)
{
    int lo = (int)(x / h);
    if (lo > n - 2) lo = n - 2;
    const int hi = lo + 1;
    const double a = hi - x / h, b = 1 - a;
    return SVAL(a, b, y, lo, hi, ydd, h);
}

static void r_to_r2(const oracle_sys_t *o, const double *src, double *dst)
{
    double *dd = (double *)malloc(sizeof(double) * o->Nr);
    spline_prepare(o->dr, src, o->Nr, dd);
    for (int i = 0; i < o->Nr2; i++) dst[i] = spline_at(o->dr, src, dd, o->Nr, sqrt(i * o->dr2));
    free(dd);
}

int oracle_load_setfl(oracle_sys_t *o, const char *path, char *names, int names_len, double *cutoff)
{
    FILE *fp = fopen(path, "r");
    if (!fp) return -1;
    char line[1024];
    for (int i = 0; i < 3; i++)
        if (!fgets(line, sizeof line, fp)) { fclose(fp); return -2; }
    int ne;
    if (fscanf(fp, "%d", &ne) != 1 || ne < 1 || ne > 16) { fclose(fp); return -2; }
    if (names && names_len > 0) names[0] = 0;
    for (int i = 0; i < ne; i++)
    {
        char nm[64];
        if (fscanf(fp, "%63s", nm) != 1) { fclose(fp); return -2; }
        if (names && (int)(strlen(names) + strlen(nm) + 2) < names_len)
        {
            if (i) strcat(names, " ");
            strcat(names, nm);
        }
    }
    double rc;
    if (fscanf(fp, "%d%lf%d%lf%lf", &o->Nrho, &o->drho, &o->Nr, &o->dr, &rc) != 5) { fclose(fp); return -2; }
    o->Nr2 = (o->Nr += 2);
    if ((o->Nr - 1) * o->dr <= rc) { fclose(fp); return -2; }
    o->eam_rc2 = rc * rc;
    if (cutoff) *cutoff = rc;
    o->dr2 = ((o->Nr - 1) * o->dr) * ((o->Nr - 1) * o->dr) / (o->Nr2 - 1);
    o->nelem = ne;
    free(o->F); free(o->FDD); free(o->rho); free(o->rhoDD); free(o->phi); free(o->phiDD);
    o->F = (double *)malloc(sizeof(double) * ne * o->Nrho);
    o->FDD = (double *)malloc(sizeof(double) * ne * o->Nrho);
    o->rho = (double *)malloc(sizeof(double) * ne * o->Nr2);
    o->rhoDD = (double *)malloc(sizeof(double) * ne * o->Nr2);
    o->phi = (double *)malloc(sizeof(double) * ne * ne * o->Nr2);
    o->phiDD = (double *)malloc(sizeof(double) * ne * ne * o->Nr2);
    double *tmp = (double *)malloc(sizeof(double) * o->Nr);
    for (int e = 0; e < ne; e++)
    {
        char z[64], lat[64];
        if (fscanf(fp, "%63s%lf%lf%63s", z, &o->elem_mass[e], &o->elem_lat[e], lat) != 4) goto bad;
        for (int j = 0; j < o->Nrho; j++)
            if (fscanf(fp, "%lf", &o->F[(size_t)e * o->Nrho + j]) != 1) goto bad;
        for (int j = 0; j < o->Nr - 2; j++)
            if (fscanf(fp, "%lf", &tmp[j]) != 1) goto bad;
        tmp[o->Nr - 1] = tmp[o->Nr - 2] = 0.;
        r_to_r2(o, tmp, o->rho + (size_t)e * o->Nr2);
        spline_prepare(o->drho, o->F + (size_t)e * o->Nrho, o->Nrho, o->FDD + (size_t)e * o->Nrho);
        spline_prepare(o->dr2, o->rho + (size_t)e * o->Nr2, o->Nr2, o->rhoDD + (size_t)e * o->Nr2);
    }
    for (int i = 0; i < ne; i++)
        for (int j = 0; j <= i; j++)
        {
            for (int k = 0; k < o->Nr - 2; k++)
            {
                if (fscanf(fp, "%lf", &tmp[k]) != 1) goto bad;
                if (k == 0) tmp[k] = FLT_MAX;
                else tmp[k] /= k * o->dr;
            }
            tmp[o->Nr - 1] = tmp[o->Nr - 2] = 0.;
            double *p = o->phi + ((size_t)i * ne + j) * o->Nr2;
            r_to_r2(o, tmp, p);
            spline_prepare(o->dr2, p, o->Nr2, o->phiDD + ((size_t)i * ne + j) * o->Nr2);
            if (i != j)
            {
                memcpy(o->phi + ((size_t)j * ne + i) * o->Nr2, p, sizeof(double) * o->Nr2);
                memcpy(o->phiDD + ((size_t)j * ne + i) * o->Nr2, o->phiDD + ((size_t)i * ne + j) * o->Nr2,
                       sizeof(double) * o->Nr2);
            }
        }
    free(tmp);
    fclose(fp);
    return ne;
bad:
    free(tmp);
    fclose(fp);
    return -2;
}

int oracle_eam_table(oracle_sys_t *o, int el, int which, double *out, int *n)
{
    const double *src;
    int len;
    switch (which)
    {
        case 0: src = o->F + (size_t)el * o->Nrho; len = o->Nrho; break;
        case 1: src = o->FDD + (size_t)el * o->Nrho; len = o->Nrho; break;
        case 2: src = o->rho + (size_t)el * o->Nr2; len = o->Nr2; break;
        case 3: src = o->rhoDD + (size_t)el * o->Nr2; len = o->Nr2; break;
        case 4: src = o->phi + ((size_t)el * o->nelem + el) * o->Nr2; len = o->Nr2; break;
        default: src = o->phiDD + ((size_t)el * o->nelem + el) * o->Nr2; len = o->Nr2; break;
    }
    if (out) memcpy(out, src, sizeof(double) * len);
    if (n) *n = len;
    return 0;
}

/* ------------------------------------------------------------- atoms */

int oracle_upload(oracle_sys_t *o, int n, const int *cell_count, const double *x, const double *v,
                  const unsigned *kind, const int *group, const unsigned *atomid)
{
    for (int c = 0; c < o->ngrid; c++) o->grid[c].n = 0;
    int k = 0;
    for (int c = 0; c < o->ncell; c++)
    {
        ocell_t *cl = icell(o, c);
        for (int i = 0; i < cell_count[c]; i++, k++)
        {
            const int j = cell_append(cl);
            memcpy(cl->x + 3 * j, x + 3 * k, 3 * sizeof(double));
            memcpy(cl->v + 3 * j, v + 3 * k, 3 * sizeof(double));
            memset(cl->F + 3 * j, 0, 3 * sizeof(double));
            cl->va[j] = 0.0;
            cl->kind[j] = kind[k];
            cl->group[j] = group[k];
            cl->id[j] = atomid[k];
        }
    }
    return k == n ? 0 : -1;
}

int oracle_natoms(oracle_sys_t *o)
{
    int n = 0;
    for (int c = 0; c < o->ncell; c++) n += icell(o, c)->n;
    return n;
}

int oracle_download(oracle_sys_t *o, int *cell_of, double *x, double *v, double *F, double *vaream,
                    unsigned *kind, int *group, unsigned *atomid)
{
    int k = 0;
    for (int c = 0; c < o->ncell; c++)
    {
        ocell_t *cl = icell(o, c);
        for (int i = 0; i < cl->n; i++, k++)
        {
            if (cell_of) cell_of[k] = c;
            if (x) memcpy(x + 3 * k, cl->x + 3 * i, 3 * sizeof(double));
            if (v) memcpy(v + 3 * k, cl->v + 3 * i, 3 * sizeof(double));
            if (F) memcpy(F + 3 * k, cl->F + 3 * i, 3 * sizeof(double));
            if (vaream) vaream[k] = cl->va[i];
            if (kind) kind[k] = cl->kind[i];
            if (group) group[k] = cl->group[i];
            if (atomid) atomid[k] = cl->id[i];
        }
    }
    return k;
}

int oracle_set_state(oracle_sys_t *o, const double *x, const double *v)
{
    int k = 0;
    for (int c = 0; c < o->ncell; c++)
    {
        ocell_t *cl = icell(o, c);
        for (int i = 0; i < cl->n; i++, k++)
        {
            if (x) memcpy(cl->x + 3 * i, x + 3 * k, 3 * sizeof(double));
            if (v) memcpy(cl->v + 3 * i, v + 3 * k, 3 * sizeof(double));
        }
    }
    return 0;
}

unsigned oracle_errors(oracle_sys_t *o) { return o->err; }

/* ----------------------------------------------------------- refresh */

/* migration of the ghost layer along d (src/md-ghost.c:827-869 with the
   index ranges of set_cell_indexes_for_migration_in_direction_d) */
static void migrate(oracle_sys_t *o)
{
    for (int d = 0; d < 3; d++)
    {
        int lo[3], hi[3];
        for (int side = 0; side < 2; side++)
        {
            for (int dd = 0; dd < 3; dd++)
            {
                if (dd == d) { lo[dd] = side == 0 ? 0 : o->nc[dd] + 1; hi[dd] = lo[dd] + 1; }
                else if (dd > d) { lo[dd] = 0; hi[dd] = o->ng[dd]; }
                else { lo[dd] = 1; hi[dd] = o->nc[dd] + 1; }
            }
            int c[3];
            for (c[0] = lo[0]; c[0] < hi[0]; c[0]++)
                for (c[1] = lo[1]; c[1] < hi[1]; c[1]++)
                    for (c[2] = lo[2]; c[2] < hi[2]; c[2]++)
                    {
                        ocell_t *src = &o->grid[gidx(o, c[0], c[1], c[2])];
                        if (src->n == 0) continue;
                        if (!o->pbc[d])
                        {
                            src->n = 0;   /* atoms leaving an open face are dropped */
                            continue;
                        }
                        int t[3] = {c[0], c[1], c[2]};
                        t[d] = side == 0 ? c[d] + o->nc[d] : c[d] - o->nc[d];
                        ocell_t *dst = &o->grid[gidx(o, t[0], t[1], t[2])];
                        const double shift = side == 0 ? o->l[d] : -o->l[d];
                        for (int i = 0; i < src->n; i++)
                        {
                            const int j = cell_append(dst);
                            cell_copy(src, i, dst, j);
                            dst->x[3 * j + d] += shift;
                        }
                        src->n = 0;
                    }
        }
    }
}

/* re-binning of every interior atom in storage order (src/misc.c:268-308) */
int oracle_refresh(oracle_sys_t *o)
{
    for (int c = 0; c < o->ncell; c++)
    {
        ocell_t *cl = icell(o, c);
        int i = 0;
        while (i < cl->n)
        {
            int j[3];
            int bad = 0;
            for (int d = 0; d < 3; d++)
            {
                j[d] = (int)floor(cl->x[3 * i + d] / o->cellh[d]) + 1;
                if (j[d] < 0 || j[d] >= o->ng[d]) bad = 1;
            }
            if (bad)
            {
                o->err |= 1u;   /* the reference returns from the refresh here */
                return -1;
            }
            ocell_t *c2 = &o->grid[gidx(o, j[0], j[1], j[2])];
            if (c2 != cl)
            {
                const int k = cell_append(c2);
                cell_copy(cl, i, c2, k);
                cell_remove(cl, i);
            }
            else
                i++;
        }
    }
    migrate(o);
    return 0;
}

/* ------------------------------------------------------------ forces */

typedef struct
{
    double *F;      /* 3 per atom, flat index */
    double *va;
    double pe;
    double vir;     /* pair virial sum r_ij . F_ij (no reference counterpart on the hot path) */
} acc_t;

static void flat_starts(oracle_sys_t *o)
{
    int k = 0;
    for (int c = 0; c < o->ncell; c++)
    {
        o->start[c] = k;
        k += icell(o, c)->n;
    }
    o->start[o->ncell] = k;
}

/* upper half of the 3x3x3 block (codes 14..26, src/subdomain.c:146-170):
   neighbour interior cell and the image shift, or -1 across an open face */
static int upper_neighbour(const oracle_sys_t *o, int c, int code, double s[3])
{
    const int cc[3] = {c / (o->nc[1] * o->nc[2]), (c / o->nc[2]) % o->nc[1], c % o->nc[2]};
    const int off[3] = {code / 9 - 1, (code / 3) % 3 - 1, code % 3 - 1};
    int j[3];
    for (int d = 0; d < 3; d++)
    {
        j[d] = cc[d] + off[d];
        s[d] = 0.0;
        if (j[d] < 0)
        {
            if (!o->pbc[d]) return -1;
            j[d] += o->nc[d];
            s[d] = -o->l[d];
        }
        else if (j[d] >= o->nc[d])
        {
            if (!o->pbc[d]) return -1;
            j[d] -= o->nc[d];
            s[d] = o->l[d];
        }
    }
    return j[2] + o->nc[2] * (j[1] + o->nc[1] * j[0]);
}

typedef void (*pair_fn)(oracle_sys_t *o, acc_t *a, int pass, ocell_t *c1, int i1, int g1, ocell_t *c2, int i2, int g2,
                        const double s[3]);

/* one pair (i1 in c1, i2 in c2 shifted by s); pass 1 = EAM density,
   pass 0 = forces and energy.  rv = x1 - (x2 + s) (src/forces.h:25-34) */
static void pair_update(oracle_sys_t *o, acc_t *a, int pass, ocell_t *c1, int i1, int g1, ocell_t *c2, int i2,
                        int g2, const double s[3])
{
    const int k1 = c1->kind[i1], k2 = c2->kind[i2];
    const oracle_pair_t *pp = &o->pairs[k1 * o->nkinds + k2];
    double rv[3], r2 = 0.0;
    for (int d = 0; d < 3; d++)
    {
        rv[d] = c1->x[3 * i1 + d] - (c2->x[3 * i2 + d] + s[d]);
        r2 += rv[d] * rv[d];
    }
    if (pass == 1)
    {
        if (pp->cat != 2 || !(r2 < pp->p[2])) return;
        /* src/eam.h:270-352 */
        const double h = o->dr2;
        const int lo = (int)(r2 / h), hi = lo + 1;
        const double aa = hi - r2 / h, bb = 1 - aa;
        const double *rj = o->rho + (size_t)pp->jloc * o->Nr2, *rjd = o->rhoDD + (size_t)pp->jloc * o->Nr2;
        const double *ri = o->rho + (size_t)pp->iloc * o->Nr2, *rid = o->rhoDD + (size_t)pp->iloc * o->Nr2;
        a->va[g1] += SVAL(aa, bb, rj, lo, hi, rjd, h);
        a->va[g2] += SVAL(aa, bb, ri, lo, hi, rid, h);
        return;
    }
    double mag3[3];
    if (pp->cat == 1)
    {
        if (!(r2 < pp->p[2])) return;
        /* src/lj.h:39-56 */
        const double inv_r2 = 1.0 / r2;
        const double inv_rs2 = pp->p[1] * inv_r2;
        const double inv_rs6 = inv_rs2 * inv_rs2 * inv_rs2;
        const double inv_rs12 = inv_rs6 * inv_rs6;
        const double factor = 12.0 * pp->p[0] * inv_r2 * (inv_rs12 - 0.5 * inv_rs6);
        for (int d = 0; d < 3; d++) mag3[d] = rv[d] * factor;
        a->pe += pp->p[0] * (inv_rs12 - inv_rs6);
    }
    else if (pp->cat == 3)
    {
        if (!(r2 < pp->p[3])) return;
        /* src/morse.h:39-56 */
        const double r = sqrt(r2), inv_r = 1.0 / r;
        const double e1 = exp(-pp->p[1] * (r - pp->p[2])), e2 = e1 * e1;
        const double factor = 2.0 * pp->p[1] * pp->p[0] * inv_r * (e2 - e1);
        for (int d = 0; d < 3; d++) mag3[d] = factor * rv[d];
        a->pe += pp->p[0] * (e2 - 2.0 * e1);
    }
    else
    {
        if (!(r2 < pp->p[2])) return;
        /* src/eam.h:176-228 */
        const double h = o->dr2;
        const int lo = (int)(r2 / h), hi = lo + 1;
        const double aa = hi - r2 / h, bb = 1 - aa;
        const int ei = pp->iloc, ej = pp->jloc;
        const double *ph = o->phi + ((size_t)ei * o->nelem + ej) * o->Nr2;
        const double *phd = o->phiDD + ((size_t)ei * o->nelem + ej) * o->Nr2;
        const double phi_d = SDER(aa, bb, ph, lo, hi, phd, h);
        const double rho_ip = SDER(aa, bb, o->rho + (size_t)ei * o->Nr2, lo, hi, o->rhoDD + (size_t)ei * o->Nr2, h);
        const double rho_jp = (ei == ej) ? rho_ip
            : SDER(aa, bb, o->rho + (size_t)ej * o->Nr2, lo, hi, o->rhoDD + (size_t)ej * o->Nr2, h);
        const double mag = 2 * (c1->va[i1] * rho_jp + c2->va[i2] * rho_ip + phi_d);
        for (int d = 0; d < 3; d++) mag3[d] = -mag * rv[d];
        a->pe += SVAL(aa, bb, ph, lo, hi, phd, h);
    }
    for (int d = 0; d < 3; d++)
    {
        a->F[3 * g1 + d] += mag3[d];
        a->F[3 * g2 + d] -= mag3[d];
    }
    /* pair virial r_12 . F_12, F_12 = mag3 the force on atom 1 (the
       reference's only virial, src/misc.c:66-82, is unused and sums x . F,
       which is wrong under periodic images; this is the pair form over the
       same pairs and forces as src/lj.h:26-58, src/morse.h:26-58,
       src/eam.h:177-228) */
    a->vir += rv[0] * mag3[0] + rv[1] * mag3[1] + rv[2] * mag3[2];
}

/* half-shell sweep (src/lj.c:36-87): cell c, atoms i1, the 13 upper
   neighbour cells, then the same cell with i2 < i1 */
static void sweep_cell(oracle_sys_t *o, acc_t *a, int pass, int c, int group)
{
    ocell_t *c1 = icell(o, c);
    const int g0 = o->start[c];
    for (int i1 = 0; i1 < c1->n; i1++)
    {
        if (group >= 0 && c1->group[i1] != group) continue;
        if (pass == 1 && o->eam_elem[c1->kind[i1]] < 0) continue;
        for (int code = 14; code < 27; code++)
        {
            double s[3];
            const int nb = upper_neighbour(o, c, code, s);
            if (nb < 0) continue;
            ocell_t *c2 = icell(o, nb);
            const int h0 = o->start[nb];
            for (int i2 = 0; i2 < c2->n; i2++)
            {
                if (group >= 0 && c2->group[i2] != group) continue;
                pair_update(o, a, pass, c1, i1, g0 + i1, c2, i2, h0 + i2, s);
            }
        }
        const double z[3] = {0.0, 0.0, 0.0};
        for (int i2 = 0; i2 < i1; i2++)
        {
            if (group >= 0 && c1->group[i2] != group) continue;
            pair_update(o, a, pass, c1, i1, g0 + i1, c1, i2, g0 + i2, z);
        }
    }
}

static double run_pass(oracle_sys_t *o, int pass, int group, double *F, double *va, double *vir)
{
    const int n = o->start[o->ncell];
    const int nt = o->nthreads;
    double pe = 0.0;
    *vir = 0.0;
    if (nt <= 1)
    {
        acc_t a = {F, va, 0.0, 0.0};
        for (int c = 0; c < o->ncell; c++) sweep_cell(o, &a, pass, c, group);
        *vir = a.vir;
        return a.pe;
    }
    double *bufF = (double *)calloc((size_t)nt * 3 * n + 1, sizeof(double));
    double *bufV = (double *)calloc((size_t)nt * n + 1, sizeof(double));
    double *pes = (double *)calloc(nt, sizeof(double));
    double *virs = (double *)calloc(nt, sizeof(double));
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        const int t = omp_get_thread_num();
#else
        const int t = 0;
#endif
        acc_t a = {bufF + (size_t)t * 3 * n, bufV + (size_t)t * n, 0.0, 0.0};
#pragma omp for schedule(dynamic, 16)
        for (int c = 0; c < o->ncell; c++) sweep_cell(o, &a, pass, c, group);
        pes[t] = a.pe;
        virs[t] = a.vir;
#pragma omp for schedule(static)
        for (int g = 0; g < n; g++)
        {
            for (int q = 0; q < nt; q++)
            {
                for (int d = 0; d < 3; d++) F[3 * g + d] += bufF[(size_t)q * 3 * n + 3 * g + d];
                va[g] += bufV[(size_t)q * n + g];
            }
        }
    }
    for (int q = 0; q < nt; q++)
    {
        pe += pes[q];
        *vir += virs[q];
    }
    free(bufF); free(bufV); free(pes); free(virs);
    return pe;
}

/* ------------------------------------------------------------ TTM */

/* src/turi.c:38-42 */
static int ttm_window(const oracle_sys_t *o)
{
    const ottm_t *t = &o->ttm;
    return (o->time >= t->start - o->dt / 2.0) && ((o->time < t->stop + o->dt / 2.0) || t->stop < t->start);
}

/* local turi cell of a position (truncation, src/turi.c:971-973); a cell
   outside the local grid sets error bit 4 and is clamped */
static int ttm_cell(oracle_sys_t *o, const double *x)
{
    const ottm_t *t = &o->ttm;
    int c = (int)(x[2] / t->tcellh) + t->g2l;
    if (c < 0 || c >= t->nz)
    {
        o->err |= 4u;
        c = c < 0 ? 0 : t->nz - 1;
    }
    return c;
}

/* F_z += xi m (v_z - vcm_z) of the atom's cell (src/forces.c:292-330) */
static void ttm_friction(oracle_sys_t *o, int group)
{
    ottm_t *t = &o->ttm;
    for (int c = 0; c < o->ncell; c++)
    {
        ocell_t *cl = icell(o, c);
        for (int i = 0; i < cl->n; i++)
        {
            if (group >= 0 && cl->group[i] != group) continue;
            const int k = ttm_cell(o, cl->x + 3 * i);
            cl->F[3 * i + 2] += t->xi[k] * o->mass[cl->kind[i]] * (cl->v[3 * i + 2] - t->vcm[3 * k + 2]);
        }
    }
}

/* mass, vcm, number and temperature of every turi cell (src/turi.c:1112-1178,
   1190-1261): sums over all atoms of the interior cells, vcm = sum m v / M,
   T = sum m |v - vcm|^2 / (3 k_B N) */
static void ttm_fields(oracle_sys_t *o)
{
    ottm_t *t = &o->ttm;
    for (int k = t->lo; k < t->hi; k++)
    {
        t->mass[k] = 0.0;
        t->Ti[k] = 0.0;
        t->num[k] = 0;
        for (int d = 0; d < 3; d++) t->vcm[3 * k + d] = 0.0;
    }
    for (int c = 0; c < o->ncell; c++)
    {
        ocell_t *cl = icell(o, c);
        for (int i = 0; i < cl->n; i++)
        {
            const int k = ttm_cell(o, cl->x + 3 * i);
            const double m = o->mass[cl->kind[i]];
            t->mass[k] += m;
            for (int d = 0; d < 3; d++) t->vcm[3 * k + d] += m * cl->v[3 * i + d];
        }
    }
    for (int k = t->lo; k < t->hi; k++)
        for (int d = 0; d < 3; d++) t->vcm[3 * k + d] /= t->mass[k];
    for (int c = 0; c < o->ncell; c++)
    {
        ocell_t *cl = icell(o, c);
        for (int i = 0; i < cl->n; i++)
        {
            const int k = ttm_cell(o, cl->x + 3 * i);
            const double m = o->mass[cl->kind[i]];
            double vt2 = 0.0;
            for (int d = 0; d < 3; d++)
            {
                const double vt = cl->v[3 * i + d] - t->vcm[3 * k + d];
                vt2 += vt * vt;
            }
            t->Ti[k] += m * vt2;
            t->num[k]++;
        }
    }
    for (int k = t->lo; k < t->hi; k++) t->Ti[k] /= (3.0 * K_B * t->num[k]);
}

/* natural spline on tabulated knots, bisection as src/cspline.h:29-44 */
static double table_spline(const double *xs, const double *ys, const double *dd, int n, double x)
{
    int klo = 0, khi = n - 1;
    while (khi - klo > 1)
    {
        const int k = (khi + klo) >> 1;
        if (xs[k] > x) khi = k;
        else klo = k;
    }
    const double h = xs[khi] - xs[klo];
    const double a = (xs[khi] - x) / h, b = (x - xs[klo]) / h;
    return SVAL(a, b, ys, klo, khi, dd, h);
}

/* type 2: C, K (Zhigilei) and G of the active cells (src/ttm.c:154-192) */
static void ttm_type2_coeffs(oracle_sys_t *o)
{
    ottm_t *t = &o->ttm;
    const oracle_ttm_params_t *p = &t->p;
    for (int i = t->lo; i < t->hi; i++)
    {
        const double te = t->Te[i];
        if (te < 0.0) continue;
        if (te < p->T_C[0] || te > p->T_C[p->nC - 1]) o->err |= 16u;
        t->Ce[i] = table_spline(p->T_C, p->Ct, p->C_DD, p->nC, te);
        t->Ke[i] = 1. / 3. * t->Ce[i] * p->Kzh_v2 / (p->Kzh_A * (te * te) + p->Kzh_B * t->Ti[i]);
        if (te < p->T_G[0] || te > p->T_G[p->nG - 1]) o->err |= 16u;
        t->Gc[i] = table_spline(p->T_G, p->Gt, p->G_DD, p->nG, te);
    }
}

/* cell deactivation below min_atoms, activation from the count-weighted
   neighbour average, xi reset (src/ttm.c:194-248) */
static void ttm_presolve(oracle_sys_t *o)
{
    ottm_t *t = &o->ttm;
    for (int i = t->lo; i < t->hi; i++)
    {
        t->xi[i] = 0.0;
        if (t->Te[i] < 0.0 && t->num[i] >= t->p.min_atoms)
        {
            int count = 0;
            double sum = 0.0;
            const int im1 = (i == t->lo) ? 0 : i - 1;
            if (t->Te[im1] >= 0.0) { sum += t->Te[im1] * t->num[im1]; count += t->num[im1]; }
            if (t->Te[i + 1] >= 0.0) { sum += t->Te[i + 1] * t->num[i + 1]; count += t->num[i + 1]; }
            t->Te[i] = (count > 0) ? sum / count : t->Ti[i];
        }
        if (t->num[i] < t->p.min_atoms) t->Te[i] = t->Te2[i] = -1.0;
    }
    if (t->p.type == 2) ttm_type2_coeffs(o);
}

/* `ratio` explicit substeps with Neumann reflection at inactive neighbours
   and the Gaussian source, then xi (src/ttm.c:250-383) */
static void ttm_solve(oracle_sys_t *o)
{
    ottm_t *t = &o->ttm;
    const oracle_ttm_params_t *p = &t->p;
    const int calc_source = fabs(o->time - p->laser_t0) < p->laser_tdiff;
    const double dte = o->dt / p->ratio;
    for (int j = 0; j < p->ratio; j++)
    {
        double spc = 0.0;
        if (calc_source)
        {
            const double tt = o->time + j * dte - p->laser_t0;
            spc = p->laser_factor * exp(p->laser_m_2sig2_inv * (tt * tt));
        }
        for (int i = t->lo; i < t->hi; i++)
        {
            const double te = t->Te[i];
            if (te < 0) continue;
            double source = 0.0;
            if (calc_source)
            {
                const double z = (i - t->g2l + 0.5) * t->tcellh;
                source = spc * exp(p->laser_m_absdepth_inv * (z - p->frontsurf));
            }
            const int im1 = (i == t->lo) ? 0 : i - 1;
            const int ilo = (t->Te[im1] < 0) ? i : im1;
            const int ihi = (t->Te[i + 1] < 0) ? i : i + 1;
            if (p->type == 1)
                t->Te2[i] = te + dte / (p->C_gamma * te) *
                            (p->K * (t->Te[ihi] - 2 * te + t->Te[ilo]) / p->dz2 - p->G * (te - t->Ti[i]) + source);
            else
            {
                const double KeL = 0.5 * (t->Ke[i] + t->Ke[ilo]);
                const double KeR = 0.5 * (t->Ke[i] + t->Ke[ihi]);
                t->Te2[i] = te + dte / t->Ce[i] *
                            ((KeR * (t->Te[ihi] - te) - KeL * (te - t->Te[ilo])) / p->dz2 -
                             t->Gc[i] * (te - t->Ti[i]) + source);
            }
            t->xi[i] += t->Te2[i];
        }
        double *tmp = t->Te2;
        t->Te2 = t->Te;
        t->Te = tmp;
        if (p->type == 2 && j < p->ratio - 1) ttm_type2_coeffs(o);
    }
    for (int i = t->lo; i < t->hi; i++)
        if (t->num[i] >= p->min_atoms)
        {
            const double Gi = (p->type == 1) ? p->G : t->Gc[i];
            t->xi[i] = Gi * t->vol * (t->xi[i] / p->ratio - t->Ti[i]) / (3 * K_B * t->num[i] * t->Ti[i]);
        }
}

int oracle_ttm_setup(oracle_sys_t *o, int nz, int g2l_z, int lo, int hi, double tcellh_z, double tcell_volume,
                     double starttime, double stoptime, const oracle_ttm_params_t *p, double Te_init)
{
    if (nz < 3 || lo < 1 || hi > nz - 1 || lo >= hi || p->ratio < 1 || (p->type != 1 && p->type != 2)) return -1;
    ottm_t *t = &o->ttm;
    free_ttm(t);
    t->p = *p;
    if (p->type == 2)
    {
        const int nc = p->nC, ng = p->nG;
        if (nc < 2 || ng < 2) return -1;
        t->tabs = (double *)malloc(sizeof(double) * 3 * (size_t)(nc + ng));
        double *q = t->tabs;
        memcpy(q, p->T_C, sizeof(double) * nc); t->p.T_C = q; q += nc;
        memcpy(q, p->Ct, sizeof(double) * nc); t->p.Ct = q; q += nc;
        memcpy(q, p->C_DD, sizeof(double) * nc); t->p.C_DD = q; q += nc;
        memcpy(q, p->T_G, sizeof(double) * ng); t->p.T_G = q; q += ng;
        memcpy(q, p->Gt, sizeof(double) * ng); t->p.Gt = q; q += ng;
        memcpy(q, p->G_DD, sizeof(double) * ng); t->p.G_DD = q;
    }
    t->nz = nz; t->g2l = g2l_z; t->lo = lo; t->hi = hi;
    t->tcellh = tcellh_z; t->vol = tcell_volume; t->start = starttime; t->stop = stoptime;
    t->num = (unsigned *)calloc(nz, sizeof(unsigned));
    t->mass = (double *)calloc(nz, sizeof(double));
    t->vcm = (double *)calloc(3 * (size_t)nz, sizeof(double));
    t->Ti = (double *)calloc(nz, sizeof(double));
    t->Te = (double *)malloc(sizeof(double) * nz);
    t->Te2 = (double *)malloc(sizeof(double) * nz);
    t->xi = (double *)calloc(nz, sizeof(double));
    t->Ke = (double *)calloc(nz, sizeof(double));
    t->Ce = (double *)calloc(nz, sizeof(double));
    t->Gc = (double *)calloc(nz, sizeof(double));
    for (int i = 0; i < nz; i++) t->Te[i] = t->Te2[i] = (i >= lo && i < hi) ? Te_init : -1.0;
    t->on = 1;
    return 0;
}

int oracle_set_time(oracle_sys_t *o, double time, double dt)
{
    o->time = time;
    o->dt = dt;
    return 0;
}

int oracle_turi_update(oracle_sys_t *o)
{
    if (!o->ttm.on || !ttm_window(o)) return 0;
    ttm_fields(o);
    ttm_presolve(o);
    ttm_solve(o);
    return 0;
}

int oracle_ttm_1d(oracle_sys_t *o, unsigned *num, double *vcm, double *Ti, double *Te, double *xi)
{
    const ottm_t *t = &o->ttm;
    if (!t->on) return -1;
    for (int i = 0; i < t->nz; i++)
    {
        if (num) num[i] = t->num[i];
        if (Ti) Ti[i] = t->Ti[i];
        if (Te) Te[i] = t->Te[i];
        if (xi) xi[i] = t->xi[i];
        if (vcm) for (int d = 0; d < 3; d++) vcm[3 * i + d] = t->vcm[3 * i + d];
    }
    return t->nz;
}

/* src/forces.c:332-382 */
int oracle_compute_forces(oracle_sys_t *o, int group)
{
    flat_starts(o);
    const int n = o->start[o->ncell];
    double *F = (double *)calloc((size_t)3 * n + 1, sizeof(double));
    double *va = (double *)calloc((size_t)n + 1, sizeof(double));
    double emb = 0.0;
    if (o->cats & (1 << 2))
    {
        /* pass 1: host densities, then F'(rho) and the embedding energy
           (src/eam.c:160-223) */
        double unused;
        run_pass(o, 1, group, F, va, &unused);
        for (int c = 0; c < o->ncell; c++)
        {
            ocell_t *cl = icell(o, c);
            for (int i = 0; i < cl->n; i++)
            {
                const int g = o->start[c] + i;
                const int e = o->eam_elem[cl->kind[i]];
                if ((group >= 0 && cl->group[i] != group) || e < 0) { cl->va[i] = 0.0; continue; }
                const double rho = va[g], h = o->drho;
                int lo = (int)(rho / h);
                if (lo >= o->Nrho - 1 || lo < 0)
                {
                    o->err |= 2u;
                    lo = lo < 0 ? 0 : o->Nrho - 2;
                }
                const int hi = lo + 1;
                const double aa = hi - rho / h, bb = 1 - aa;
                const double *Ft = o->F + (size_t)e * o->Nrho, *Fd = o->FDD + (size_t)e * o->Nrho;
                cl->va[i] = SDER(aa, bb, Ft, lo, hi, Fd, h);
                emb += SVAL(aa, bb, Ft, lo, hi, Fd, h);
            }
        }
    }
    double vir = 0.0;
    const double pe = run_pass(o, 0, group, F, va, &vir);
    for (int c = 0; c < o->ncell; c++)
    {
        ocell_t *cl = icell(o, c);
        for (int i = 0; i < cl->n; i++)
            memcpy(cl->F + 3 * i, F + 3 * (o->start[c] + i), 3 * sizeof(double));
    }
    o->th.potential = pe + emb;
    o->th.virial = vir;
    free(F);
    free(va);
    if (o->ttm.on && ttm_window(o)) ttm_friction(o, group);
    return 0;
}

/* ------------------------------------------------------------ dynamics */

static void group_sums(oracle_sys_t *o, int group)
{
    double mv2 = 0.0, P[3] = {0, 0, 0};
    int cnt = 0;
    for (int c = 0; c < o->ncell; c++)
    {
        ocell_t *cl = icell(o, c);
        for (int i = 0; i < cl->n; i++)
        {
            if (group >= 0 && cl->group[i] != group) continue;
            cnt++;
            const double m = o->mass[cl->kind[i]];
            const double *v = cl->v + 3 * i;
            for (int d = 0; d < 3; d++) P[d] += m * v[d];
            mv2 += m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        }
    }
    o->th.kinetic = 0.5 * mv2;
    o->th.temperature = mv2 / (3.0 * cnt * K_B);
    for (int d = 0; d < 3; d++) o->th.momentum[d] = P[d];
    o->th.count = cnt;
}

int oracle_thermo(oracle_sys_t *o, int group, oracle_thermo_t *out)
{
    group_sums(o, group);
    if (out) *out = o->th;
    return 0;
}

int oracle_get_thermo(oracle_sys_t *o, oracle_thermo_t *out)
{
    *out = o->th;
    return 0;
}

/* velocity Verlet (src/integrators.c:40-126, 227-264); the Berendsen scale
   uses the temperature left by the previous step */
int oracle_vv_steps(oracle_sys_t *o, int nsteps, double dt, int group, int thermostat, double tau, double T0)
{
    for (int s = 0; s < nsteps; s++)
    {
        double lam = 1.0;
        if (thermostat) lam = sqrt(1 + dt / tau * (T0 / o->th.temperature - 1));
        for (int c = 0; c < o->ncell; c++)
        {
            ocell_t *cl = icell(o, c);
            for (int i = 0; i < cl->n; i++)
            {
                if (group >= 0 && cl->group[i] != group) continue;
                const double m = o->mass[cl->kind[i]];
                for (int d = 0; d < 3; d++)
                {
                    if (thermostat) cl->v[3 * i + d] *= lam;
                    cl->v[3 * i + d] += dt * 0.5 / m * cl->F[3 * i + d];
                    cl->x[3 * i + d] += dt * cl->v[3 * i + d];
                }
            }
        }
        if (oracle_refresh(o) != 0) return -1;
        oracle_compute_forces(o, group);
        for (int c = 0; c < o->ncell; c++)
        {
            ocell_t *cl = icell(o, c);
            for (int i = 0; i < cl->n; i++)
            {
                if (group >= 0 && cl->group[i] != group) continue;
                const double m = o->mass[cl->kind[i]];
                for (int d = 0; d < 3; d++) cl->v[3 * i + d] += dt * 0.5 / m * cl->F[3 * i + d];
            }
        }
        group_sums(o, group);
    }
    return 0;
}

/* symplectic Euler under TTM coupling (src/integrators.c:129-225): v += dt
   F / m, x += dt v, refresh, group sums; time += dt; the turi fields and
   the TTM solve; forces with the friction term */
int oracle_se_steps(oracle_sys_t *o, int nsteps, double dt, int group)
{
    o->dt = dt;
    for (int s = 0; s < nsteps; s++)
    {
        for (int c = 0; c < o->ncell; c++)
        {
            ocell_t *cl = icell(o, c);
            for (int i = 0; i < cl->n; i++)
            {
                if (group >= 0 && cl->group[i] != group) continue;
                const double m = o->mass[cl->kind[i]];
                for (int d = 0; d < 3; d++)
                {
                    cl->v[3 * i + d] += dt * cl->F[3 * i + d] / m;
                    cl->x[3 * i + d] += dt * cl->v[3 * i + d];
                }
            }
        }
        if (oracle_refresh(o) != 0) return -1;
        group_sums(o, group);
        o->time += dt;
        oracle_turi_update(o);
        oracle_compute_forces(o, group);
    }
    return 0;
}
