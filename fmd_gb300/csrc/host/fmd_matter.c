/*
 * Matter: the pre-distribution global grid, lattice builders, velocities,
 * state files, configuration files and the thermodynamic getters.
 *
 * Reference semantics: global grid creation (src/misc.c:41-62), lattice
 * builders (src/structure.c:33-265), state load/save (src/misc.c:121-266,
 * 310-422), matter operations (src/matter.c:117-648), configuration output
 * (src/matter.c:650-829).  Random numbers: the reference seeds a Mersenne
 * twister from the wall clock; here a splitmix64/xoshiro256** generator is
 * seeded from FMD_SEED (environment) or fmdx_set_seed when given, else from
 * the clock, so runs are reproducible on request.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "fmd_private.h"

/* ------------------------------------------------------------- rng */

static uint64_t splitmix64(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

unsigned long long _fmdh_rng_seed(fmd_t *md)
{
    const char *e = getenv("FMD_SEED");
    if (e != NULL)
    {
        md->seed_fixed = true;
        return strtoull(e, NULL, 10);
    }
    return (unsigned long long)time(NULL) ^ ((unsigned long long)(uintptr_t)md << 16);
}

void fmdx_set_seed(fmd_t *md, unsigned long long seed)
{
    md->seed = seed;
    md->seed_fixed = true;
    md->rng_calls = 0;
}

double _fmdh_rng_uniform(fmd_t *md, unsigned long long *state)
{
    (void)md;
    return (double)(splitmix64((uint64_t *)state) >> 11) * (1.0 / 9007199254740992.0);
}

/* Marsaglia polar method */
double _fmdh_rng_gauss(fmd_t *md, unsigned long long *state, double sigma)
{
    double u, v, s;
    do
    {
        u = 2.0 * _fmdh_rng_uniform(md, state) - 1.0;
        v = 2.0 * _fmdh_rng_uniform(md, state) - 1.0;
        s = u * u + v * v;
    } while (s >= 1.0 || s == 0.0);
    return sigma * u * sqrt(-2.0 * log(s) / s);
}

static unsigned long long new_stream(fmd_t *md)
{
    uint64_t s = md->seed * 0x100000001B3ull + (md->rng_calls++) * 0x9E3779B97F4A7C15ull;
    splitmix64(&s);
    return s;
}

/* ------------------------------------------------------ global grid */

void _fmdh_create_global_grid(fmd_t *md)
{
    const double cutoff = _fmdh_largest_cutoff(md);
    if (!(cutoff > 0.0)) return;
    for (int d = 0; d < 3; d++)
    {
        md->nc[d] = (int)(md->l[d] / cutoff);
        if (md->nc[d] < 1)
        {
            FMD_ERR(md, FMD_ERR_UNEXPECTED_POSITION, true, "box length %g below the cutoff %g", md->l[d], cutoff);
            return;
        }
        md->cellh[d] = md->l[d] / md->nc[d];
    }
    const size_t nc = (size_t)md->nc[0] * md->nc[1] * md->nc[2];
    md->ggrid = (hcell_t *)calloc(nc, sizeof(hcell_t));
    if (md->ggrid == NULL) FMD_ERR(md, FMD_ERR_UNABLE_ALLOCATE_MEM, true, "global grid of %zu cells", nc);
}

void _fmdh_ggrid_free(fmd_t *md)
{
    if (md->ggrid == NULL) return;
    const size_t nc = (size_t)md->nc[0] * md->nc[1] * md->nc[2];
    for (size_t c = 0; c < nc; c++)
    {
        hcell_t *h = &md->ggrid[c];
        free(h->x); free(h->v); free(h->group); free(h->kind); free(h->id);
    }
    free(md->ggrid);
    md->ggrid = NULL;
}

static int hcell_push(fmd_t *md, hcell_t *c)
{
    if (c->n == c->cap)
    {
        int cap = c->cap ? 2 * c->cap : 8;
        double *x = (double *)realloc(c->x, sizeof(double) * 3 * cap);
        if (x) c->x = x;
        double *v = (double *)realloc(c->v, sizeof(double) * 3 * cap);
        if (v) c->v = v;
        int *g = (int *)realloc(c->group, sizeof(int) * cap);
        if (g) c->group = g;
        unsigned *k = (unsigned *)realloc(c->kind, sizeof(unsigned) * cap);
        if (k) c->kind = k;
        unsigned *id = (unsigned *)realloc(c->id, sizeof(unsigned) * cap);
        if (id) c->id = id;
        if (!x || !v || !g || !k || !id)
        {
            FMD_ERR(md, FMD_ERR_UNABLE_ALLOCATE_MEM, true, "cell storage");
            return -1;
        }
        c->cap = cap;
    }
    return c->n++;
}

/* swap-with-last removal (src/cell.c:151-160) */
static void hcell_remove(hcell_t *c, int i)
{
    c->n--;
    if (c->n != i)
    {
        memcpy(c->x + 3 * i, c->x + 3 * c->n, 3 * sizeof(double));
        memcpy(c->v + 3 * i, c->v + 3 * c->n, 3 * sizeof(double));
        c->group[i] = c->group[c->n];
        c->kind[i] = c->kind[c->n];
        c->id[i] = c->id[c->n];
    }
}

static hcell_t *gcell_of(fmd_t *md, const double x[3])
{
    int ic[3];
    for (int d = 0; d < 3; d++)
    {
        const double q = floor(x[d] / md->cellh[d]);
        if (!(q >= 0.0 && q < md->nc[d])) return NULL;
        ic[d] = (int)q;
    }
    return md->ggrid + (ic[2] + md->nc[2] * (ic[1] + md->nc[1] * ic[0]));
}

static int add_atom(fmd_t *md, const double x[3], const double v[3], unsigned kind, int group)
{
    hcell_t *c = gcell_of(md, x);
    if (c == NULL)
    {
        FMD_ERR(md, FMD_ERR_UNEXPECTED_POSITION, false, "atom at (%g, %g, %g) is outside the box", x[0], x[1], x[2]);
        return -1;
    }
    const int j = hcell_push(md, c);
    if (j < 0) return -1;
    for (int d = 0; d < 3; d++)
    {
        c->x[3 * j + d] = x[d];
        c->v[3 * j + d] = v[d];
    }
    c->kind[j] = kind;
    c->group[j] = group;
    c->id[j] = md->TotalNoOfParticles++;
    return 0;
}

static size_t ggrid_ncells(const fmd_t *md) { return (size_t)md->nc[0] * md->nc[1] * md->nc[2]; }

/* ------------------------------------------------------- lattices */

typedef enum { LAT_SC, LAT_BCC, LAT_FCC } lattice_t;

static void make_cuboid(fmd_t *md, lattice_t lt, double x0, double y0, double z0, int dimx, int dimy,
                        int dimz, double lp, const double *ratio, int GroupID, double temp)
{
    static const double r_fcc[4][3] = {{0.0, 0.0, 0.0}, {0.0, 0.5, 0.5}, {0.5, 0.0, 0.5}, {0.5, 0.5, 0.0}};
    static const double r_bcc[2][3] = {{0.0, 0.0, 0.0}, {0.5, 0.5, 0.5}};
    static const double r_sc[1][3] = {{0.0, 0.0, 0.0}};
    const double (*rp)[3] = lt == LAT_FCC ? r_fcc : (lt == LAT_BCC ? r_bcc : r_sc);
    const int ppc = lt == LAT_FCC ? 4 : (lt == LAT_BCC ? 2 : 1);

    if (md->ParticlesDistributed)
    {
        FMD_ERR(md, FMD_ERR_NOT_SUPPORTED_YET, false, "matter cannot be added after the first run");
        return;
    }
    if (md->ggrid == NULL) _fmdh_create_global_grid(md);
    if (md->ggrid == NULL) return;
    if (GroupID == md->ActiveGroup || md->ActiveGroup == FMD_GROUP_ALL) md->KineticEnergyUpdated = false;
    if (GroupID < 0)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "GroupID %d", GroupID);
        return;
    }
    double cum[FMD_MAX_KINDS], sum = 0.0;
    for (unsigned k = 0; k < md->nkinds; k++) cum[k] = (sum += ratio[k]);
    unsigned long long st = new_stream(md);
    double P[3] = {0.0, 0.0, 0.0};
    const double r0[3] = {x0, y0, z0};
    long added = 0;
    int cc[3];
    for (cc[0] = 0; cc[0] < dimx; cc[0]++)
        for (cc[1] = 0; cc[1] < dimy; cc[1]++)
            for (cc[2] = 0; cc[2] < dimz; cc[2]++)
                for (int p = 0; p < ppc; p++)
                {
                    double x[3], v[3];
                    for (int d = 0; d < 3; d++) x[d] = r0[d] + (cc[d] + .25 + rp[p][d]) * lp;
                    const double rn = sum * _fmdh_rng_uniform(md, &st);
                    unsigned k;
                    for (k = 0; k < md->nkinds; k++)
                        if (rn < cum[k]) break;
                    if (k == md->nkinds) k = md->nkinds - 1;
                    const double m = md->kinds[k].mass;
                    const double sd = sqrt(FMD_K_BOLTZMANN * temp / m);
                    for (int d = 0; d < 3; d++)
                    {
                        v[d] = _fmdh_rng_gauss(md, &st, sd);
                        P[d] += m * v[d];
                    }
                    if (add_atom(md, x, v, k, FMD_RESERVED_GROUP) == 0) added++;
                }
    /* remove the net momentum of the new atoms (src/structure.c:33-51) */
    const long natoms = (long)ppc * dimx * dimy * dimz;
    for (size_t c = 0; c < ggrid_ncells(md); c++)
    {
        hcell_t *h = &md->ggrid[c];
        for (int i = 0; i < h->n; i++)
            if (h->group[i] == FMD_RESERVED_GROUP)
            {
                h->group[i] = GroupID;
                const double m = md->kinds[h->kind[i]].mass;
                for (int d = 0; d < 3; d++) h->v[3 * i + d] -= P[d] / (natoms * m);
            }
    }
    (void)added;
}

static void cuboid_single(fmd_t *md, lattice_t lt, double x, double y, double z, int dx, int dy, int dz,
                          double lp, unsigned kind, int g, double T)
{
    if (kind >= md->nkinds)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "atom kind %u", kind);
        return;
    }
    double ratio[FMD_MAX_KINDS] = {0};
    ratio[kind] = 1.0;
    make_cuboid(md, lt, x, y, z, dx, dy, dz, lp, ratio, g, T);
}

void fmd_matt_makeCuboidSC(fmd_t *md, fmd_real_t x, fmd_real_t y, fmd_real_t z, int dimx, int dimy, int dimz,
                           fmd_real_t lp, unsigned atomkind, int GroupID, fmd_real_t temp)
{ cuboid_single(md, LAT_SC, x, y, z, dimx, dimy, dimz, lp, atomkind, GroupID, temp); }
void fmd_matt_makeCuboidBCC(fmd_t *md, fmd_real_t x, fmd_real_t y, fmd_real_t z, int dimx, int dimy, int dimz,
                            fmd_real_t lp, unsigned atomkind, int GroupID, fmd_real_t temp)
{ cuboid_single(md, LAT_BCC, x, y, z, dimx, dimy, dimz, lp, atomkind, GroupID, temp); }
void fmd_matt_makeCuboidFCC(fmd_t *md, fmd_real_t x, fmd_real_t y, fmd_real_t z, int dimx, int dimy, int dimz,
                            fmd_real_t lp, unsigned atomkind, int GroupID, fmd_real_t temp)
{ cuboid_single(md, LAT_FCC, x, y, z, dimx, dimy, dimz, lp, atomkind, GroupID, temp); }
void fmd_matt_makeCuboidSC_mix(fmd_t *md, fmd_real_t x, fmd_real_t y, fmd_real_t z, int dimx, int dimy, int dimz,
                               fmd_real_t lp, fmd_real_t ratio[], int GroupID, fmd_real_t temp)
{ make_cuboid(md, LAT_SC, x, y, z, dimx, dimy, dimz, lp, ratio, GroupID, temp); }
void fmd_matt_makeCuboidBCC_mix(fmd_t *md, fmd_real_t x, fmd_real_t y, fmd_real_t z, int dimx, int dimy, int dimz,
                                fmd_real_t lp, fmd_real_t ratio[], int GroupID, fmd_real_t temp)
{ make_cuboid(md, LAT_BCC, x, y, z, dimx, dimy, dimz, lp, ratio, GroupID, temp); }
void fmd_matt_makeCuboidFCC_mix(fmd_t *md, fmd_real_t x, fmd_real_t y, fmd_real_t z, int dimx, int dimy, int dimz,
                                fmd_real_t lp, fmd_real_t ratio[], int GroupID, fmd_real_t temp)
{ make_cuboid(md, LAT_FCC, x, y, z, dimx, dimy, dimz, lp, ratio, GroupID, temp); }

/* -------------------------------------------- device distribution */

static bool ensure_device(fmd_t *md)
{
    if (md->dev == NULL)
    {
        int dev = 0;
        const char *e = getenv("FMD_DEVICE");
        if (e) dev = atoi(e);
        if (!_fmdh_dev_ok(md, fmdg_create(&md->dev, dev), "fmdg_create")) return false;
    }
    return true;
}

/* Single-rank distribution (src/matter.c:399-447): the global grid's cells,
   in cell order and insertion order, become the device system. */
bool _fmdh_distribute(fmd_t *md)
{
    if (md->ParticlesDistributed) return true;
    if (!_fmdh_pots_ready(md)) return false;
    if (md->ggrid == NULL) _fmdh_create_global_grid(md);
    if (md->ggrid == NULL) return false;
    if (!ensure_device(md)) return false;
    int pbc[3] = {md->PBC[0], md->PBC[1], md->PBC[2]};
    if (!_fmdh_dev_ok(md, fmdg_set_box(md->dev, md->l, pbc, md->nc, md->cellh), "fmdg_set_box")) return false;
    md->dev_tables_ok = false;
    if (!_fmdh_dev_ok(md, _fmdh_upload_tables(md), "upload tables")) return false;
    const size_t ncell = ggrid_ncells(md);
    size_t n = 0;
    for (size_t c = 0; c < ncell; c++) n += md->ggrid[c].n;
    int *count = (int *)malloc(sizeof(int) * ncell);
    double *x = (double *)malloc(sizeof(double) * 3 * (n ? n : 1));
    double *v = (double *)malloc(sizeof(double) * 3 * (n ? n : 1));
    unsigned *kind = (unsigned *)malloc(sizeof(unsigned) * (n ? n : 1));
    int *group = (int *)malloc(sizeof(int) * (n ? n : 1));
    unsigned *id = (unsigned *)malloc(sizeof(unsigned) * (n ? n : 1));
    size_t k = 0;
    for (size_t c = 0; c < ncell; c++)
    {
        const hcell_t *h = &md->ggrid[c];
        count[c] = h->n;
        for (int i = 0; i < h->n; i++, k++)
        {
            memcpy(x + 3 * k, h->x + 3 * i, 3 * sizeof(double));
            memcpy(v + 3 * k, h->v + 3 * i, 3 * sizeof(double));
            kind[k] = h->kind[i];
            group[k] = h->group[i];
            id[k] = h->id[i];
        }
    }
    const int rc = fmdg_upload(md->dev, (int)n, count, x, v, kind, group, id);
    free(count); free(x); free(v); free(kind); free(group); free(id);
    if (!_fmdh_dev_ok(md, rc, "fmdg_upload")) return false;
    _fmdh_ggrid_free(md);
    md->ParticlesDistributed = true;
    return true;
}

/* Current atoms in cell order (device copy after distribution, else the
   global grid).  Arrays are malloc'ed; the caller frees them. */
int _fmdh_current_atoms(fmd_t *md, int *n, double **x, double **v, unsigned **kind, int **group, unsigned **id)
{
    *x = *v = NULL; *kind = NULL; *group = NULL; *id = NULL; *n = 0;
    if (md->ParticlesDistributed)
    {
        int na = 0;
        if (fmdg_natoms(md->dev, &na)) return -1;
        const size_t m = na > 0 ? (size_t)na : 1;
        *x = (double *)malloc(sizeof(double) * 3 * m);
        *v = (double *)malloc(sizeof(double) * 3 * m);
        *kind = (unsigned *)malloc(sizeof(unsigned) * m);
        *group = (int *)malloc(sizeof(int) * m);
        *id = (unsigned *)malloc(sizeof(unsigned) * m);
        if (fmdg_download(md->dev, NULL, *x, *v, NULL, NULL, *kind, *group, *id)) return -1;
        *n = na;
        return 0;
    }
    if (md->ggrid == NULL) return 0;
    size_t na = 0;
    for (size_t c = 0; c < ggrid_ncells(md); c++) na += md->ggrid[c].n;
    const size_t m = na > 0 ? na : 1;
    *x = (double *)malloc(sizeof(double) * 3 * m);
    *v = (double *)malloc(sizeof(double) * 3 * m);
    *kind = (unsigned *)malloc(sizeof(unsigned) * m);
    *group = (int *)malloc(sizeof(int) * m);
    *id = (unsigned *)malloc(sizeof(unsigned) * m);
    size_t k = 0;
    for (size_t c = 0; c < ggrid_ncells(md); c++)
    {
        const hcell_t *h = &md->ggrid[c];
        for (int i = 0; i < h->n; i++, k++)
        {
            memcpy(*x + 3 * k, h->x + 3 * i, 3 * sizeof(double));
            memcpy(*v + 3 * k, h->v + 3 * i, 3 * sizeof(double));
            (*kind)[k] = h->kind[i];
            (*group)[k] = h->group[i];
            (*id)[k] = h->id[i];
        }
    }
    *n = (int)na;
    return 0;
}

/* ------------------------------------------------ matter operations */

void fmd_matt_addVelocity(fmd_t *md, int GroupID, fmd_real_t vx, fmd_real_t vy, fmd_real_t vz)
{
    if (md->ParticlesDistributed)
    {
        const double dv[3] = {vx, vy, vz};
        _fmdh_dev_ok(md, fmdg_add_velocity(md->dev, GroupID, dv), "fmdg_add_velocity");
    }
    else if (md->ggrid != NULL)
    {
        for (size_t c = 0; c < ggrid_ncells(md); c++)
        {
            hcell_t *h = &md->ggrid[c];
            for (int i = 0; i < h->n; i++)
                if (GroupID == FMD_GROUP_ALL || GroupID == h->group[i])
                {
                    h->v[3 * i] += vx;
                    h->v[3 * i + 1] += vy;
                    h->v[3 * i + 2] += vz;
                }
        }
    }
    if (md->ActiveGroup == FMD_GROUP_ALL || GroupID == FMD_GROUP_ALL || md->ActiveGroup == GroupID)
        md->KineticEnergyUpdated = false;
}

void fmd_matt_changeGroupID(fmd_t *md, int old, int new)
{
    if (new < 0)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "GroupID %d", new);
        return;
    }
    if (md->ParticlesDistributed)
        _fmdh_dev_ok(md, fmdg_change_group(md->dev, old, new), "fmdg_change_group");
    else if (md->ggrid != NULL)
        for (size_t c = 0; c < ggrid_ncells(md); c++)
        {
            hcell_t *h = &md->ggrid[c];
            for (int i = 0; i < h->n; i++)
                if (old == FMD_GROUP_ALL || h->group[i] == old) h->group[i] = new;
        }
    if (md->ActiveGroup != FMD_GROUP_ALL && (md->ActiveGroup == old || md->ActiveGroup == new))
        md->KineticEnergyUpdated = false;
}

void fmd_matt_findLimits(fmd_t *md, int GroupID, fmd_rtriple_t LowerLimit, fmd_rtriple_t UpperLimit)
{
    int n;
    double *x, *v;
    unsigned *kind, *id;
    int *group;
    for (int d = 0; d < 3; d++)
    {
        LowerLimit[d] = 1.7976931348623157e308;
        UpperLimit[d] = 2.2250738585072014e-308;   /* DBL_MIN, as src/matter.c:215-218 */
    }
    if (_fmdh_current_atoms(md, &n, &x, &v, &kind, &group, &id) == 0)
        for (int i = 0; i < n; i++)
            if (GroupID == FMD_GROUP_ALL || GroupID == group[i])
                for (int d = 0; d < 3; d++)
                {
                    if (x[3 * i + d] < LowerLimit[d]) LowerLimit[d] = x[3 * i + d];
                    if (x[3 * i + d] > UpperLimit[d]) UpperLimit[d] = x[3 * i + d];
                }
    free(x); free(v); free(kind); free(group); free(id);
}

/* translation before distribution (src/matter.c:483-566): atoms leaving a
   non-periodic face are deleted, periodic ones wrapped; then re-binned */
void fmd_matt_translate(fmd_t *md, int GroupID, fmd_real_t dx, fmd_real_t dy, fmd_real_t dz)
{
    if (md->ParticlesDistributed)
    {
        FMD_ERR(md, FMD_ERR_NOT_SUPPORTED_YET, false,
                "matter cannot be translated after particles are distributed");
        return;
    }
    if (md->ActiveGroup == FMD_GROUP_ALL || GroupID == FMD_GROUP_ALL || md->ActiveGroup == GroupID)
        if ((!md->PBC[0] && dx != 0.) || (!md->PBC[1] && dy != 0.) || (!md->PBC[2] && dz != 0.))
            md->KineticEnergyUpdated = false;
    if (md->ggrid == NULL) return;
    const double dr[3] = {dx, dy, dz};
    const size_t nc = ggrid_ncells(md);
    for (size_t c = 0; c < nc; c++)
    {
        hcell_t *h = &md->ggrid[c];
        for (int i = 0; i < h->n; i++)
            if (GroupID == FMD_GROUP_ALL || GroupID == h->group[i])
                for (int d = 0; d < 3; d++)
                {
                    double *x = &h->x[3 * i + d];
                    *x += dr[d];
                    if (*x < 0.0 || *x >= md->l[d])
                    {
                        if (!md->PBC[d])
                        {
                            hcell_remove(h, i);
                            md->TotalNoOfParticles--;
                            i--;
                            break;
                        }
                        *x += (*x < 0.0 ? md->l[d] : -md->l[d]);
                    }
                }
    }
    for (size_t c = 0; c < nc; c++)
    {
        hcell_t *h = &md->ggrid[c];
        for (int i = 0; i < h->n; i++)
            if (GroupID == FMD_GROUP_ALL || GroupID == h->group[i])
            {
                hcell_t *c2 = gcell_of(md, h->x + 3 * i);
                if (c2 == NULL)
                {
                    FMD_ERR(md, FMD_ERR_UNEXPECTED_POSITION, false, "translated atom left the box");
                    return;
                }
                if (c2 != h)
                {
                    const int j = hcell_push(md, c2);
                    if (j < 0) return;
                    memcpy(c2->x + 3 * j, h->x + 3 * i, 3 * sizeof(double));
                    memcpy(c2->v + 3 * j, h->v + 3 * i, 3 * sizeof(double));
                    c2->group[j] = h->group[i];
                    c2->kind[j] = h->kind[i];
                    c2->id[j] = h->id[i];
                    hcell_remove(h, i);
                    i--;
                }
            }
    }
}

void fmd_matt_giveMaxwellDistribution(fmd_t *md, int GroupID, fmd_real_t temp)
{
    int n;
    double *x, *v;
    unsigned *kind, *id;
    int *group;
    unsigned long long st = new_stream(md);
    if (md->ParticlesDistributed)
    {
        if (_fmdh_current_atoms(md, &n, &x, &v, &kind, &group, &id) == 0)
        {
            for (int i = 0; i < n; i++)
                if (GroupID == FMD_GROUP_ALL || GroupID == group[i])
                {
                    const double sd = sqrt(FMD_K_BOLTZMANN * temp / md->kinds[kind[i]].mass);
                    for (int d = 0; d < 3; d++) v[3 * i + d] = _fmdh_rng_gauss(md, &st, sd);
                }
            _fmdh_dev_ok(md, fmdg_set_state(md->dev, NULL, v), "fmdg_set_state");
        }
        free(x); free(v); free(kind); free(group); free(id);
    }
    else if (md->ggrid != NULL)
    {
        for (size_t c = 0; c < ggrid_ncells(md); c++)
        {
            hcell_t *h = &md->ggrid[c];
            for (int i = 0; i < h->n; i++)
                if (GroupID == FMD_GROUP_ALL || GroupID == h->group[i])
                {
                    const double sd = sqrt(FMD_K_BOLTZMANN * temp / md->kinds[h->kind[i]].mass);
                    for (int d = 0; d < 3; d++) h->v[3 * i + d] = _fmdh_rng_gauss(md, &st, sd);
                }
        }
    }
    if (md->ActiveGroup == FMD_GROUP_ALL || GroupID == FMD_GROUP_ALL || md->ActiveGroup == GroupID)
        md->KineticEnergyUpdated = false;
}

/* ------------------------------------------------ thermodynamics */

/* copy the device's last thermo record into the cache */
void _fmdh_thermo_from_device(fmd_t *md)
{
    fmdg_thermo_t th;
    if (!_fmdh_dev_ok(md, fmdg_get_thermo(md->dev, &th), "fmdg_get_thermo")) return;
    md->GroupKineticEnergy = th.kinetic;
    md->GroupTemperature = th.temperature;
    for (int d = 0; d < 3; d++) md->GroupMomentum[d] = th.momentum[d];
    md->GroupParticlesNum = (unsigned)th.count;
    md->GroupPotentialEnergy = th.potential;
    md->GroupVirial = th.virial;
    md->thermo_pending = false;
}

/* KE, T, momentum of the active group from the current velocities
   (src/matter.c:31-115) */
void _fmdh_thermo_refresh(fmd_t *md)
{
    if (md->ParticlesDistributed)
    {
        fmdg_thermo_t th;
        if (!_fmdh_dev_ok(md, fmdg_thermo(md->dev, md->ActiveGroup, &th), "fmdg_thermo")) return;
        md->GroupKineticEnergy = th.kinetic;
        md->GroupTemperature = th.temperature;
        for (int d = 0; d < 3; d++) md->GroupMomentum[d] = th.momentum[d];
        md->GroupParticlesNum = (unsigned)th.count;
    }
    else
    {
        /* global-grid variant (src/matter.c:70-115) */
        double m_v2 = 0.0;
        unsigned cnt = 0;
        double P[3] = {0, 0, 0};
        if (md->ggrid != NULL)
            for (size_t c = 0; c < ggrid_ncells(md); c++)
            {
                const hcell_t *h = &md->ggrid[c];
                for (int i = 0; i < h->n; i++)
                {
                    if (md->ActiveGroup != FMD_GROUP_ALL && h->group[i] != md->ActiveGroup) continue;
                    cnt++;
                    const double m = md->kinds[h->kind[i]].mass;
                    for (int d = 0; d < 3; d++)
                    {
                        m_v2 += m * h->v[3 * i + d] * h->v[3 * i + d];
                        P[d] += m * h->v[3 * i + d];
                    }
                }
            }
        md->GroupParticlesNum = cnt;
        md->GroupTemperature = m_v2 / (3.0 * cnt * FMD_K_BOLTZMANN);
        for (int d = 0; d < 3; d++) md->GroupMomentum[d] = P[d];
        md->GroupKineticEnergy = 3.0 / 2.0 * cnt * FMD_K_BOLTZMANN * md->GroupTemperature;
    }
    md->KineticEnergyUpdated = true;
    md->thermo_pending = false;
}

static void thermo_current(fmd_t *md)
{
    if (md->thermo_pending) _fmdh_thermo_from_device(md);
    if (!md->KineticEnergyUpdated) _fmdh_thermo_refresh(md);
}

fmd_real_t fmd_matt_getKineticEnergy(fmd_t *md)
{
    thermo_current(md);
    return md->GroupKineticEnergy;
}

fmd_real_t fmd_matt_getTotalEnergy(fmd_t *md)
{
    thermo_current(md);
    return md->GroupKineticEnergy + md->GroupPotentialEnergy;
}

fmd_real_t fmd_matt_getTemperature(fmd_t *md)
{
    thermo_current(md);
    return md->GroupTemperature;
}

void fmd_matt_getMomentum(fmd_t *md, fmd_rtriple_t out)
{
    thermo_current(md);
    for (int d = 0; d < 3; d++) out[d] = md->GroupMomentum[d] * FMD_MASS_UNIT;
}

/* ------------------------------------------------------ state files */

void fmd_io_loadState(fmd_t *md, fmd_string_t path, bool UseTime)
{
    FILE *fp = fopen(path, "r");
    if (fp == NULL) { FMD_ERR(md, FMD_ERR_UNABLE_OPEN_FILE, false, "%s", path); return; }
    double t, l0, l1, l2;
    unsigned num;
    int p0, p1, p2;
    if (fscanf(fp, "%lf", &t) != 1 || fscanf(fp, "%u\n", &num) != 1 ||
        fscanf(fp, "%lf%lf%lf", &l0, &l1, &l2) != 3 || fscanf(fp, "%d%d%d", &p0, &p1, &p2) != 3)
    {
        FMD_ERR(md, FMD_ERR_FILE_CORRUPTED, false, "state file %s", path);
        fclose(fp);
        return;
    }
    if (md->ParticlesDistributed)
    {
        FMD_ERR(md, FMD_ERR_NOT_SUPPORTED_YET, false, "a state cannot be loaded after the first run");
        fclose(fp);
        return;
    }
    if (UseTime) md->time = t;
    if (!md->BoxSizeDetermined)
    {
        md->l[0] = l0; md->l[1] = l1; md->l[2] = l2;
        md->BoxSizeDetermined = true;
    }
    if (!md->PBCdetermined)
    {
        md->PBC[0] = p0; md->PBC[1] = p1; md->PBC[2] = p2;
        md->PBCdetermined = true;
    }
    if (md->ggrid == NULL) _fmdh_create_global_grid(md);
    if (md->ggrid == NULL) { fclose(fp); return; }
    for (unsigned i = 0; i < num; i++)
    {
        char name[64];
        int GroupID;
        double x[3], v[3];
        if (fscanf(fp, "%63s%d", name, &GroupID) != 2)
        {
            FMD_ERR(md, FMD_ERR_FILE_CORRUPTED, false, "state file %s", path);
            break;
        }
        if (GroupID < 0)
        {
            FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "GroupID %d", GroupID);
            break;
        }
        unsigned k;
        for (k = 0; k < md->nkinds; k++)
            if (strcmp(name, md->kinds[k].name) == 0) break;
        if (k == md->nkinds)
        {
            FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "atomkind %s", name);
            break;
        }
        if (fscanf(fp, "%lf%lf%lf", &x[0], &x[1], &x[2]) != 3 || fscanf(fp, "%lf%lf%lf", &v[0], &v[1], &v[2]) != 3)
        {
            FMD_ERR(md, FMD_ERR_FILE_CORRUPTED, false, "state file %s", path);
            break;
        }
        add_atom(md, x, v, k, GroupID);
    }
    fclose(fp);
    md->KineticEnergyUpdated = false;
}

static const char *fmt3 = "%.16e\t%.16e\t%.16e\n";

void fmd_io_saveState(fmd_t *md, fmd_string_t filename)
{
    char path[FMD_MAX_PATH * 2];
    snprintf(path, sizeof path, "%s%s", md->SaveDirectory, filename);
    int n;
    double *x, *v;
    unsigned *kind, *id;
    int *group;
    if (_fmdh_current_atoms(md, &n, &x, &v, &kind, &group, &id) != 0)
    {
        FMD_ERR(md, FMD_ERR_FUNCTION_FAILED, false, "reading atoms: %s", fmdg_last_error());
        return;
    }
    FILE *fp = fopen(path, "w");
    if (fp == NULL)
    {
        FMD_ERR(md, FMD_ERR_UNABLE_OPEN_FILE, false, "%s", path);
    }
    else
    {
        if (md->ParticlesDistributed) md->TotalNoOfParticles = (unsigned)n;
        fprintf(fp, "%.16e\n", md->time);
        fprintf(fp, "%u\n", md->TotalNoOfParticles);
        fprintf(fp, fmt3, md->l[0], md->l[1], md->l[2]);
        fprintf(fp, "%d %d %d\n", md->PBC[0], md->PBC[1], md->PBC[2]);
        for (int i = 0; i < n; i++)
        {
            fprintf(fp, "%s %d\n", md->kinds[kind[i]].name, group[i]);
            fprintf(fp, fmt3, x[3 * i], x[3 * i + 1], x[3 * i + 2]);
            fprintf(fp, fmt3, v[3 * i], v[3 * i + 1], v[3 * i + 2]);
        }
        fclose(fp);
    }
    free(x); free(v); free(kind); free(group); free(id);
}

/* ------------------------------------------------ configuration files */

typedef struct { float x[3]; float var; unsigned kind; } cfg_atom_t;

static void save_xyz(fmd_t *md, FILE *fp, const cfg_atom_t *a, int n)
{
    fprintf(fp, "%d\n\n", n);
    for (unsigned k = 0; k < md->nkinds; k++)
        for (int i = 0; i < n; i++)
            if (a[i].kind == k)
                fprintf(fp, "%s\t%.2f\t%.2f\t%.2f\n", md->kinds[k].name, a[i].x[0], a[i].x[1], a[i].x[2]);
}

void fmd_matt_saveConfiguration(fmd_t *md)
{
    int n;
    double *x, *v;
    unsigned *kind, *id;
    int *group;
    if (!md->ParticlesDistributed)
    {
        /* the reference writes the distributed local grid only */
        FMD_ERR(md, FMD_ERR_UNPREPARED, false, "configuration before the first run");
        return;
    }
    if (_fmdh_current_atoms(md, &n, &x, &v, &kind, &group, &id) != 0)
    {
        FMD_ERR(md, FMD_ERR_FUNCTION_FAILED, false, "reading atoms: %s", fmdg_last_error());
        return;
    }
    cfg_atom_t *a = (cfg_atom_t *)malloc(sizeof(cfg_atom_t) * (n > 0 ? n : 1));
    for (int i = 0; i < n; i++)
    {
        for (int d = 0; d < 3; d++) a[i].x[d] = (float)x[3 * i + d];
        a[i].var = (float)group[i];
        a[i].kind = kind[i];
    }
    md->TotalNoOfParticles = (unsigned)n;
    char path[FMD_MAX_PATH * 2];
    FILE *fp;
    switch (md->SaveConfigMode)
    {
        case FMD_SCM_XYZ_ATOMSNUM:
            if ((int)md->TotalNoOfParticles != md->OldNumberOfParticles)
            {
                if (md->OldNumberOfParticles != -1 && md->ConfigFilep) fclose(md->ConfigFilep);
                snprintf(path, sizeof path, "%s%d.xyz", md->SaveDirectory, (int)md->TotalNoOfParticles);
                md->ConfigFilep = fopen(path, "w");
                md->OldNumberOfParticles = (int)md->TotalNoOfParticles;
                if (md->ConfigFilep == NULL)
                {
                    md->OldNumberOfParticles = -1;
                    FMD_ERR(md, FMD_ERR_UNABLE_OPEN_FILE, false, "%s", path);
                    break;
                }
            }
            save_xyz(md, md->ConfigFilep, a, n);
            fflush(md->ConfigFilep);
            break;
        case FMD_SCM_XYZ_SEPARATE:
            snprintf(path, sizeof path, "%s%05d.xyz", md->SaveDirectory, md->FileIndex++);
            fp = fopen(path, "w");
            if (fp == NULL) { FMD_ERR(md, FMD_ERR_UNABLE_OPEN_FILE, false, "%s", path); break; }
            save_xyz(md, fp, a, n);
            fclose(fp);
            break;
        case FMD_SCM_CSV:
            snprintf(path, sizeof path, "%s%05d.csv", md->SaveDirectory, md->FileIndex++);
            fp = fopen(path, "w");
            if (fp == NULL) { FMD_ERR(md, FMD_ERR_UNABLE_OPEN_FILE, false, "%s", path); break; }
            for (unsigned k = 0; k < md->nkinds; k++)
                for (int i = 0; i < n; i++)
                    if (a[i].kind == k)
                        fprintf(fp, "%.2f, %.2f, %.2f, %d, %.4f\n", a[i].x[0], a[i].x[1], a[i].x[2], (int)k, a[i].var);
            fclose(fp);
            break;
        case FMD_SCM_VTF:
        {
            snprintf(path, sizeof path, "%s%05d.vtf", md->SaveDirectory, md->FileIndex++);
            fp = fopen(path, "w");
            if (fp == NULL) { FMD_ERR(md, FMD_ERR_UNABLE_OPEN_FILE, false, "%s", path); break; }
            int aid = 0;
            for (unsigned k = 0; k < md->nkinds; k++)
            {
                int count = 0;
                for (int i = 0; i < n; i++)
                    if (a[i].kind == k) count++;
                fprintf(fp, "atom %d:%d\tname %s\n", aid, aid + count - 1, md->kinds[k].name);
                aid += count;
            }
            aid = 0;
            for (unsigned k = 0; k < md->nkinds; k++)
                for (int i = 0; i < n; i++)
                    if (a[i].kind == k) fprintf(fp, "%d\tbeta %.4f\n", aid++, a[i].var);
            fprintf(fp, "timestep\n");
            for (unsigned k = 0; k < md->nkinds; k++)
                for (int i = 0; i < n; i++)
                    if (a[i].kind == k) fprintf(fp, "%.2f\t%.2f\t%.2f\n", a[i].x[0], a[i].x[1], a[i].x[2]);
            fclose(fp);
            break;
        }
    }
    free(a);
    free(x); free(v); free(kind); free(group); free(id);
}
