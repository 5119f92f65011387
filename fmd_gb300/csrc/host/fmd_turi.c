/*
 * Continuum grids ("turies"), their fields, the two-temperature model and
 * the symplectic-Euler time loop used under TTM coupling.
 *
 * Reference semantics (FMD 0.4.0):
 *   turi geometry ......... src/turi.c:648-738 (one subdomain: itc_glob_to_loc
 *                           = itc_start; 1-D TTM grids have a one-cell margin
 *                           at both ends along z)
 *   fields, dependencies .. src/turi.c:1420-1507
 *   update order, events .. src/turi.c:959-1373, 1509-1665.  The test that
 *                           selects per-step updates,
 *                           `cat == FMD_TURI_TTM_TYPE1 || FMD_TURI_TTM_TYPE2`
 *                           (src/turi.c:1635), is always true, so every
 *                           field of every turi is updated every step; this
 *                           is reproduced.
 *   field arrays .......... src/turi.c:267-397, 1667-1721
 *   TTM set-up ............ src/ttm.c:63-80, 385-548, 549-816
 *   time loop ............. src/integrators.c:181-225
 * The per-cell sums and the electron solver run on the GPU (fmdg_turi.cu).
 * The reference leaves the two margin cells of a 1-D TTM grid uninitialised
 * (src/array.c malloc); here they hold Te = -1, i.e. an inactive neighbour,
 * which gives a zero-flux boundary at both ends of the grid.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "fmd_private.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#define MAX_FIELDS 8
#define MAX_TURIES 4

typedef struct
{
    fmd_field_t cat;
    int deps[2];
    int ndeps;
} hfield_t;

struct turi
{
    fmd_turi_t cat;
    int tdims_global[3];
    int itc_start[3], itc_stop[3], tdims_local[3];
    double tcellh[3], tcell_volume;
    double starttime, stoptime;
    hfield_t fields[MAX_FIELDS];
    int nfields;
    int dev;                 /* device handle, -1 before upload */
    /* TTM */
    int is_ttm;
    int iTe, ixi;
    double C_gamma, K, G;
    double Kzh_v2, Kzh_A, Kzh_B;
    int nC, nG;
    double *T_C, *Ct, *C_DD, *T_G, *Gt, *G_DD;
    double Te_init;
    bool Te_set;
    int ratio;
    double CellActivFrac;
    double laser_t0, laser_tdiff, laser_m_2sig2_inv, laser_m_absdepth_inv, laser_factor;
    bool laser_set;
    double frontsurf;
    unsigned initial_atoms_num, min_atoms_num;
    bool in_te_event;        /* handler is running for this turi's Te event */
    int last_iter;           /* time_iteration of the last field update */
};

struct _fmd_array3s
{
    void ***data;
    fmd_utriple_t dims;
    size_t elsize;
};

static turi_t *get_turi(fmd_t *md, fmd_handle_t h)
{
    if (h < 0 || h >= md->turies_num)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "turi handle %d", h);
        return NULL;
    }
    return &md->turies[h];
}

/* ------------------------------------------------------------ fields */

static int field_add(fmd_t *md, turi_t *t, fmd_field_t cat)
{
    int dep1 = -1, dep2 = -1;
    switch (cat)
    {
        case FMD_FIELD_TEMPERATURE:
            dep1 = field_add(md, t, FMD_FIELD_NUMBER);
            dep2 = field_add(md, t, FMD_FIELD_VCM);
            break;
        case FMD_FIELD_VCM: dep1 = field_add(md, t, FMD_FIELD_MASS); break;
        case FMD_FIELD_NUMBER_DENSITY: dep1 = field_add(md, t, FMD_FIELD_NUMBER); break;
        case FMD_FIELD_TTM_TE:
        case FMD_FIELD_TTM_XI: dep1 = field_add(md, t, FMD_FIELD_TEMPERATURE); break;
        default: break;
    }
    for (int i = 0; i < t->nfields; i++)
        if (t->fields[i].cat == cat) return i;
    if (t->nfields == MAX_FIELDS) return -1;
    hfield_t *f = &t->fields[t->nfields];
    f->cat = cat;
    f->deps[0] = dep1;
    f->deps[1] = dep2;
    f->ndeps = dep2 >= 0 ? 2 : (dep1 >= 0 ? 1 : 0);
    return t->nfields++;
}

fmd_handle_t fmd_turi_add(fmd_t *md, fmd_turi_t cat, int dimx, int dimy, int dimz, fmd_real_t starttime,
                          fmd_real_t stoptime)
{
    if (cat != FMD_TURI_CUSTOM && cat != FMD_TURI_TTM_TYPE1 && cat != FMD_TURI_TTM_TYPE2)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "turi category %d", (int)cat);
        return -1;
    }
    if (dimx < 1 || dimy < 1 || dimz < 1 || md->turies_num == MAX_TURIES)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "turi dimensions %dx%dx%d", dimx, dimy, dimz);
        return -1;
    }
    turi_t *arr = (turi_t *)realloc(md->turies, sizeof(turi_t) * (md->turies_num + 1));
    if (!arr) { FMD_ERR(md, FMD_ERR_UNABLE_ALLOCATE_MEM, false, "turi"); return -1; }
    md->turies = arr;
    turi_t *t = &arr[md->turies_num];
    memset(t, 0, sizeof *t);
    t->cat = cat;
    t->tdims_global[0] = dimx; t->tdims_global[1] = dimy; t->tdims_global[2] = dimz;
    t->starttime = starttime;
    t->stoptime = stoptime;
    const bool one_d = (dimx == 1 && dimy == 1);
    for (int d = 0; d < 3; d++)
    {
        if (cat == FMD_TURI_CUSTOM) t->itc_start[d] = 0;
        else t->itc_start[d] = (d == 2) ? 1 : (one_d ? 0 : 1);
        t->tcellh[d] = md->l[d] / t->tdims_global[d];
        t->itc_stop[d] = t->itc_start[d] + t->tdims_global[d];
        t->tdims_local[d] = t->itc_start[d] + t->itc_stop[d];
    }
    t->tcell_volume = t->tcellh[0] * t->tcellh[1] * t->tcellh[2];
    t->dev = -1;
    t->last_iter = -1;
    t->CellActivFrac = 0.1;
    if (cat != FMD_TURI_CUSTOM)
    {
        /* src/ttm.c:385-390 */
        field_add(md, t, FMD_FIELD_NUMBER);
        field_add(md, t, FMD_FIELD_VCM);
        field_add(md, t, FMD_FIELD_TEMPERATURE);
        t->iTe = field_add(md, t, FMD_FIELD_TTM_TE);
        t->ixi = field_add(md, t, FMD_FIELD_TTM_XI);
        t->is_ttm = 1;
    }
    const int h = md->turies_num++;
    if (cat != FMD_TURI_CUSTOM) md->active_ttm_turi = &md->turies[h];
    /* realloc may have moved the array */
    for (int i = 0; i < md->turies_num; i++)
        if (md->turies[i].is_ttm) md->active_ttm_turi = &md->turies[i];
    return h;
}

fmd_handle_t fmd_field_add(fmd_t *md, fmd_handle_t turi, fmd_field_t cat, fmd_real_t interval)
{
    (void)interval;   /* every field is updated every step (see the file comment) */
    turi_t *t = get_turi(md, turi);
    if (!t) return -1;
    if ((int)cat < FMD_FIELD_MASS || (int)cat > FMD_FIELD_TTM_XI)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "field category %d", (int)cat);
        return -1;
    }
    return field_add(md, t, cat);
}

fmd_handle_t fmd_field_find(fmd_t *md, fmd_handle_t turi, fmd_field_t cat)
{
    turi_t *t = get_turi(md, turi);
    if (!t) return -1;
    for (int i = 0; i < t->nfields; i++)
        if (t->fields[i].cat == cat) return i;
    return -1;
}

/* event sequence of one field update pass (src/turi.c:1509-1665) */
static void ev(fmd_t *md, int ti, int fi, bool *upd)
{
    upd[fi] = true;
    fmd_event_params_field_update_t p;
    p.turi = ti;
    p.field = fi;
    turi_t *t = &md->turies[ti];
    const bool te = t->is_ttm && fi == t->iTe;
    if (te) t->in_te_event = true;
    md->EventHandler(md, FMD_EVENT_FIELD_UPDATE, md->userobject, (fmd_params_t *)&p);
    if (te) md->turies[ti].in_te_event = false;
}

static void upd_vcm(fmd_t *md, int ti, turi_t *t, int fv, bool *upd)
{
    const int fm = t->fields[fv].deps[0];
    if (!upd[fm]) ev(md, ti, fm, upd);
    ev(md, ti, fv, upd);
}

static void upd_temperature(fmd_t *md, int ti, turi_t *t, int ft, bool *upd)
{
    const int fn = t->fields[ft].deps[0], fv = t->fields[ft].deps[1];
    if (!upd[fv]) upd_vcm(md, ti, t, fv, upd);
    if (!upd[fn]) ev(md, ti, fn, upd);
    ev(md, ti, ft, upd);
}

static void field_events(fmd_t *md, int ti, turi_t *t, bool with_ttm)
{
    bool upd[MAX_FIELDS] = {false};
    for (int fi = t->nfields - 1; fi >= 0; fi--)
    {
        if (upd[fi]) continue;
        hfield_t *f = &t->fields[fi];
        switch (f->cat)
        {
            case FMD_FIELD_TEMPERATURE: upd_temperature(md, ti, t, fi, upd); break;
            case FMD_FIELD_VCM: upd_vcm(md, ti, t, fi, upd); break;
            case FMD_FIELD_NUMBER_DENSITY:
                if (!upd[f->deps[0]]) ev(md, ti, f->deps[0], upd);
                ev(md, ti, fi, upd);
                break;
            case FMD_FIELD_NUMBER:
            case FMD_FIELD_MASS: ev(md, ti, fi, upd); break;
            case FMD_FIELD_TTM_TE:
            case FMD_FIELD_TTM_XI:
                if (!with_ttm) break;
                {
                    const int ft = f->deps[0];
                    if (!upd[ft]) upd_temperature(md, ti, t, ft, upd);
                    ev(md, ti, t->iTe, upd);
                    upd[t->ixi] = true;
                }
                break;
        }
    }
}

static bool within_window(const fmd_t *md, const turi_t *t)
{
    return (md->time >= t->starttime - md->timestep / 2.0) &&
           ((md->time < t->stoptime + md->timestep / 2.0) || t->stoptime < t->starttime);
}

/* Turies due for an update at the current iteration: inside their time
   window and not yet updated at this time_iteration (the reference marks
   every field with the iteration of its last update and skips marked
   fields, src/turi.c:1646). */
unsigned _fmdh_turies_due(fmd_t *md)
{
    unsigned mask = 0;
    for (int ti = 0; ti < md->turies_num; ti++)
        if (within_window(md, &md->turies[ti]) && md->turies[ti].last_iter != md->time_iteration)
            mask |= 1u << ti;
    return mask;
}

/* after the device updated the turies in `mask`: mark them and send the
   field-update events in the reference's order */
void _fmdh_turies_updated(fmd_t *md, unsigned mask, bool with_ttm)
{
    for (int ti = 0; ti < md->turies_num; ti++)
        if (mask & (1u << ti))
        {
            md->turies[ti].last_iter = md->time_iteration;
            if (md->EventHandler != NULL) field_events(md, ti, &md->turies[ti], with_ttm);
        }
}

void _fmdh_turies_update(fmd_t *md, bool xupd, bool vupd, bool fupd)
{
    (void)vupd;
    if (!xupd) return;   /* (F,F,T) after (T,T,F): every field is already updated */
    _fmdh_turies_updated(md, _fmdh_turies_due(md), !fupd);
}

/* ----------------------------------------------------------- device */

static bool upload_turies(fmd_t *md)
{
    for (int ti = 0; ti < md->turies_num; ti++)
    {
        turi_t *t = &md->turies[ti];
        if (t->dev >= 0) continue;
        int g2l[3] = {t->itc_start[0], t->itc_start[1], t->itc_start[2]};
        if (!_fmdh_dev_ok(md, fmdg_turi_add(md->dev, t->tdims_local, g2l, t->tcellh, t->starttime, t->stoptime,
                                            &t->dev), "fmdg_turi_add"))
            return false;
    }
    return true;
}

/* src/ttm.c:63-80 */
void _fmdh_ttm_get_ready(fmd_t *md)
{
    turi_t *t = md->active_ttm_turi;
    if (t == NULL) return;
    double ll[3], ul[3];
    fmd_matt_findLimits(md, md->ActiveGroup, ll, ul);
    t->frontsurf = ll[2];
    double vol = 1.0;
    for (int d = 0; d < 3; d++) vol *= ul[d] - ll[d];
    if (md->thermo_pending) _fmdh_thermo_from_device(md);
    t->initial_atoms_num = (unsigned)(md->GroupParticlesNum / vol * t->tcell_volume);
    t->min_atoms_num = (unsigned)(t->initial_atoms_num * t->CellActivFrac);
}

static bool upload_ttm(fmd_t *md, turi_t *t)
{
    if (t->tdims_global[0] != 1 || t->tdims_global[1] != 1)
    {
        /* the reference has no 3-D electron solver (src/ttm.c:458-461) */
        FMD_ERR(md, FMD_ERR_NOT_SUPPORTED_YET, true, "TTM turies must be 1x1xN (1-D along z)");
        return false;
    }
    fmdg_ttm_params_t p;
    memset(&p, 0, sizeof p);
    p.type = t->cat == FMD_TURI_TTM_TYPE1 ? 1 : 2;
    p.ratio = t->ratio;
    p.min_atoms = t->min_atoms_num;
    p.C_gamma = t->C_gamma;
    p.K = t->K;
    p.G = t->G;
    p.dz2 = t->tcellh[2] * t->tcellh[2];
    p.frontsurf = t->frontsurf;
    if (t->laser_set)
    {
        p.laser_t0 = t->laser_t0;
        p.laser_tdiff = t->laser_tdiff;
        p.laser_m_2sig2_inv = t->laser_m_2sig2_inv;
        p.laser_m_absdepth_inv = t->laser_m_absdepth_inv;
        p.laser_factor = t->laser_factor;
    }
    else
        p.laser_tdiff = -1.0;   /* |time - t0| < tdiff never holds: no source */
    p.Kzh_v2 = t->Kzh_v2; p.Kzh_A = t->Kzh_A; p.Kzh_B = t->Kzh_B;
    p.nC = t->nC; p.nG = t->nG;
    p.T_C = t->T_C; p.Ct = t->Ct; p.C_DD = t->C_DD;
    p.T_G = t->T_G; p.Gt = t->Gt; p.G_DD = t->G_DD;
    if (!_fmdh_dev_ok(md, fmdg_ttm_setup(md->dev, t->dev, t->itc_start[2], t->itc_stop[2], &p), "fmdg_ttm_setup"))
        return false;
    if (t->Te_set)
    {
        const int nz = t->tdims_local[2];
        double *Te = (double *)malloc(sizeof(double) * nz);
        for (int i = 0; i < nz; i++) Te[i] = (i >= t->itc_start[2] && i < t->itc_stop[2]) ? t->Te_init : -1.0;
        const int rc = fmdg_ttm_set_te(md->dev, t->dev, Te);
        free(Te);
        t->Te_set = false;
        if (!_fmdh_dev_ok(md, rc, "fmdg_ttm_set_te")) return false;
    }
    return true;
}

/* symplectic Euler with TTM coupling (src/integrators.c:181-225) */
void _fmdh_se_integrate(fmd_t *md, double duration)
{
    const double start = md->time;
    const double dt = md->timestep;
    if (!upload_turies(md)) return;
    _fmdh_ttm_get_ready(md);
    if (md->active_ttm_turi && !upload_ttm(md, md->active_ttm_turi)) return;
    if (!_fmdh_dev_ok(md, fmdg_set_time(md->dev, md->time, dt), "fmdg_set_time")) return;
    const unsigned due = _fmdh_turies_due(md);
    if (due && !_fmdh_dev_ok(md, fmdg_turi_update(md->dev, dt, due), "fmdg_turi_update")) return;
    _fmdh_turies_updated(md, due, true);
    if (!_fmdh_dev_ok(md, fmdg_compute_forces(md->dev, md->ActiveGroup), "fmdg_compute_forces")) return;
    md->thermo_pending = true;
    md->KineticEnergyUpdated = true;
    _fmdh_check_device_errors(md);
    if (md->EventHandler != NULL) _fmdh_send_timer_events(md);
    while (md->time < start + duration)
    {
        int k = 0;
        double t = md->time;
        do
        {
            k++;
            t += dt;
        } while (k < (1 << 20) && t < start + duration && md->EventHandler == NULL);
        if (!_fmdh_dev_ok(md, fmdg_se_steps(md->dev, k, dt, md->ActiveGroup), "fmdg_se_steps")) return;
        for (int s = 0; s < k; s++)
        {
            md->time += dt;
            md->time_iteration++;
        }
        md->thermo_pending = true;
        md->KineticEnergyUpdated = true;
        _fmdh_turies_update(md, true, true, false);
        _fmdh_check_device_errors(md);
        if (md->EventHandler != NULL) _fmdh_send_timer_events(md);
    }
}

bool _fmdh_prepare_turies(fmd_t *md) { return upload_turies(md); }

/* ------------------------------------------------------------ arrays */

static fmd_array3s_t *array3_new(const int dims[3], size_t elsize)
{
    fmd_array3s_t *a = (fmd_array3s_t *)calloc(1, sizeof *a);
    if (!a) return NULL;
    const size_t n0 = dims[0], n1 = dims[1], n2 = dims[2];
    /* one block: row pointers, then plane pointers, then the elements */
    const size_t bytes = n0 * sizeof(void **) + n0 * n1 * sizeof(void *) + n0 * n1 * n2 * elsize + 64;
    char *blk = (char *)calloc(1, bytes);
    if (!blk) { free(a); return NULL; }
    void ***p0 = (void ***)blk;
    void **p1 = (void **)(blk + n0 * sizeof(void **));
    char *el = blk + n0 * sizeof(void **) + n0 * n1 * sizeof(void *);
    el = (char *)(((uintptr_t)el + 15) & ~(uintptr_t)15);
    for (size_t i = 0; i < n0; i++)
    {
        p0[i] = p1 + i * n1;
        for (size_t j = 0; j < n1; j++) p1[i * n1 + j] = el + ((i * n1 + j) * n2) * elsize;
    }
    a->data = p0;
    for (int d = 0; d < 3; d++) a->dims[d] = (unsigned)dims[d];
    a->elsize = elsize;
    return a;
}

void fmd_array3s_free(fmd_array3s_t *array)
{
    if (array == NULL) return;
    free(array->data);
    free(array);
}

fmd_array3s_t *fmd_field_getArray(fmd_t *md, fmd_handle_t turi, fmd_handle_t field, fmd_array3_t *array,
                                  fmd_utriple_t dims)
{
    turi_t *t = get_turi(md, turi);
    if (!t) return NULL;
    if (field < 0 || field >= t->nfields)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "field handle %d", field);
        return NULL;
    }
    if (t->dev < 0 || md->dev == NULL)
    {
        FMD_ERR(md, FMD_ERR_UNPREPARED, false, "turi fields exist only after the first run");
        return NULL;
    }
    const fmd_field_t cat = t->fields[field].cat;
    if (cat == FMD_FIELD_TTM_XI)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "field category %d", (int)cat);
        return NULL;
    }
    const int nl = t->tdims_local[0] * t->tdims_local[1] * t->tdims_local[2];
    unsigned *num = (unsigned *)malloc(sizeof(unsigned) * nl);
    double *mass = (double *)malloc(sizeof(double) * nl);
    double *vcm = (double *)malloc(sizeof(double) * 3 * nl);
    double *Ti = (double *)malloc(sizeof(double) * nl);
    double *Te = (double *)malloc(sizeof(double) * (t->tdims_local[2] + 1));
    int rc = fmdg_turi_download(md->dev, t->dev, num, mass, vcm, Ti, NULL, NULL);
    if (rc == FMDG_OK && t->is_ttm) rc = fmdg_ttm_download_te(md->dev, t->dev, t->in_te_event ? 1 : 0, Te);
    if (!_fmdh_dev_ok(md, rc, "fmdg_turi_download"))
    {
        free(num); free(mass); free(vcm); free(Ti); free(Te);
        return NULL;
    }
    const size_t elsize = cat == FMD_FIELD_VCM ? 3 * sizeof(double)
                        : (cat == FMD_FIELD_NUMBER ? sizeof(unsigned) : sizeof(double));
    fmd_array3s_t *a = array3_new(t->tdims_global, elsize);
    if (a)
    {
        for (int i = 0; i < t->tdims_global[0]; i++)
            for (int j = 0; j < t->tdims_global[1]; j++)
                for (int k = 0; k < t->tdims_global[2]; k++)
                {
                    const int li = i + t->itc_start[0], lj = j + t->itc_start[1], lk = k + t->itc_start[2];
                    const int c = lk + t->tdims_local[2] * (lj + t->tdims_local[1] * li);
                    void *dst = (char *)a->data[i][j] + (size_t)k * elsize;
                    switch (cat)
                    {
                        case FMD_FIELD_NUMBER: *(unsigned *)dst = num[c]; break;
                        case FMD_FIELD_MASS: *(double *)dst = mass[c] * FMD_MASS_UNIT; break;
                        case FMD_FIELD_VCM: memcpy(dst, vcm + 3 * c, 3 * sizeof(double)); break;
                        case FMD_FIELD_TEMPERATURE: *(double *)dst = Ti[c]; break;
                        case FMD_FIELD_NUMBER_DENSITY: *(double *)dst = num[c] / t->tcell_volume; break;
                        case FMD_FIELD_TTM_TE: *(double *)dst = Te[lk]; break;
                        default: break;
                    }
                }
        *array = a->data;
        for (int d = 0; d < 3; d++) dims[d] = a->dims[d];
    }
    free(num); free(mass); free(vcm); free(Ti); free(Te);
    return a;
}

void fmd_field_save_as_hdf5(fmd_t *md, fmd_handle_t turi, fmd_handle_t field, fmd_string_t filename)
{
    (void)turi; (void)field; (void)filename;
    FMD_ERR(md, FMD_ERR_NOT_SUPPORTED_YET, false, "HDF5 output is not available in this build");
}

void _fmdh_turies_free(fmd_t *md)
{
    for (int i = 0; i < md->turies_num; i++)
    {
        turi_t *t = &md->turies[i];
        free(t->T_C); free(t->Ct); free(t->C_DD); free(t->T_G); free(t->Gt); free(t->G_DD);
    }
    free(md->turies);
    md->turies = NULL;
    md->turies_num = 0;
    md->active_ttm_turi = NULL;
}

/* -------------------------------------------------------- TTM setters */

static turi_t *ttm_of(fmd_t *md, fmd_handle_t h, int need_type)
{
    turi_t *t = get_turi(md, h);
    if (!t) return NULL;
    const bool ok = need_type == 0 ? (t->cat == FMD_TURI_TTM_TYPE1 || t->cat == FMD_TURI_TTM_TYPE2)
                                   : (int)t->cat == need_type;
    if (!ok)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "turi category %d", (int)t->cat);
        return NULL;
    }
    return t;   /* parameters take effect at the next run */
}

void _fmd_ttm_setHeatCapacity_linear(fmd_t *md, fmd_handle_t turi, fmd_ttm_heat_capacity_linear_t c)
{
    turi_t *t = ttm_of(md, turi, FMD_TURI_TTM_TYPE1);
    if (t) t->C_gamma = c.gamma * FMD_J_M3_K2;
}

/* two-column table file: T [1e4 K], value [scale] (src/ttm.c:549-606) */
static int read_table(fmd_t *md, const char *path, double tscale, double vscale, double **T, double **V, double **DD)
{
    FILE *fp = fopen(path, "r");
    if (!fp) { FMD_ERR(md, FMD_ERR_UNABLE_OPEN_FILE, false, "%s", path); return -1; }
    int n = 0, cap = 0;
    double *tt = NULL, *vv = NULL, a, b;
    while (fscanf(fp, "%lf%lf", &a, &b) == 2)
    {
        if (n == cap)
        {
            cap += 100;
            tt = (double *)realloc(tt, sizeof(double) * cap);
            vv = (double *)realloc(vv, sizeof(double) * cap);
        }
        tt[n] = a * tscale;
        vv[n] = b * vscale;
        n++;
    }
    fclose(fp);
    if (n < 2)
    {
        FMD_ERR(md, FMD_ERR_FILE_CORRUPTED, false, "table %s", path);
        free(tt); free(vv);
        return -1;
    }
    double *dd = (double *)malloc(sizeof(double) * n);
    _fmdh_spline_prepare_adv(tt, vv, n, dd);
    free(*T); free(*V); free(*DD);
    *T = tt; *V = vv; *DD = dd;
    return n;
}

void _fmd_ttm_setHeatCapacity_file(fmd_t *md, fmd_handle_t turi, fmd_string_t path)
{
    turi_t *t = ttm_of(md, turi, FMD_TURI_TTM_TYPE2);
    if (!t) return;
    const int n = read_table(md, path, 1e4, 1e5 * FMD_J_M3_K, &t->T_C, &t->Ct, &t->C_DD);
    if (n > 0) t->nC = n;
}

void _fmd_ttm_setHeatConductivity_constant1(fmd_t *md, fmd_handle_t turi, fmd_real_t k)
{
    turi_t *t = ttm_of(md, turi, FMD_TURI_TTM_TYPE1);
    if (t) t->K = k * FMD_W_M_K;
}

void _fmd_ttm_setHeatConductivity_constant2(fmd_t *md, fmd_handle_t turi, fmd_ttm_heat_conductivity_constant_t k)
{
    _fmd_ttm_setHeatConductivity_constant1(md, turi, k.value);
}

void _fmd_ttm_setHeatConductivity_zhigilei(fmd_t *md, fmd_handle_t turi, fmd_ttm_heat_conductivity_zhigilei_t k)
{
    turi_t *t = ttm_of(md, turi, FMD_TURI_TTM_TYPE2);
    if (!t) return;
    t->Kzh_A = k.A / FMD_SECOND;
    t->Kzh_B = k.B / FMD_SECOND;
    const double v = k.v * 1e-2;   /* m/s -> A/ps */
    t->Kzh_v2 = v * v;
}

void _fmd_ttm_setCouplingFactor_constant1(fmd_t *md, fmd_handle_t turi, fmd_real_t g)
{
    turi_t *t = ttm_of(md, turi, FMD_TURI_TTM_TYPE1);
    if (t) t->G = g * FMD_W_M3_K;
}

void _fmd_ttm_setCouplingFactor_constant2(fmd_t *md, fmd_handle_t turi, fmd_ttm_coupling_factor_constant_t g)
{
    _fmd_ttm_setCouplingFactor_constant1(md, turi, g.value);
}

void _fmd_ttm_setCouplingFactor_file(fmd_t *md, fmd_handle_t turi, fmd_string_t path)
{
    turi_t *t = ttm_of(md, turi, FMD_TURI_TTM_TYPE2);
    if (!t) return;
    const int n = read_table(md, path, 1e4, 1e17 * FMD_W_M3_K, &t->T_G, &t->Gt, &t->G_DD);
    if (n > 0) t->nG = n;
}

void fmd_ttm_setElectronTemperature(fmd_t *md, fmd_handle_t turi, fmd_real_t Te)
{
    turi_t *t = ttm_of(md, turi, 0);
    if (!t) return;
    t->Te_init = Te;
    t->Te_set = true;
    if (t->dev >= 0 && md->dev)
    {
        const int nz = t->tdims_local[2];
        double *arr = (double *)malloc(sizeof(double) * nz);
        for (int i = 0; i < nz; i++) arr[i] = (i >= t->itc_start[2] && i < t->itc_stop[2]) ? Te : -1.0;
        if (fmdg_ttm_set_te(md->dev, t->dev, arr) == FMDG_OK) t->Te_set = false;
        free(arr);
    }
}

void fmd_ttm_setTimestepRatio(fmd_t *md, fmd_handle_t turi, int ratio)
{
    turi_t *t = ttm_of(md, turi, 0);
    if (t) t->ratio = ratio;
}

void fmd_ttm_setCellActivationFraction(fmd_t *md, fmd_handle_t turi, fmd_real_t value)
{
    turi_t *t = ttm_of(md, turi, 0);
    if (!t) return;
    if (value < 0 || value > 1)
    {
        FMD_ERR(md, FMD_ERR_OUTSIDE_REAL_INTERVAL, false, "cell activation fraction %g outside [0 1]", value);
        return;
    }
    t->CellActivFrac = value;
}

/* Gaussian pulse with exponential absorption (src/ttm.c:794-816) */
void _fmd_ttm_setLaserSource_gaussian(fmd_t *md, fmd_handle_t turi, fmd_ttm_laser_gaussian_t laser)
{
    turi_t *t = ttm_of(md, turi, 0);
    if (!t) return;
    const double Lp = laser.AbsorptionDepth * FMD_METER;
    const double R = laser.reflectance;
    const double I0 = sqrt(4 * log(2) / M_PI) * laser.fluence / laser.duration * FMD_W_M2;
    const double sigma = laser.duration / sqrt(8 * log(2)) * FMD_SECOND;
    t->laser_t0 = laser.t0 * FMD_SECOND;
    t->laser_tdiff = 4 * sqrt(2) * sigma;
    t->laser_m_2sig2_inv = -0.5 / (sigma * sigma);
    t->laser_m_absdepth_inv = -1. / Lp;
    t->laser_factor = I0 * (1 - R) / Lp;
    t->laser_set = true;
}

/* white-box access to the derived parameters of the active 1-D TTM turi,
   in the layout the golden files record for the reference (d: C_gamma, K,
   G, dz2, frontsurf, laser_t0, laser_tdiff, laser_m_2sig2_inv,
   laser_m_absdepth_inv, laser_factor, Kzh v2, A, B, tcell_volume,
   starttime, stoptime, tcellh_z; k: type, ratio, min_atoms, nC, nG,
   itc_start_z, itc_stop_z, nz, glob-to-loc offset z); the type-2 tables
   through `tables` (T_C, Ct, C_DD, T_G, Gt, G_DD pointers, may be NULL).
   For the CPU oracle's TTM runs (tests, the bench's CPU baseline).
   Returns -1 without a TTM turi. */
int fmdx_ttm_params(fmd_t *md, double *d, int *k, const double **tables)
{
    turi_t *t = md->active_ttm_turi;
    if (t == NULL) return -1;
    const double dv[17] = {t->C_gamma, t->K, t->G, t->tcellh[2] * t->tcellh[2], t->frontsurf, t->laser_t0,
                           t->laser_set ? t->laser_tdiff : -1.0, t->laser_m_2sig2_inv, t->laser_m_absdepth_inv,
                           t->laser_factor, t->Kzh_v2, t->Kzh_A, t->Kzh_B, t->tcell_volume, t->starttime,
                           t->stoptime, t->tcellh[2]};
    const int kv[9] = {t->cat == FMD_TURI_TTM_TYPE1 ? 1 : 2, t->ratio, (int)t->min_atoms_num, t->nC, t->nG,
                       t->itc_start[2], t->itc_stop[2], t->tdims_local[2], t->itc_start[2]};
    memcpy(d, dv, sizeof dv);
    memcpy(k, kv, sizeof kv);
    if (tables)
    {
        tables[0] = t->T_C; tables[1] = t->Ct; tables[2] = t->C_DD;
        tables[3] = t->T_G; tables[4] = t->Gt; tables[5] = t->G_DD;
    }
    return 0;
}

/* white-box access to the 1-D TTM arrays of the active TTM turi (local
   cells incl. margins), for parity tests; returns the local length */
int fmdx_ttm_1d(fmd_t *md, unsigned *num, double *vcm, double *Ti, double *Te, double *xi)
{
    turi_t *t = md->active_ttm_turi;
    if (t == NULL || t->dev < 0 || md->dev == NULL) return -1;
    const int nz = t->tdims_local[2];
    if (fmdg_turi_download(md->dev, t->dev, num, NULL, vcm, Ti, Te, xi)) return -1;
    return nz;
}
