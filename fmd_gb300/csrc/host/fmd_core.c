/*
 * Instance lifetime, box, process, i/o settings, errors, timers, version.
 * Follows the reference's single-process behaviour: src/misc.c:84-119,
 * 432-450, 499-617; src/timer.c:27-84; src/error.c:20-236; src/version.c.
 */
#define _POSIX_C_SOURCE 200809L
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "fmd_private.h"

#define FMD_VERSION_MAJOR 0
#define FMD_VERSION_MINOR 4
#define FMD_VERSION_REVISION 0
#define FMD_VERSION_TYPE 'g'

double _fmdh_walltime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static const char *error_text(fmd_error_t e)
{
    switch (e)
    {
        case FMD_ERR_UNEXPECTED_POSITION: return "unexpected position";
        case FMD_ERR_UNABLE_OPEN_FILE: return "unable to open file";
        case FMD_ERR_UNABLE_ALLOCATE_MEM: return "unable to allocate memory";
        case FMD_ERR_FILE_CORRUPTED: return "file corrupted";
        case FMD_ERR_OUTSIDE_REAL_INTERVAL: return "value outside the allowed interval";
        case FMD_ERR_UNACCEPTABLE_INT_VALUE: return "unacceptable integer value";
        case FMD_ERR_UNSUCCESSFUL_HDF5: return "unsuccessful HDF5 operation";
        case FMD_ERR_FUNCTION_FAILED: return "function failed";
        case FMD_ERR_NOT_SUPPORTED_YET: return "not supported";
        case FMD_ERR_UNPREPARED: return "unprepared";
        case FMD_ERR_WRONG_POTENTIAL: return "wrong potential";
    }
    return "error";
}

/* Error reporting convention of the reference (src/error.c): optional
   message on stderr, then FMD_EVENT_ERROR to the handler; never aborts. */
void _fmdh_error(fmd_t *md, fmd_error_t err, bool major, const char *file, const char *func, int line,
                 const char *fmt, ...)
{
    char msg[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof msg, fmt, ap);
    va_end(ap);
    if (md == NULL || md->ShowErrorMessages)
        fprintf(stderr, "FMD %s ERROR (%s, %s:%d in %s): %s\n", major ? "MAJOR" : "MINOR",
                error_text(err), file, line, func, msg);
    if (md != NULL && md->EventHandler != NULL)
    {
        fmd_event_params_error_t p;
        p.error = err;
        p.major = major;
        p.source = (fmd_string_t)file;
        p.func = (fmd_string_t)func;
        p.line = line;
        p.p1 = p.p2 = p.p3 = NULL;
        md->EventHandler(md, FMD_EVENT_ERROR, md->userobject, (fmd_params_t *)&p);
    }
}

bool _fmdh_dev_ok(fmd_t *md, int rc, const char *what)
{
    if (rc == FMDG_OK) return true;
    _fmdh_error(md, rc == FMDG_E_NOMEM ? FMD_ERR_UNABLE_ALLOCATE_MEM : FMD_ERR_FUNCTION_FAILED, true,
                __FILE__, what, __LINE__, "device engine: %s", fmdg_last_error());
    return false;
}

fmd_t *fmd_create()
{
    fmd_t *md = (fmd_t *)calloc(1, sizeof(fmd_t));
    if (md == NULL) return NULL;
    md->ns[0] = md->ns[1] = md->ns[2] = 1;
    md->ActiveGroup = FMD_GROUP_ALL;
    md->SaveDirectory = (char *)calloc(1, 1);
    md->SaveConfigMode = FMD_SCM_XYZ_ATOMSNUM;
    md->OldNumberOfParticles = -1;
    md->ShowErrorMessages = true;
    md->cell_increment = 3;
    md->numthreads = 1;
    md->precision = FMDG_PREC_FP64;
    const char *p = getenv("FMD_PRECISION");
    if (p && (strcmp(p, "mixed") == 0 || strcmp(p, "1") == 0)) md->precision = FMDG_PREC_MIXED;
    md->seed = _fmdh_rng_seed(md);
    md->WallTimeOrigin = _fmdh_walltime();
    return md;
}

void fmd_free(fmd_t *md)
{
    if (md == NULL) return;
    if (md->ConfigFilep != NULL && md->OldNumberOfParticles != -1) fclose(md->ConfigFilep);
    _fmdh_turies_free(md);
    _fmdh_ggrid_free(md);
    _fmdh_pots_free(md);
    if (md->dev) fmdg_destroy(md->dev);
    free(md->timers);
    free(md->SaveDirectory);
    free(md);
}

void fmd_setEventHandler(fmd_t *md, void *usp, fmd_EventHandler_t func)
{
    md->EventHandler = func;
    md->userobject = usp;
}

void fmd_box_setPBC(fmd_t *md, bool PBCx, bool PBCy, bool PBCz)
{
    md->PBC[0] = PBCx;
    md->PBC[1] = PBCy;
    md->PBC[2] = PBCz;
    md->PBCdetermined = true;
}

void fmd_box_setSize(fmd_t *md, fmd_real_t sx, fmd_real_t sy, fmd_real_t sz)
{
    if (md->ggrid != NULL || md->ParticlesDistributed) return;   /* as src/misc.c:561-570 */
    md->l[0] = sx;
    md->l[1] = sy;
    md->l[2] = sz;
    md->BoxSizeDetermined = true;
}

/* One GPU holds the whole box: only a single subdomain exists. */
bool fmd_box_setSubdomains(fmd_t *md, int dimx, int dimy, int dimz)
{
    if (dimx * dimy * dimz != 1)
    {
        FMD_ERR(md, FMD_ERR_NOT_SUPPORTED_YET, false,
                "the box is simulated on one GPU; subdomain grid %dx%dx%d replaced by 1x1x1", dimx, dimy, dimz);
    }
    md->ns[0] = md->ns[1] = md->ns[2] = 1;
    return true;
}

fmd_real_t fmd_proc_getWallTime(fmd_t *md) { return _fmdh_walltime() - md->WallTimeOrigin; }
bool fmd_proc_hasSubdomain(fmd_t *md) { (void)md; return true; }
bool fmd_proc_isRoot(fmd_t *md) { (void)md; return true; }
void fmd_proc_setNumThreads(fmd_t *md, int num) { md->numthreads = num; }
int fmd_proc_getCellIncrement(fmd_t *md) { return md->cell_increment; }

void fmd_proc_setCellIncrement(fmd_t *md, int incr)
{
    if (incr <= 0)
    {
        FMD_ERR(md, FMD_ERR_UNACCEPTABLE_INT_VALUE, false, "cell increment value %d", incr);
        return;
    }
    md->cell_increment = incr;   /* host cells grow geometrically; kept for the API */
}

void fmd_io_setSaveDirectory(fmd_t *md, fmd_string_t directory)
{
    char *p = (char *)realloc(md->SaveDirectory, strlen(directory) + 1);
    if (p == NULL) { FMD_ERR(md, FMD_ERR_UNABLE_ALLOCATE_MEM, false, "save directory"); return; }
    strcpy(p, directory);
    md->SaveDirectory = p;
}

void fmd_io_setSaveConfigMode(fmd_t *md, fmd_SaveConfigMode_t mode) { md->SaveConfigMode = mode; }
void fmd_io_setShowErrorMessages(fmd_t *md, bool show) { md->ShowErrorMessages = show; }

void fmd_io_printf(fmd_t *md, const fmd_string_t restrict format, ...)
{
    (void)md;
    va_list ap;
    va_start(ap, format);
    vprintf(format, ap);
    va_end(ap);
}

/* ---- timers (src/timer.c:27-84) ---- */

fmd_handle_t fmd_timer_makeSimple(fmd_t *md, fmd_real_t start, fmd_real_t interval, fmd_real_t stop)
{
    fmd_timer_t *t = (fmd_timer_t *)realloc(md->timers, (md->timers_num + 1) * sizeof(fmd_timer_t));
    if (t == NULL) { FMD_ERR(md, FMD_ERR_UNABLE_ALLOCATE_MEM, false, "timer"); return -1; }
    md->timers = t;
    t[md->timers_num].enabled = true;
    t[md->timers_num].start = start;
    t[md->timers_num].interval = interval;
    t[md->timers_num].stop = stop;
    return md->timers_num++;
}

/* ---- version ---- */

int fmd_version_getMajor() { return FMD_VERSION_MAJOR; }
int fmd_version_getMinor() { return FMD_VERSION_MINOR; }
int fmd_version_getRevision() { return FMD_VERSION_REVISION; }
char fmd_version_getType() { return FMD_VERSION_TYPE; }

fmd_string_t fmd_version_getString()
{
    char *s = (char *)malloc(32);
    if (s) snprintf(s, 32, "%d.%d.%d%c", FMD_VERSION_MAJOR, FMD_VERSION_MINOR, FMD_VERSION_REVISION,
                    FMD_VERSION_TYPE);
    return s;
}
