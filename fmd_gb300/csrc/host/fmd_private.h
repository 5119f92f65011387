/*
 * Private state of one FMD instance on the host side of libfmd.so.
 *
 * The host keeps what the reference keeps on the host for set-up (box,
 * atom kinds, potentials, timers, the pre-distribution "global grid" of
 * atoms) and hands the per-timestep work to the device engine (fmdg.h).
 * Before the first integrate/equilibrate the atoms live in host cells, in
 * insertion order per cell, exactly as the reference's global grid
 * (src/misc.c:41-62, src/structure.c:53-136, src/misc.c:121-266); the first
 * run uploads them in cell order (the single-rank distribution of
 * src/matter.c:329-447) and from then on the device copy is authoritative.
 */
#ifndef FMD_PRIVATE_H
#define FMD_PRIVATE_H

#include <stdarg.h>
#include <stdbool.h>
#include <stdio.h>
#include "fmd.h"
#include "fmdg.h"

#define FMD_MASS_UNIT        9.6485332907e+03   /* Da per internal mass unit */
#define FMD_K_BOLTZMANN      8.6173303e-5       /* eV / K */
#define FMD_METER            1e10
#define FMD_SECOND           1e12
#define FMD_J_M3_K           6.2415091259e-12   /* J/(m^3 K)   -> eV/(A^3 K)   */
#define FMD_J_M3_K2          6.2415091259e-12   /* J/(m^3 K^2) -> eV/(A^3 K^2) */
#define FMD_W_M_K            6.2415091259e-4    /* W/(m K)     -> eV/(ps A K)  */
#define FMD_W_M2             6.2415091259e-14   /* W/m^2       -> eV/(ps A^2)  */
#define FMD_W_M3_K           6.2415091259e-24   /* W/(m^3 K)   -> eV/(ps A^3 K) */
#define FMD_MAX_KINDS        8
#define FMD_MAX_PATH         256
#define FMD_RESERVED_GROUP   (-2)

typedef enum { POTCAT_NONE = 0, POTCAT_LJ = 1, POTCAT_EAM = 2, POTCAT_MORSE = 3 } potcat_t;

typedef struct
{
    char name[64];
    double mass, lattice;
    double *F, *F_DD;         /* Nrho */
    double *rho, *rhoDD;      /* Nr2 (r^2 grid) */
} eam_element_t;

typedef struct
{
    int nelem;
    int Nrho, Nr, Nr2;
    double drho, dr, dr2, cutoff_sqr;
    eam_element_t *el;
    double **phi, **phiDD;    /* nelem*nelem, symmetric (shared pointers) */
} eam_t;

typedef struct { double eps, eps4, sig, sig_sqr, cutoff_sqr; } lj_t;
typedef struct { double D0, alpha, r0, cutoff_sqr; } morse_t;

struct _fmd_pot
{
    potcat_t cat;
    void *data;
    struct _fmd_pot *next;    /* list of every loaded/created potential */
};

typedef struct
{
    potcat_t cat;
    fmd_pot_t *pot;
    int iloc, jloc;
} potpair_t;

typedef struct
{
    char name[64];
    double mass;              /* internal units */
    int eam_elem;             /* index in the applied EAM, or -1 */
} atomkind_t;

/* pre-distribution cell (insertion order) */
typedef struct
{
    int n, cap;
    double *x, *v;
    int *group;
    unsigned *kind, *id;
} hcell_t;

typedef struct
{
    bool enabled;
    double start, interval, stop;
} fmd_timer_t;

typedef struct turi turi_t;   /* fmd_turi.c */

struct _fmd
{
    /* box */
    double l[3];
    int PBC[3];
    bool BoxSizeDetermined, PBCdetermined;
    int ns[3];
    int nc[3];
    double cellh[3];
    /* kinds & potentials */
    unsigned nkinds;
    atomkind_t kinds[FMD_MAX_KINDS];
    potpair_t pottable[FMD_MAX_KINDS][FMD_MAX_KINDS];
    bool pottable_made;
    fmd_pot_t *potlist;
    eam_t *applied_eam;
    /* atoms before distribution */
    hcell_t *ggrid;
    unsigned TotalNoOfParticles;
    bool ParticlesDistributed;
    /* device */
    fmdg_sys_t *dev;
    bool dev_tables_ok;
    int precision;
    /* dynamics */
    double time, timestep;
    int time_iteration;
    int ActiveGroup;
    double DesiredTemperature, BerendsenThermostatParam;
    bool KineticEnergyUpdated;
    double GroupTemperature, GroupKineticEnergy, GroupPotentialEnergy;
    double GroupVirial;    /* pair virial of the last force evaluation (no reference counterpart) */
    double GroupMomentum[3];
    unsigned GroupParticlesNum;
    bool thermo_pending;      /* device thermo record newer than the cache */
    /* events */
    fmd_EventHandler_t EventHandler;
    void *userobject;
    fmd_timer_t *timers;
    int timers_num;
    /* turies (continuum grids) */
    turi_t *turies;
    int turies_num;
    turi_t *active_ttm_turi;
    /* io */
    char *SaveDirectory;
    fmd_SaveConfigMode_t SaveConfigMode;
    FILE *ConfigFilep;
    int OldNumberOfParticles, FileIndex;
    bool ShowErrorMessages;
    double WallTimeOrigin;
    int cell_increment;
    int numthreads;
    unsigned long long seed;
    bool seed_fixed;
    unsigned long long rng_calls;
};

/* fmd_core.c */
void _fmdh_error(fmd_t *md, fmd_error_t err, bool major, const char *file, const char *func, int line,
                 const char *fmt, ...);
#define FMD_ERR(md, code, major, ...) _fmdh_error((md), (code), (major), __FILE__, __func__, __LINE__, __VA_ARGS__)
double _fmdh_walltime(void);
bool _fmdh_dev_ok(fmd_t *md, int rc, const char *what);

/* fmd_pot.c */
double _fmdh_largest_cutoff(fmd_t *md);
bool _fmdh_pots_ready(fmd_t *md);
int _fmdh_upload_tables(fmd_t *md);
void _fmdh_eam_flatten(const eam_t *e, double *F, double *FDD, double *rho, double *rhoDD, double *phi,
                       double *phiDD);
void _fmdh_pots_free(fmd_t *md);
void _fmdh_spline_prepare(double h, const double *y, int n, double *yDD);
void _fmdh_spline_prepare_adv(const double *x, const double *y, int n, double *yDD);

/* fmd_matter.c */
void _fmdh_create_global_grid(fmd_t *md);
void _fmdh_ggrid_free(fmd_t *md);
bool _fmdh_distribute(fmd_t *md);
void _fmdh_thermo_refresh(fmd_t *md);
void _fmdh_thermo_from_device(fmd_t *md);
int _fmdh_current_atoms(fmd_t *md, int *n, double **x, double **v, unsigned **kind, int **group, unsigned **id);

/* fmd_turi.c */
void _fmdh_turies_free(fmd_t *md);
void _fmdh_turies_update(fmd_t *md, bool xupd, bool vupd, bool fupd);
void _fmdh_ttm_get_ready(fmd_t *md);
void _fmdh_se_integrate(fmd_t *md, double duration);
bool _fmdh_prepare_turies(fmd_t *md);
unsigned _fmdh_turies_due(fmd_t *md);
void _fmdh_turies_updated(fmd_t *md, unsigned mask, bool with_ttm);

/* fmd_dync.c */
void _fmdh_send_timer_events(fmd_t *md);
void _fmdh_check_device_errors(fmd_t *md);

/* rng (fmd_matter.c) */
double _fmdh_rng_uniform(fmd_t *md, unsigned long long *state);
double _fmdh_rng_gauss(fmd_t *md, unsigned long long *state, double sigma);
unsigned long long _fmdh_rng_seed(fmd_t *md);

#endif
