/*
 * CPU restatement of FMD 0.4.0's per-timestep hot path -- TEST
 * INFRASTRUCTURE ONLY.  Used by tests/ as the restatement the GPU engine is
 * compared with, by __graft_entry__.smoke(), and by bench.py as the timed
 * CPU baseline.
 * Nothing in the product (libfmd.so) links or calls it.
 *
 * It follows the reference's algorithms (file:line in fmd_oracle.c) with the
 * same binary64 arithmetic: per-cell atom lists with swap-remove refresh and
 * periodic migration, half-shell cell-pair loops with Newton's third law,
 * LJ / Morse / EAM (r^2-grid cubic splines) / hybrid pair updates, velocity
 * Verlet with Berendsen scaling, group thermodynamics, and the 1-D
 * two-temperature model (turi fields, electron solver types 1 and 2,
 * friction term, symplectic Euler).  Ghost cells are
 * represented by image shifts of the interior cells.  Parity pins: the
 * golden vectors in tests/golden/ were produced by the reference compiled
 * from its own sources; tests/test_oracle_cpu.py checks this restatement
 * against them.
 *
 * The interface mirrors include/fmdg.h so tests drive both identically.
 */
#ifndef FMD_ORACLE_H
#define FMD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_sys oracle_sys_t;

typedef struct
{
    int cat;           /* 1 LJ, 2 EAM, 3 Morse */
    int iloc, jloc;
    int pad;
    double p[4];       /* as fmdg_pair_t */
} oracle_pair_t;

typedef struct
{
    /* virial: pair virial sum over pairs r_ij . F_ij of the last force
       evaluation (pressure P V = N k T + virial / 3) */
    double kinetic, temperature, momentum[3], potential, count, virial;
} oracle_thermo_t;

oracle_sys_t *oracle_create(void);
void oracle_destroy(oracle_sys_t *o);
int oracle_set_threads(oracle_sys_t *o, int nthreads);
int oracle_set_box(oracle_sys_t *o, const double l[3], const int pbc[3], const int nc[3], const double cellh[3]);
int oracle_set_kinds(oracle_sys_t *o, int nkinds, const double *mass, const int *eam_elem);
int oracle_set_pairs(oracle_sys_t *o, const oracle_pair_t *table);
/* EAM tables: either given directly (same layout as fmdg_set_eam) ... */
int oracle_set_eam(oracle_sys_t *o, int nelem, int Nrho, double drho, int Nr2, double dr2,
                   const double *F, const double *F_DD, const double *rho, const double *rhoDD,
                   const double *phi, const double *phiDD);
/* ... or read from a DYNAMO setfl file (src/eam.c:376-555); returns the
   number of elements and writes the element names (space separated) */
int oracle_load_setfl(oracle_sys_t *o, const char *path, char *names, int names_len, double *cutoff);
/* the r^2-grid tables of element `el` after oracle_load_setfl */
int oracle_eam_table(oracle_sys_t *o, int el, int which, double *out, int *n);

int oracle_upload(oracle_sys_t *o, int n, const int *cell_count, const double *x, const double *v,
                  const unsigned *kind, const int *group, const unsigned *atomid);
int oracle_natoms(oracle_sys_t *o);
int oracle_download(oracle_sys_t *o, int *cell_of, double *x, double *v, double *F, double *vaream,
                    unsigned *kind, int *group, unsigned *atomid);
int oracle_set_state(oracle_sys_t *o, const double *x, const double *v);
int oracle_refresh(oracle_sys_t *o);
int oracle_compute_forces(oracle_sys_t *o, int group);
int oracle_thermo(oracle_sys_t *o, int group, oracle_thermo_t *out);
int oracle_vv_steps(oracle_sys_t *o, int nsteps, double dt, int group, int thermostat, double tau, double T0);
int oracle_get_thermo(oracle_sys_t *o, oracle_thermo_t *out);
unsigned oracle_errors(oracle_sys_t *o);

/* 1-D two-temperature model (src/ttm.c, src/turi.c, src/forces.c:292-330,
   src/integrators.c:129-225).  The parameters are the reference's derived
   ones (what its fmd_ttm_set* calls and _fmd_ttm_getReady leave in its
   ttm_t): heat capacity / conductivity / coupling in internal units, laser
   constants, the activation threshold and the front surface. */
typedef struct
{
    int type;                 /* 1: C = gamma Te, constant K and G; 2: tabulated C(Te), G(Te), Zhigilei K */
    int ratio;                /* TTM substeps per MD step */
    unsigned min_atoms;       /* cells with fewer atoms are inactive */
    int nC, nG;
    double C_gamma, K, G, dz2, frontsurf;
    double laser_t0, laser_tdiff, laser_m_2sig2_inv, laser_m_absdepth_inv, laser_factor;
    double Kzh_v2, Kzh_A, Kzh_B;
    const double *T_C, *Ct, *C_DD, *T_G, *Gt, *G_DD;
} oracle_ttm_params_t;

/* a turi of one cell across x and y and nz local cells along z (margins
   included), itc_z = (int)(z / tcellh_z) + g2l_z; interior [lo, hi); the
   electron temperature starts at Te_init in the interior, -1 elsewhere */
int oracle_ttm_setup(oracle_sys_t *o, int nz, int g2l_z, int lo, int hi, double tcellh_z, double tcell_volume,
                     double starttime, double stoptime, const oracle_ttm_params_t *p, double Te_init);
int oracle_set_time(oracle_sys_t *o, double time, double dt);
/* the turi fields and the TTM solve at the current time (a run's first
   update, src/integrators.c:187-189), when within the turi's window */
int oracle_turi_update(oracle_sys_t *o);
/* symplectic Euler steps, each followed by the turi update and the forces
   with the TTM friction term (src/integrators.c:129-225) */
int oracle_se_steps(oracle_sys_t *o, int nsteps, double dt, int group);
/* the 1-D arrays (nz entries each; vcm 3 per cell) */
int oracle_ttm_1d(oracle_sys_t *o, unsigned *num, double *vcm, double *Ti, double *Te, double *xi);

#ifdef __cplusplus
}
#endif

#endif
