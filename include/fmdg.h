/*
 * fmdg.h -- C-ABI of the GB300 device engine behind libfmd.so.
 *
 * Plain C: opaque handles, plain pointers and sizes, int status codes
 * (0 = success, see FMDG_E_*).  The host side of libfmd.so (the fmd.h
 * implementation, written in C) calls these entry points; the Python test
 * and benchmark harness calls them through ctypes for kernel-level parity
 * checks.  Each entry point names the reference routine (FMD 0.4.0, path
 * within its project) whose per-timestep work it replaces.
 *
 * Data model: one device system (fmdg_sys_t) holds the whole periodic box of
 * one FMD instance in HBM as structure-of-arrays, sorted by interior cell in
 * the reference's cell order (flat index z + nz*(y + ny*x), src/general.h:56)
 * and, inside each cell, in the reference's in-cell order.  All arithmetic on
 * positions, velocities, forces and energies is IEEE binary64 in the drop-in
 * precision mode.
 */
#ifndef FMDG_H
#define FMDG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define FMDG_OK              0
#define FMDG_E_CUDA          1   /* a CUDA runtime call failed (message: fmdg_last_error) */
#define FMDG_E_ARG           2   /* invalid argument */
#define FMDG_E_NOMEM         3   /* device allocation failed */
#define FMDG_E_STATE         4   /* call made in the wrong state (e.g. no atoms) */

/* sticky device error bits, read with fmdg_get_errors (mirror the reference's
   error events raised from the per-step code) */
#define FMDG_ERRBIT_POSITION   0x1  /* atom left the local grid: src/misc.c:286-290 */
#define FMDG_ERRBIT_RHO_RANGE  0x2  /* EAM density beyond the F(rho) table: src/eam.c:168-171 */
#define FMDG_ERRBIT_TTM        0x4  /* TTM turi-cell index outside the grid */
#define FMDG_ERRBIT_INTERNAL   0x8  /* an internal index check failed (the access was skipped) */
#define FMDG_ERRBIT_TTM_TABLE  0x10 /* electron temperature outside a TTM table: src/ttm.c:162-183 */

/* pair categories: values of the reference's potcat_t (src/potential.h:26-32) */
#define FMDG_POT_NONE  0
#define FMDG_POT_LJ    1
#define FMDG_POT_EAM   2
#define FMDG_POT_MORSE 3

/* precision modes */
#define FMDG_PREC_FP64   0   /* drop-in: all pair arithmetic in binary64 */
#define FMDG_PREC_MIXED  1   /* pair/spline/embedding in binary32, sums in binary64 */

typedef struct fmdg_sys fmdg_sys_t;

/* One entry of the kinds x kinds pair table (src/potential.h:40-45).
   LJ    (src/lj.h:60-67):    p = {eps4, sig_sqr, cutoff_sqr, 0}
   Morse (src/morse.h:60-66): p = {D0, alpha, r0, cutoff_sqr}
   EAM   (src/eam.h:424-430): p = {0, 0, cutoff_sqr, 0}, iloc/jloc = element
                              indexes of the two kinds inside the EAM tables */
typedef struct
{
    int cat;
    int iloc, jloc;
    int pad;
    double p[4];
} fmdg_pair_t;

/* Thermodynamic reductions of the active group (src/integrators.c:78-92,
   src/matter.c:31-68) plus the last potential energy (src/lj.c:89) and
   pair virial.  The virial has no live counterpart in the reference (its
   only one, src/misc.c:66-82, is unused and sums x . F, wrong under
   periodic images): here it is the pair form over the same pairs and pair
   forces as the energy, sum over pairs of r_ij . F_ij (eV), so that
   P V = N k_B T + virial / 3. */
typedef struct
{
    double kinetic;        /* 0.5 * sum m v^2                        */
    double temperature;    /* sum m v^2 / (3 N k_B)                  */
    double momentum[3];    /* sum m v (internal units)               */
    double potential;      /* pair + embedding energy                */
    double count;          /* atoms in the active group              */
    double virial;         /* sum over pairs r_ij . F_ij (last force evaluation) */
} fmdg_thermo_t;

/* --- lifetime -------------------------------------------------------- */
int  fmdg_create(fmdg_sys_t **out, int device);
void fmdg_destroy(fmdg_sys_t *s);
const char *fmdg_last_error(void);
int  fmdg_device_count(int *count);

/* --- set-up (replaces the single-rank parts of src/subdomain.c:224-305,
       src/misc.c:41-62 and the potential tables of src/potential.c) ---- */
/* box length, periodicity and cell grid: nc[d] = (int)(l[d]/rc_max),
   cellh[d] = l[d]/nc[d] (src/misc.c:41-50) */
int fmdg_set_box(fmdg_sys_t *s, const double l[3], const int pbc[3], const int nc[3], const double cellh[3]);
/* masses in internal units (src/potential.c:47); eam_elem[k] = element
   index of kind k inside the EAM tables or -1 */
int fmdg_set_kinds(fmdg_sys_t *s, int nkinds, const double *mass, const int *eam_elem);
int fmdg_set_pairs(fmdg_sys_t *s, const fmdg_pair_t *table /* nkinds*nkinds */);
/* EAM tables on the r^2 grid (src/eam.c:376-555): F, F_DD [nelem*Nrho];
   rho, rhoDD [nelem*Nr2]; phi, phiDD [nelem*nelem*Nr2] (symmetric) */
int fmdg_set_eam(fmdg_sys_t *s, int nelem, int Nrho, double drho, int Nr2, double dr2,
                 const double *F, const double *F_DD, const double *rho, const double *rhoDD,
                 const double *phi, const double *phiDD);
int fmdg_set_precision(fmdg_sys_t *s, int mode);
/* Verlet skin (A) of the neighbour list, before fmdg_upload: the list holds
   the pairs within the largest cutoff + skin, indexed by stable atom slots,
   and is rebuilt on the device once an atom has moved more than skin/2.
   Used when every periodic box length exceeds twice the list radius and
   the radius spans at most two cells; otherwise (and with skin 0) the
   exact stencil list is rebuilt every step.  Default: 0.5 A for systems in
   mixed precision at upload (environment FMD_SKIN overrides), none in
   binary64 unless set here. */
int fmdg_set_skin(fmdg_sys_t *s, double skin);
/* Neighbour-list entries per atom (before fmdg_upload; 0, the default:
   1.3 x the count at the fullest cell's density + 16).  A multiple of 8 up
   to 1024.  An atom with more neighbours than the list holds scans its
   stencil directly (same results, slower), so this bounds list memory
   only. */
int fmdg_set_list_capacity(fmdg_sys_t *s, int entries);
/* Threads per atom of this system's skin-list builds: 0 (default) picks
   them by size (16 up to 2^14 atoms, 8 up to 2^16, else 1); 1, 2, 4, 8,
   16 or 32 fix them.
   Every choice builds the same list, entry for entry. */
int fmdg_set_build_lanes(fmdg_sys_t *s, int lanes);

/* --- atoms (replaces the distribution of the global grid to the local grid,
       src/matter.c:329-447, and the state gathers of src/misc.c:310-422) -- */
/* n atoms in cell order: cell_count[c] atoms of cell c, in in-cell order;
   x, v: n*3 interleaved (x0 y0 z0 x1 ...) */
int fmdg_upload(fmdg_sys_t *s, int n, const int *cell_count, const double *x, const double *v,
                const unsigned *kind, const int *group, const unsigned *atomid);
int fmdg_natoms(fmdg_sys_t *s, int *n);
/* any output pointer may be NULL; arrays are in cell order */
int fmdg_download(fmdg_sys_t *s, int *cell_of, double *x, double *v, double *F, double *vaream,
                  unsigned *kind, int *group, unsigned *atomid);
/* overwrite positions and/or velocities (cell order, n*3 interleaved) */
int fmdg_set_state(fmdg_sys_t *s, const double *x, const double *v);

/* --- per-timestep work ---------------------------------------------- */
/* cell-list refresh with the reference's cell assignment and in-cell order
   (src/misc.c:268-308 + src/md-ghost.c:827-869) */
int fmdg_refresh(fmdg_sys_t *s);
/* force field evaluation: src/forces.c:332-382 (LJ src/lj.c:28-90, Morse
   src/morse.c:30-92, EAM src/eam.c:29-322, hybrid src/forces.c:33-290) */
int fmdg_compute_forces(fmdg_sys_t *s, int active_group);
/* group thermodynamics from current velocities (src/matter.c:31-68) */
int fmdg_thermo(fmdg_sys_t *s, int active_group, fmdg_thermo_t *out);
/* velocity-Verlet steps (src/integrators.c:40-126,227-264): startStep with
   optional Berendsen scaling (lambda from the previous step's temperature),
   refresh, forces, finishStep.  thermostat=0: tau, T0 ignored. */
int fmdg_vv_steps(fmdg_sys_t *s, int nsteps, double dt, int active_group,
                  int thermostat, double tau, double T0);
/* Berendsen scale of the first step of a run from the current velocities
   (src/integrators.c:44-47 when the kinetic energy is not up to date) */
int fmdg_prepare_thermostat(fmdg_sys_t *s, int active_group, double dt, double tau, double T0);
/* last thermodynamic record (device->host copy; synchronises) */
int fmdg_get_thermo(fmdg_sys_t *s, fmdg_thermo_t *out);
/* sticky error bits since the last clear; clear=1 resets them */
int fmdg_get_errors(fmdg_sys_t *s, unsigned *bits, int clear);

/* --- continuum grids and the two-temperature model -------------------- */
/* Parameters of a 1-D TTM solver (src/ttm.h:35-90) in internal units
   (eV, A, ps, K); table pointers are host arrays copied by fmdg_ttm_setup. */
typedef struct
{
    int type;                /* 1: C = gamma Te, constant K, G; 2: tabulated C, G, Zhigilei K */
    int ratio;               /* MD steps / electron substeps (timestep_ratio) */
    unsigned min_atoms;      /* cells with fewer atoms are deactivated */
    int nC, nG;
    int pad;
    double C_gamma, K, G, dz2, frontsurf;
    double laser_t0, laser_tdiff, laser_m_2sig2_inv, laser_m_absdepth_inv, laser_factor;
    double Kzh_v2, Kzh_A, Kzh_B;
    const double *T_C, *Ct, *C_DD, *T_G, *Gt, *G_DD;
} fmdg_ttm_params_t;

/* a turi grid (src/turi.c:648-738): local dimensions incl. margins,
   itc_local = (int)(x/tcellh) + g2l, active in [starttime, stoptime] */
int fmdg_turi_add(fmdg_sys_t *s, const int dims_local[3], const int g2l[3], const double tcellh[3],
                  double starttime, double stoptime, int *handle);
/* attach the 1-D TTM electron solver to turi `turi` along z (interior
   cells [itc_lo, itc_hi)); its xi and vcm drive the friction term */
int fmdg_ttm_setup(fmdg_sys_t *s, int turi, int itc_lo, int itc_hi, const fmdg_ttm_params_t *p);
/* electron temperature of every local cell (margins included) */
int fmdg_ttm_set_te(fmdg_sys_t *s, int turi, const double *Te);
/* per-cell fields of turi `turi` (local cells incl. margins); any output may
   be NULL: num, mass (internal units), vcm (3 per cell), Ti, Te, xi */
int fmdg_turi_download(fmdg_sys_t *s, int turi, unsigned *num, double *mass, double *vcm, double *Ti,
                       double *Te, double *xi);
/* electron temperature of every local cell: presolve=1 gives the state after
   cell activation and before the substeps of the last update (what the
   reference's Te field holds during its field-update event), 0 the state
   after the substeps */
int fmdg_ttm_download_te(fmdg_sys_t *s, int turi, int presolve, double *Te);
/* simulation time and time step the device uses for turi windows, the
   laser source and the friction term; steps advance the time by dt */
int fmdg_set_time(fmdg_sys_t *s, double time, double dt);
/* field update of the turies selected by bit k of mask at the current time
   (src/turi.c:1627-1665): mass, vcm, number, temperature; then the TTM
   solver */
int fmdg_turi_update(fmdg_sys_t *s, double dt, unsigned mask);
/* symplectic-Euler steps under TTM coupling (src/integrators.c:129-225):
   kick-drift, refresh, time += dt, turi updates, forces + friction term */
int fmdg_se_steps(fmdg_sys_t *s, int nsteps, double dt, int active_group);

/* --- host-buffer path ------------------------------------------------ */
/* pinned host memory for the host-buffer path */
int fmdg_host_alloc(void **p, size_t bytes);
int fmdg_host_free(void *p);
/* positions/velocities in (structure of arrays: 3 rows of n, n = current
   atom count, current order), nsteps velocity-Verlet steps
   (src/integrators.c:227-264 without events), positions/velocities/atom ids
   in the new order and the thermo record out; any pointer may be NULL */
int fmdg_run_host(fmdg_sys_t *s, int nsteps, double dt, int group, const double *x_in, const double *v_in,
                  double *x_out, double *v_out, unsigned *id_out, fmdg_thermo_t *th_out);

/* --- allocation-free pair forces ------------------------------------ */
/* No counterpart in the reference.  Binary64 LJ / Morse forces and the
   total potential energy for callers that cannot let a library allocate
   device memory (work being recorded into a CUDA graph, hosts that own all
   device memory through their own pool, serving loops that must not incur
   cudaMalloc's implicit synchronisation).  Every input and output is the
   caller's device memory: x (structure of arrays, 3 rows of n), kind[n],
   cell_start[ncell+1] and cell_of[n] of atoms sorted by cell (flat cell
   index z + nz*(y + ny*x)); F (3 rows of n) and *pe (one double) receive the
   result.  pairs: host table of nkinds*nkinds entries (LJ or Morse only,
   nkinds <= 4); kind[i] must lie in [0, nkinds): an atom whose kind, or a
   neighbour's, lies outside gets NaN forces and *pe is NaN (the table is
   never read out of range).  stream: a cudaStream_t or NULL.  Scratch is a fixed
   512 KiB file-scope device array: at most 1048576 atoms per call (larger
   n returns FMDG_E_ARG with a message); the first call on a device looks up
   that array's address (under a lock: first calls from several host
   threads are safe) and should come before any stream capture; after a
   cudaDeviceReset of a device do not call it on that device again in the
   same process; calls that overlap on the GPU share the array and race. */
int fmdg_pair_forces_noalloc(int n, const int nc[3], const int pbc[3], const double l[3], int nkinds,
                             const fmdg_pair_t *pairs, const double *x, const unsigned *kind,
                             const int *cell_start, const int *cell_of, double *F, double *pe, void *stream);

/* --- whole-system edits after distribution -------------------------- */
int fmdg_add_velocity(fmdg_sys_t *s, int group, const double dv[3]);
int fmdg_change_group(fmdg_sys_t *s, int old_group, int new_group);

/* --- timing (CUDA events on the system's stream) --------------------- */
int fmdg_sync(fmdg_sys_t *s);
int fmdg_timer_start(fmdg_sys_t *s);
int fmdg_timer_stop(fmdg_sys_t *s, float *ms);
/* with profiling on, fmdg_vv_steps and fmdg_se_steps launch each phase
   between CUDA events (no graph) and accumulate its device time: phases
   "bin" (start step / kick-drift + refresh), "nlist", "density" (EAM pass 1
   + embedding), "force" (pair forces + finish step; fmdg_se_steps: list,
   density and forces together), "turi" (field passes), "ttm" (fmdg_se_steps:
   the TTM electron solver; fmdg_vv_steps counts it under "turi"); ms summed
   over steps */
int fmdg_set_profiling(fmdg_sys_t *s, int on);
int fmdg_get_profile(fmdg_sys_t *s, const char *name, float *ms, int *launches);
int fmdg_launch_count(fmdg_sys_t *s, long long *count);
/* issue-rate ceiling of the CUDA cores: independent FMA chains over all
   SMs, 2 flops per FMA (fp64=1: binary64, else binary32) */
int fmdg_measure_fma_peak(fmdg_sys_t *s, int fp64, double *tflops);
/* self-check of the integer binary64 -> binary32 rounding of the step
   kernels (d2f_rn): for n inputs, its results and the conversion
   instruction's */
int fmdg_check_d2f(fmdg_sys_t *s, const double *x, int n, float *ours, float *ref);
/* self-check of the TTM solver's binary64 reciprocal (a binary32 seed and
   two Newton-Raphson steps): for n inputs, its results and 1.0 / x */
int fmdg_check_recip(fmdg_sys_t *s, const double *x, int n, double *ours, double *ref);
/* write a buffer larger than L2 so the next kernel starts cold */
int fmdg_flush_l2(fmdg_sys_t *s);

/* --- shared EAM tables ---------------------------------------------- */
/* Use the EAM tables of `owner` (same device) without copying them; the
   owner must outlive `s`.  Many systems with one potential then read one
   copy of the tables (one L2 footprint). */
int fmdg_share_eam(fmdg_sys_t *s, const fmdg_sys_t *owner);

/* --- served mode: continuous batching of independent jobs --------------
   No counterpart in the reference, which runs one simulation per process
   (one fmd_t, src/integrators.c:227-264).  Jobs wait in a FIFO queue until
   the device bytes they need fit the HBM budget; admitted jobs of one pack
   class and precision are stepped together by one launch per kernel
   (velocity Verlet, NVE), chunk_steps steps per captured CUDA graph; the
   threads per block of the list/density/force kernels are autotuned per
   pack unless fixed with fmdg_srv_set_tuning.  A job's arithmetic does not
   depend on the other jobs: alone or in any mix its trajectory is the same
   bit for bit.  Pack class: the pair category (FMDG_POT_LJ, _EAM, _MORSE)
   of a job whose kind pairs all use one, 0 for a job that mixes categories
   (src/potential.h:26-32 hybrid tables, e.g. EAM metal + LJ gas). */
typedef struct fmdg_server fmdg_server_t;

typedef struct
{
    double l[3];              /* box lengths (A) */
    int pbc[3];               /* periodic axes */
    int nkinds;               /* 1..8 */
    const double *mass;       /* [nkinds], internal units (src/potential.c:47) */
    const int *eam_elem;      /* [nkinds] element in the EAM tables, or NULL */
    const fmdg_pair_t *pairs; /* [nkinds*nkinds] */
    int eam_key;              /* jobs with EAM pairs: tables registered with fmdg_srv_set_eam */
    int n;                    /* atoms */
    const double *x, *v;      /* n*3 interleaved, positions inside [0, l) */
    const unsigned *kind;     /* [n] */
    int steps;                /* velocity-Verlet steps */
    double dt;                /* time step (ps) */
    int precision;            /* FMDG_PREC_* */
    int keep_state;           /* keep the final positions/velocities/forces */
} fmdg_job_desc_t;

typedef struct
{
    int state;                /* 0 queued, 1 running, 2 done, 3 failed */
    int error;                /* FMDG_E_* of a failed job */
    int n, steps;
    double t_submit, t_start, t_done;   /* seconds on the server clock */
    fmdg_thermo_t first, last;          /* before the first step, after the last
                                           (both filled once the job is done) */
    unsigned errbits;                   /* sticky device error bits */
    unsigned pad;
    double device_bytes;                /* admission estimate */
} fmdg_job_result_t;

typedef struct
{
    int queued, running;
    long long admitted, finished, failed;
    double atom_steps;                  /* completed atom-steps */
    long long kernels;                  /* kernels launched (graph replays included) */
    double bytes_in_use, bytes_peak;    /* admission accounting */
    int pack_fblk[4][2];                /* tuned threads per block [class][mixed], 0 = not yet */
    long long pack_chunks[4][2], pack_rebuilds[4][2];
} fmdg_srv_stats_t;

int  fmdg_srv_create(fmdg_server_t **out, int device, size_t hbm_budget, int max_jobs, int chunk_steps);
void fmdg_srv_destroy(fmdg_server_t *srv);
/* EAM tables shared by every job that names `key` (arguments as fmdg_set_eam) */
int  fmdg_srv_set_eam(fmdg_server_t *srv, int key, int nelem, int Nrho, double drho, int Nr2, double dr2,
                      const double *F, const double *F_DD, const double *rho, const double *rhoDD,
                      const double *phi, const double *phiDD);
/* 0: autotune (default); 64, 128 or 256: fixed threads per block */
int  fmdg_srv_set_tuning(fmdg_server_t *srv, int fblk);
/* Verlet skin of the packed neighbour lists (default 0.8 A): a job's list
   holds the pairs within its largest cutoff + skin and is rebuilt once an
   atom has moved more than skin/2 since the last build; the skin is capped
   at 0.99 of the cutoff and below half of every periodic box length minus
   the cutoff.  Jobs need periodic box lengths above twice the cutoff. */
int  fmdg_srv_set_skin(fmdg_server_t *srv, double skin);
/* list entries per atom of the jobs submitted from now on (as
   fmdg_set_list_capacity, fixed at submission like the skin; 0: estimated
   per job from its initial density) */
int  fmdg_srv_set_list_capacity(fmdg_server_t *srv, int entries);
/* queue a job (the description is copied) */
int  fmdg_srv_submit(fmdg_server_t *srv, const fmdg_job_desc_t *job, long long *id);
/* one turn of the serving loop (reap finished chunks, admit, launch);
   wait=1 blocks on the oldest chunk when nothing new could be launched;
   *active = queued + running jobs */
int  fmdg_srv_progress(fmdg_server_t *srv, int wait, int *active);
int  fmdg_srv_result(fmdg_server_t *srv, long long id, fmdg_job_result_t *out);
/* final state of a finished keep_state job, cell order (n*3 interleaved) */
int  fmdg_srv_state(fmdg_server_t *srv, long long id, double *x, double *v, double *F, unsigned *atomid);
/* forget a finished job */
int  fmdg_srv_release(fmdg_server_t *srv, long long id);
int  fmdg_srv_now(fmdg_server_t *srv, double *seconds);
int  fmdg_srv_stats(fmdg_server_t *srv, fmdg_srv_stats_t *out);
/* benchmark helpers: admit every queued job that fits (no steps);
   advance every admitted job by k chunks and return the device time;
   one un-captured step of one pack timed phase by phase (ms[0] refresh,
   ms[1] neighbour lists, ms[2] EAM density, ms[3] forces + finish step) */
int  fmdg_srv_admit(fmdg_server_t *srv);
int  fmdg_srv_run_resident(fmdg_server_t *srv, int k, float *ms);
int  fmdg_srv_profile_pack(fmdg_server_t *srv, int pack_class, int mixed, float ms[4], double *atoms,
                           int *members);

#ifdef __cplusplus
}
#endif

#endif /* FMDG_H */
