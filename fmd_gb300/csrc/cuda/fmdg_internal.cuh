// Internal definitions shared by the device-engine translation units.
//
// HBM layout of one system (capacity `cap` atoms, `ncell` interior cells):
//   two ping-pong sides, each holding the atoms sorted by cell:
//     x[3*cap], v[3*cap]   binary64, structure of arrays (x[d*cap + i])
//     kind[cap], group[cap], atomid[cap], cell_of[cap], cell_start[ncell+1]
//   F[3*cap], vaream[cap]  (forces; EAM density, then F'(rho)) in the
//                          current order only: they are recomputed after
//                          every refresh, never permuted
//   binning scratch (per atom / per cell), reduction partials, thermo record.
// Dynamic scalars that change on the device (current side, atom count,
// simulation time) live in `Dyn` in device memory so the whole step can be
// captured once as a CUDA graph and replayed.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include "fmdg.h"
#include "fmdg_turi.cuh"

#define FMDG_MAXK 8            // atom kinds per system
#define FMDG_MAXE 4            // EAM elements per system

#define K_BOLTZMANN_D 8.6173303e-5

struct Dyn
{
    int cur;            // current ping-pong side
    int n;              // live atoms
    int n_next;         // atom count after the refresh in flight
    int any_move;       // a refresh moved at least one atom
    unsigned err;       // sticky error bits (FMDG_ERRBIT_*)
    unsigned blocks_done;   // ticket of the force kernel's last-block reduction
    int steps_left;     // packed launches: steps this system still takes
    int rebuild;        // skin list: rebuild before the next force pass
    unsigned nl_done;   // ticket of the skin-list build's last block
    int pad;
    double lambda;      // Berendsen scale for the next start step
    double time;        // simulation time (advanced by every step)
    double dt;          // time step of the current run (turi windows)
};

struct Side
{
    double *x, *v;
    unsigned *kind;
    int *group;
    unsigned *atomid;
    int *cell_of;
    int *cell_start;
    int *slot;          // skin-list systems: stable slot number of the atom
};

// integrator arguments of the step in flight (set by the host before a
// launch or a capture; per system in packed launches)
struct StepArgs
{
    double dt, tau, T0;
    int group, thermostat;
    double hk[FMDG_MAXK];   // half-kick coefficient dt * 0.5 / m of each kind (set_step_dt)
};

struct Geo   // passed by value to kernels
{
    StepArgs st;
    int cap, ncell;
    int nc[3];
    int pbc[3];
    double l[3], cellh[3], inv_cellh[3];
    float l_f[3], inv_cellh_f[3];   // binary32 copies (fast paths with binary64 fallbacks)
    const double4_32a *corig;       // per cell: frame origin, the centre (cx + 1/2, cy + 1/2, cz + 1/2) * cellh, binary64
    Side side[2];
    double *F, *vaream;
    float *fpf;        // binary32 copy of F'(rho) (mixed-precision EAM force pass)
    // per-step neighbour list (built after every refresh)
    float4 *xf4;       // cell-local coordinates (binary32) + kind bits, current order
    int *nbr;          // nbr[k*cap + i] = j | (stencil offset code << 26)
    int *nbr_count;    // true count (entries beyond maxnb are not stored)
    int maxnb;
    float rlist2;      // binary32 prefilter radius^2 (largest cutoff + margin)
    float cellh_f[3];  // binary32 cell widths (remainders cellh - cellh_f formed per block)
    // packed spline tables: per interval k {y_k, y_k+1, y''_k, y''_k+1}
    const double4_32a *pk_rho, *pk_phi, *pk_F;     // binary64
    const float4 *pkf_rho, *pkf_phi, *pkf_F;   // binary32 copies (mixed mode)
    const float4 *pkf_pr;       // per element e and interval k: {phi_ee, rho_e} side by side (one 32 B row)
    // binary64 mode, EAM: double-float forms (fmdg_df.cuh) of the tables
    // (per interval {hi coefficients, lo coefficients}), of the cell-local
    // coordinates and of F'(rho)
    const float4 *pkd_rho, *pkd_phi;
    float4 *xdf;       // per index {xf4, lo parts}: one 32-byte row (one 256-bit load per neighbour)
    float2 *fpdf;
    float4 *xll;       // skin lists, binary64 mode: lo parts of xl (double-float build-frame positions)
    double inv_dr2, inv_drho;
    // binning scratch
    int *bdest;        // destination interior cell, -1 deleted, -2 stays
    int *bpath;        // migration key bits
    int *bslot;        // final slot of a stayer inside its cell
    int *brank;        // departure rank inside the source cell
    int *bnewidx;      // new index of an arriving atom
    int *dep_count, *arr_lower, *arr_total, *bucket_fill;   // per cell
    int *arr_base;     // per cell + 1, exclusive scan of arr_total
    int *new_start;    // alias of the next side's cell_start
    int *bucket, *arr_slot;   // per arrival
    // potentials
    int nkinds;
    const fmdg_pair_t *pairs;     // nkinds*nkinds, device copy
    const float4 *pairf;          // nkinds*nkinds: p[0..3] rounded to binary32
    const float2 *paird;          // nkinds*nkinds*4: p[0..3] as double-float (hi, lo)
    const double *mass;           // nkinds
    const int *eam_elem;          // nkinds
    int nelem, Nrho, Nr2;
    double drho, dr2;
    const double *eF, *eFDD, *erho, *erhoDD, *ephi, *ephiDD;
    int has_eam;
    int prec;
    // TTM friction term (src/forces.c:292-330), 1-D along z
    int ttm_on;
    int ttm_g2l_z, ttm_nz;
    double ttm_tcellh_z, ttm_inv_tcellh_z, ttm_start, ttm_stop;
    const double *ttm_xi, *ttm_vcm;
    // reductions
    double *partials;             // per block: 8 doubles
    fmdg_thermo_t *thermo;
    Dyn *dyn;
    // Verlet-skin neighbour list of packed (served) systems, indexed by a
    // stable slot number: the reference's binning renumbers atoms every step,
    // the slots do not, so the list (radius largest cutoff + skin) is reused
    // until an atom has moved more than skin/2 since its build.  List entries
    // hold the neighbour's slot and the stencil offset between the two
    // atoms' cells at the build; positions are kept relative to the cell an
    // atom had at the build (unwrapped across periodic faces), so the offset
    // stays valid for the list's lifetime.
    int skin_on;
    int *pos;              // pos[slot] = current index, -1 after deletion
    int *cb;               // by slot: cell at the last build
    float4 *xl;            // by slot: position relative to that cell, kind bits
    float4 *xb;            // by slot: xl at the last build
    double4_32a *xd;       // by slot: binary64 position, kind
    int *gslot;            // by slot: group
    float *fpb;            // by slot: F'(rho) binary32
    double *fpd;           // by slot: F'(rho) binary64
    int srad;              // stencil radius in cells of the list build
    float rskin2;          // (largest cutoff + skin)^2, scaled units (xs)
    float half_skin2;      // (skin/2)^2, scaled units: displacement that triggers a rebuild
    // Scaled frame of the skin-list binary32 coordinates (xl, xb, xf4 of a
    // skin system): x' = xs x with xs = binary32(cellh[0]) / cellh[0] in
    // mixed precision (1 in binary64 mode).  The scaled cell width along x
    // is then a binary32 number, so the stencil offsets o * cellh_s are
    // exact (on every axis of a cubic grid) and a pair vector is off only
    // by the rounding of the two coordinates.  The binary32 pair kernels
    // work in scaled units with parameters scaled on the host
    // (skin_params), form the real force factor, and scale each atom's
    // force by 1/xs and its virial by 1/xs^2 in binary64; energies need no
    // scaling.  (Binary32 xs^2 and the EAM index factor inv_dr2 / xs^2 of a
    // scaled r^2 are formed per thread from xs.)
    double xs, inv_xs;
    float cellh_s[3];      // scaled cell widths, binary32 (remainders cellh xs - cellh_s formed per block)
};

struct fmdg_sys
{
    int device;
    cudaStream_t stream;
    Geo g;
    Geo *d_geo;
    bool box_set, atoms;
    bool uploaded;                // atoms were uploaded at least once (the device time carries over)
    int nkinds;
    fmdg_pair_t h_pairs[FMDG_MAXK * FMDG_MAXK];
    double h_mass[FMDG_MAXK];
    int h_eam_elem[FMDG_MAXK];
    int cats;                     // bit mask of pair categories present
    cudaEvent_t ev0, ev1;
    cudaEvent_t pev[6];
    bool profiling;
    float prof_ms[6];
    int prof_n[6];
    long long launches;
    // captured multi-step graph
    cudaGraphExec_t graph;
    int graph_key_valid;
    double graph_dt, graph_tau, graph_T0;
    int graph_group, graph_thermo, graph_steps;
    void *l2buf;
    size_t l2bytes;
    // continuum grids
    DTuri turi[FMDG_MAXT];
    int nturi;
    int ttm_turi;                 // index of the TTM turi or -1
    int graph_mode;               // 0 velocity Verlet, 1 symplectic Euler
    int fblk;                     // threads per block of the list/density/force kernels
    bool eam_borrowed;            // EAM tables belong to another system
    char *arena;                  // one device allocation holding the per-atom and per-cell buffers
    bool skin_set;                // skin chosen by the caller (any precision)
    int list_capacity;            // neighbour-list entries per atom; 0: estimated at upload
    int build_lanes;              // threads per atom of a skin-list build; 0: by size
    double rsk;                   // skin-list radius (largest cutoff + skin), real units
    double skin;                  // Verlet skin of the neighbour list (A), 0: exact per-step list
};

// the skin kernels' binary32 pair parameters in the scaled frame: the
// second half of the binary32 parameter table
__host__ __device__ inline const float4 *skin_params(const Geo &g) { return g.pairf + FMDG_MAXK * FMDG_MAXK; }

// scale of the skin-path binary32 frame and the constants that follow from
// it (Geo::xs ...); called whenever the cell grid, the precision, the pair
// table or the EAM tables change
int fmdg_skin_scale(fmdg_sys_t *s);

// time step of the next launches and the half-kick coefficients
// dt * 0.5 / m of every kind, in binary64 as the reference forms them
// (src/integrators.c:104-106); formed here once instead of by a binary64
// division at the start of every thread block
inline void set_step_dt(fmdg_sys_t *s, double dt)
{
    s->g.st.dt = dt;
    for (int k = 0; k < FMDG_MAXK; k++) s->g.st.hk[k] = k < s->nkinds ? dt * 0.5 / s->h_mass[k] : 0.0;
}

// ---- which system a thread block works on ------------------------------------
// The step kernels are templates over a locator.
//   LocOne : one system, its Geo in kernel parameter space.
//   LocPack: up to FMDG_PACK_MAX systems of one pair category and precision
//            in one launch, their Geo copies in kernel parameter space too.
//            bstart[s] is the first block of system s (bstart[nsys] = the
//            grid); a block finds its system by bisection over bstart.  The
//            index depends on blockIdx and parameters only, so the compiler
//            reads the Geo fields as uniform constant-bank loads instead of
//            holding them in per-thread registers.  A system whose
//            steps_left reached zero is skipped by every kernel.
#define FMDG_PACK_MAX 32

struct LocOne
{
    static constexpr int max_threads = 128;
    static constexpr int min_blocks = 0;      // 0: register count left to the compiler
    static constexpr int lean_min_blocks = 7; // lean force kernels: 7 blocks of 128 (72 registers), measured best
    static constexpr bool renumbered = false;  // skin-list slots stay the upload positions
    Geo g;
};

struct LocPack
{
    static constexpr int max_threads = 256;
    static constexpr int min_blocks = 0;
    static constexpr int lean_min_blocks = 0; // packed lean force kernels: compiler's choice, measured best
    static constexpr bool renumbered = true;   // slot = index whenever a list is built
    int nsys;
    int bstart[FMDG_PACK_MAX + 1];
    Geo geos[FMDG_PACK_MAX];
};
static_assert(sizeof(LocPack) < 32000, "a packed launch's parameters exceed the 32 KB limit");

__device__ __forceinline__ const Geo &loc_geo(const LocOne &L, int &bx, int &nb)
{
    bx = blockIdx.x;
    nb = gridDim.x;
    return L.g;
}

__device__ __forceinline__ const Geo &loc_geo(const LocPack &L, int &bx, int &nb)
{
    const int b = blockIdx.x;
    int lo = 0, hi = L.nsys;
    while (hi - lo > 1)
    {
        const int mid = (lo + hi) >> 1;
        if (L.bstart[mid] <= b) lo = mid;
        else hi = mid;
    }
    bx = b - L.bstart[lo];
    nb = L.bstart[lo + 1] - L.bstart[lo];
    return L.geos[lo];
}

__device__ __forceinline__ bool loc_idle(const LocOne &, const Geo &) { return false; }
__device__ __forceinline__ bool loc_idle(const LocPack &, const Geo &g) { return g.dyn->steps_left <= 0; }
// does this step produce a thermo record?  Single systems: every step (the
// fmd.h API reads it at any time).  Packed (served) systems report theirs
// only after their last step, so only that step forms energies, kinetic
// energy and momentum (uniform over a system's blocks: steps_left changes
// only after the last of them has finished)
__device__ __forceinline__ bool loc_thermo(const LocOne &, const Geo &) { return true; }
__device__ __forceinline__ bool loc_thermo(const LocPack &, const Geo &g) { return g.dyn->steps_left <= 1; }

// A pack: systems of one pair-category class and precision stepped
// together; one locator per block shape (its grid is bstart[nsys]).
struct fmdg_pack_launch
{
    cudaStream_t stream;
    int nsys;
    int cats;                   // bit mask (1 << FMDG_POT_*) of the members' pair categories
    int mixed;
    int lean;                   // every member has one kind (lean binary32 kernels)
    int fblk;                   // threads per block of the list/density/force kernels
    LocPack la;                 // 128-thread atom blocks
    LocPack lc;                 // 128-thread cell blocks
    LocPack lf;                 // force blocks of fblk threads
    LocPack ls;                 // one block per system
};
// all three return the number of kernels launched, or minus a status
int fmdg_pack_launch_start(const fmdg_pack_launch &P);
int fmdg_pack_launch_refresh(const fmdg_pack_launch &P);
int fmdg_pack_launch_forces(const fmdg_pack_launch &P, int phases);

// ---- helpers shared by the translation units --------------------------------
int fmdg_fail(const char *where, cudaError_t e);
int fmdg_set_error(const char *msg);

#define FMDG_CK(call)                                                    \
    do {                                                                 \
        cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) return fmdg_fail(#call, e_);              \
    } while (0)

// kernel launch wrappers (defined in their translation units)
int fmdg_launch_refresh(fmdg_sys_t *s, int mode, double dt, int group, int thermostat);
int fmdg_launch_turi(fmdg_sys_t *s, int k, double dt);
// the two halves of fmdg_launch_turi: the field passes, then the TTM solver
int fmdg_launch_turi_fields(fmdg_sys_t *s, int k, double dt);
int fmdg_launch_ttm_solve(fmdg_sys_t *s, int k, double dt);
int fmdg_launch_forces(fmdg_sys_t *s, int group, int finish, double dt, int thermostat, double tau, double T0);
int fmdg_launch_density(fmdg_sys_t *s, int group);
int fmdg_launch_nlist(fmdg_sys_t *s);
int fmdg_pack_tables(fmdg_sys_t *s);
int fmdg_launch_pair_forces(fmdg_sys_t *s, int group, int finish, double dt, int thermostat, double tau, double T0);
int fmdg_launch_thermo(fmdg_sys_t *s, int group, int thermostat, double dt, double tau, double T0);
int fmdg_force_blocks(const fmdg_sys_t *s);
int fmdg_capacity_estimate(const int *cell_count, int ncell, double cell_volume, double rlist);
int fmdg_list_capacity(const fmdg_sys_t *s, const int *cell_count, int ncell);
size_t fmdg_bytes_estimate(int n, int ncell, int maxnb);
int fmdg_set_steps_left(fmdg_sys_t *s, int steps);
// single-system path on a skin list (fmdg_skin.cu)
int fmdg_skin_launch_nlist(fmdg_sys_t *s);
int fmdg_skin_launch_density(fmdg_sys_t *s);
int fmdg_skin_launch_pair_forces(fmdg_sys_t *s, int finish);

// refresh modes
#define FMDG_REFRESH_ONLY  0     // positions already updated
#define FMDG_REFRESH_VV    1     // velocity-Verlet start step first
#define FMDG_REFRESH_SE    2     // symplectic Euler kick-drift first

static inline int fmdg_grid(int n, int b) { return (n + b - 1) / b; }

__device__ __forceinline__ void atomic_or_err(Dyn *d, unsigned bit) { atomicOr(&d->err, bit); }

// floor(x/h) exactly as binary64 division would give it: the product with
// 1/h (relative error <= 2^-52) decides unless it lies within 1e-9 of an
// integer, where the IEEE quotient is evaluated.
__device__ __forceinline__ double floor_div(double x, double h, double inv_h)
{
    const double q = x * inv_h;
    const double f = floor(q);
    const double tol = 1e-9 * fmax(1.0, fabs(q));
    if (q - f < tol || (f + 1.0) - q < tol) return floor(__ddiv_rn(x, h));
    return f;
}

// binary64 -> binary32 rounded to nearest even with integer operations
// (the conversion instruction issues at the binary64 rate on GB300): the
// 52-bit significand cut to 23 bits, the 29 dropped bits rounding the
// result (a carry into the exponent is the IEEE result); zero, subnormal
// and out-of-range inputs take the conversion instruction
__device__ __forceinline__ float d2f_rn(double x)
{
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const int e = (int)((hi >> 20) & 0x7ffu);
    if ((unsigned)(e - 897) > 253u) return __double2float_rn(x);
    unsigned f = ((unsigned)(e - 896) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;
    f += (rem > 0x10000000u) || (rem == 0x10000000u && (f & 1u));
    return __uint_as_float(f | (hi & 0x80000000u));
}

// floor_div as an int, through a binary32 estimate when its fraction is
// clear of an integer by more than its error (then both agree; one binary64
// instruction instead of a dozen -- binary64 issues at 1/64 of the binary32
// rate on GB300), else in binary64.  Results below -2 or above 2^30 come
// back as -2 (callers test against [-1, nc]).  (Conversion-free forms of
// the binary32 path -- d2f_rn, a magic-number floor -- measured no faster:
// the binning kernel is memory bound.)
__device__ __forceinline__ int cell_floor(double x, double h, double inv_h, float inv_hf)
{
    const float qf = __fmul_rn((float)x, inv_hf);
    const float ff = floorf(qf);
    const float fr = __fsub_rn(qf, ff);
    const float m = 4e-7f * (fabsf(qf) + 1.f);
    if (fr > m && fr < 1.f - m && fabsf(qf) < 1.0e6f) return (int)ff;
    const double q = floor_div(x, h, inv_h);
    return (q >= -2.0 && q <= 1073741824.0) ? (int)q : -2;
}
