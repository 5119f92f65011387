// Continuum grids ("turies"), their per-cell atomic fields and the 1-D
// two-temperature-model (TTM) electron solver.
//
// Reference (FMD 0.4.0):
//   atom -> turi cell   itc = (int)(x/tcellh) + itc_glob_to_loc  (src/turi.c:971-973)
//   MASS, VCM           src/turi.c:1112-1178 (vcm = sum m v / sum m)
//   NUMBER, TEMPERATURE src/turi.c:1190-1261 (T = sum m |v - vcm|^2 / (3 k_B N))
//   TTM presolve        src/ttm.c:194-248 (cell activation / deactivation)
//   TTM type 1 solve    src/ttm.c:250-312 (explicit FTCS substeps, C = gamma Te)
//   TTM type 2 solve    src/ttm.c:154-192, 314-383 (tabulated C, G; Zhigilei K)
//   xi                  src/ttm.c:305-311, 376-382
//   friction term       src/forces.c:292-330 (added in k_force)
// Per-cell sums over atoms are deterministic.  The atoms are in cell order,
// so the keys of a warp's 32 atoms form a few runs of equal keys; each run
// is summed by a segmented shuffle tree (binary64, a fixed order), and its
// total is added to the cell as a 64-bit fixed-point integer (integer
// atomics give the same total whatever order the additions arrive in),
// first into per-block bins in shared memory, then once per block and cell
// into the turi.  Scales: mass 2^48 (per kind, exact integer sums),
// momentum 2^46, thermal kinetic term 2^42 (internal units; resolution
// 1.4e-14 and 2.3e-13 per run, near the binary64 rounding of a single
// atom's term); a term beyond the fixed-point range is skipped and a sum
// that would wrap is detected, both setting FMDG_ERRBIT_INTERNAL.  These passes
// are binary64 work on a part whose binary64 pipe is narrow: the run trees
// cost five adds per value where a lane-by-lane group sum cost 32.
// The solver runs in one thread block: the grid has tens to hundreds of
// cells and the substeps are sequential; every quantity is binary64.
#include <algorithm>

#include "fmdg_internal.cuh"
#include "fmdg_turi.cuh"

namespace {

// (int)(x/h) with the reference's binary64 quotient: the product with 1/h
// decides except when it lies within a few ulps of an integer, where the
// IEEE division is evaluated.
__device__ __forceinline__ int trunc_div(double x, double h, double inv_h)
{
    const double q = x * inv_h;
    const double r = rint(q);
    if (fabs(q - r) <= 1e-9 * fmax(1.0, fabs(q))) return (int)__ddiv_rn(x, h);
    return (int)q;
}

__device__ __forceinline__ bool turi_window(const DTuri &t, double time, double dt)
{
    (void)dt;
    return (time >= t.starttime - dt / 2.0) && ((time < t.stoptime + dt / 2.0) || t.stoptime < t.starttime);
}

__device__ __forceinline__ int atom_tcell(const DTuri &t, const double x[3], bool *bad)
{
    int idx[3];
    for (int d = 0; d < 3; d++)
    {
        // one cell along d (the 1-D TTM grid's x and y): (int)(x/h) is 0
        // exactly for -h < x < h (the rounded quotient of such x stays
        // inside (-1, 1)), so only atoms outside need the quotient
        const bool inner = t.dims[d] == 1 && x[d] > -t.tcellh[d] && x[d] < t.tcellh[d];
        idx[d] = (inner ? 0 : trunc_div(x[d], t.tcellh[d], t.inv_tcellh[d])) + t.g2l[d];
        if (idx[d] < 0 || idx[d] >= t.dims[d]) { *bad = true; idx[d] = idx[d] < 0 ? 0 : t.dims[d] - 1; }
    }
    return idx[2] + t.dims[2] * (idx[1] + t.dims[1] * idx[0]);
}

// Runs: maximal stretches of consecutive lanes holding the same key (the
// atoms are in cell order, so a warp's keys form one to a few runs).
// Returns the last lane of this lane's run; head is set on its first lane.
__device__ __forceinline__ int run_end(int key, int lane, bool &head)
{
    const int prev = __shfl_up_sync(0xffffffffu, key, 1);
    head = lane == 0 || prev != key;
    const unsigned heads = __ballot_sync(0xffffffffu, head);
    const unsigned above = heads & ~((2u << lane) - 1u);   // heads of higher lanes (none for lane 31)
    return above ? __ffs(above) - 2 : 31;
}

// Segmented tree sum over the lanes of a run: after step o a lane holds the
// sum of its run's lanes [lane, lane + 2o - 1]; the head ends with the run
// total.  Five dependent adds per value instead of one per lane.
template <class T>
__device__ __forceinline__ T run_sum(T v, int lane, int end)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const T w = __shfl_down_sync(0xffffffffu, v, o);
        if (lane + o <= end) v += w;
    }
    return v;
}

// Fixed-point scales of the per-cell sums (powers of two: v * scale is
// exact).  FMD's internal mass unit makes m ~ 0.004-0.007 for argon and
// copper, m v ~ 1e-2 and m v^2 ~ 1e-2 per atom at room temperature: the
// scales put one quantum at ~1e-16 of such a term, and a cell total stays
// below 2^63 up to 1.3e5 (momentum) and 2.1e6 (thermal term) internal
// units -- 1e5 copper atoms at 20 A/ps, or at ~1e4 K.  A term or a sum
// beyond the range sets FMDG_ERRBIT_INTERNAL.
constexpr double FX_MASS = 281474976710656.0;  // 2^48
constexpr double FX_MOM = 70368744177664.0;    // 2^46
constexpr double FX_KIN = 4398046511104.0;     // 2^42
constexpr double FX_LIMIT = 4.0e18;            // |v * scale| below 2^62 for one term

// integer add into a bin (shared or global) with signed-overflow detection
// from the value the atomic returns
__device__ __forceinline__ void add_checked(Dyn *dyn, unsigned long long *dst, unsigned long long q)
{
    const unsigned long long old = atomicAdd(dst, q);
    const long long o = (long long)old, a = (long long)q, r = (long long)(old + q);
    if (((o ^ r) & (a ^ r)) < 0) atomic_or_err(dyn, FMDG_ERRBIT_INTERNAL);
}

// a run total as a fixed-point term; a term out of range is dropped (0) and
// sets FMDG_ERRBIT_INTERNAL
__device__ __forceinline__ unsigned long long fixed_term(Dyn *dyn, double v, double scale)
{
    const double q = v * scale;
    if (!(fabs(q) < FX_LIMIT))
    {
        atomic_or_err(dyn, FMDG_ERRBIT_INTERNAL);
        return 0ull;
    }
    return (unsigned long long)__double2ll_rn(q);
}

// Per-block bins in shared memory while the grid is small (one global
// atomic per block and cell term at the end), global atomics otherwise.
constexpr int TURI_SHARED_CELLS = 1024;   // 5 terms x 8 B x 1024 = 40 KB
constexpr int TURI_THREADS = 512;

__global__ void k_turi_clear(DTuri t)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < t.ncells; c += gridDim.x * blockDim.x)
    {
        for (int k = 0; k < 5; k++) t.acc[5 * c + k] = 0;
        t.tacc[c] = 0;
    }
}

// pass A: mass, momentum and count per turi cell (src/turi.c:1140-1155,
// 1213-1230).  Momenta are summed per run in binary64 and added as fixed
// point; masses as fixed point per kind (exact integer sums) and counts as
// run lengths.
template <bool SH>
__global__ void __launch_bounds__(TURI_THREADS) k_turi_pass_a(Geo g, DTuri t, double dt)
{
    extern __shared__ unsigned long long sbin[];   // SH: 5 terms per cell
    __shared__ long long smass[FMDG_MAXK];
    Dyn *dyn = g.dyn;
    if (!turi_window(t, dyn->time, dt)) return;
    if (threadIdx.x < g.nkinds) smass[threadIdx.x] = __double2ll_rn(g.mass[threadIdx.x] * FX_MASS);
    if (SH)
        for (int c = threadIdx.x; c < 5 * t.ncells; c += blockDim.x) sbin[c] = 0ull;
    __syncthreads();
    const int n = dyn->n;
    const Side S = g.side[dyn->cur];
    const size_t cap = g.cap;
    const int lane = threadIdx.x & 31;
    bool bad = false;
    // the bound is the same for the whole block: every lane reaches the shuffles
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x)
    {
        const int i = base + threadIdx.x;
        int key = -1;
        double p[3] = {0.0, 0.0, 0.0};
        long long mq = 0;
        if (i < n)
        {
            const double x[3] = {S.x[i], S.x[cap + i], S.x[2 * cap + i]};
            key = atom_tcell(t, x, &bad);
            const int kind = (int)S.kind[i];
            const double m = g.mass[kind];
            mq = smass[kind];
            for (int d = 0; d < 3; d++) p[d] = m * S.v[d * cap + i];
        }
        bool head;
        const int end = run_end(key, lane, head);
        for (int d = 0; d < 3; d++) p[d] = run_sum(p[d], lane, end);
        mq = run_sum(mq, lane, end);
        if (head && key >= 0)
        {
            unsigned long long q[5];
            q[0] = (unsigned long long)mq;
            for (int d = 0; d < 3; d++) q[1 + d] = fixed_term(dyn, p[d], FX_MOM);
            q[4] = (unsigned long long)(end - lane + 1);
            if (SH)
                for (int k = 0; k < 5; k++) add_checked(dyn, &sbin[5 * key + k], q[k]);
            else
                for (int k = 0; k < 5; k++)
                    add_checked(dyn, reinterpret_cast<unsigned long long *>(&t.acc[5 * key + k]), q[k]);
        }
    }
    if (bad) atomic_or_err(dyn, FMDG_ERRBIT_TTM);
    if (SH)
    {
        __syncthreads();
        for (int c = threadIdx.x; c < 5 * t.ncells; c += blockDim.x)
            if (sbin[c]) add_checked(dyn, reinterpret_cast<unsigned long long *>(&t.acc[c]), sbin[c]);
    }
}

// vcm, mass, number (src/turi.c:1163-1171 for the interior cells)
__global__ void k_turi_finish_a(Geo g, DTuri t, double dt)
{
    if (!turi_window(t, g.dyn->time, dt)) return;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < t.ncells; c += gridDim.x * blockDim.x)
    {
        const double m = (double)t.acc[5 * c] / FX_MASS;
        t.mass[c] = m;
        for (int d = 0; d < 3; d++) t.vcm[3 * c + d] = ((double)t.acc[5 * c + 1 + d] / FX_MOM) / m;
        t.num[c] = (unsigned)t.acc[5 * c + 4];
    }
}

// pass B: thermal kinetic energy about the cell's centre-of-mass velocity
// (run sums in binary64, added as fixed point)
template <bool SH>
__global__ void __launch_bounds__(TURI_THREADS) k_turi_pass_b(Geo g, DTuri t, double dt)
{
    extern __shared__ unsigned long long sbin[];   // SH: one term per cell
    Dyn *dyn = g.dyn;
    if (!turi_window(t, dyn->time, dt)) return;
    if (SH)
    {
        for (int c = threadIdx.x; c < t.ncells; c += blockDim.x) sbin[c] = 0ull;
        __syncthreads();
    }
    const int n = dyn->n;
    const Side S = g.side[dyn->cur];
    const size_t cap = g.cap;
    const int lane = threadIdx.x & 31;
    for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x)
    {
        const int i = base + threadIdx.x;
        int key = -1;
        double e = 0.0;
        if (i < n)
        {
            bool bad = false;
            const double x[3] = {S.x[i], S.x[cap + i], S.x[2 * cap + i]};
            key = atom_tcell(t, x, &bad);
            const double m = g.mass[S.kind[i]];
            double vt[3];
            for (int d = 0; d < 3; d++) vt[d] = S.v[d * cap + i] - t.vcm[3 * key + d];
            e = m * (vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
        }
        bool head;
        const int end = run_end(key, lane, head);
        e = run_sum(e, lane, end);
        if (head && key >= 0)
        {
            const unsigned long long q = fixed_term(dyn, e, FX_KIN);
            if (SH) add_checked(dyn, &sbin[key], q);
            else add_checked(dyn, reinterpret_cast<unsigned long long *>(&t.tacc[key]), q);
        }
    }
    if (SH)
    {
        __syncthreads();
        for (int c = threadIdx.x; c < t.ncells; c += blockDim.x)
            if (sbin[c]) add_checked(dyn, reinterpret_cast<unsigned long long *>(&t.tacc[c]), sbin[c]);
    }
}

__global__ void k_turi_finish_b(Geo g, DTuri t, double dt)
{
    if (!turi_window(t, g.dyn->time, dt)) return;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < t.ncells; c += gridDim.x * blockDim.x)
        t.Ti[c] = ((double)t.tacc[c] / FX_KIN) / (3.0 * K_BOLTZMANN_D * t.num[c]);
}

// natural spline on arbitrary knots with the reference's bisection
// (src/cspline.h:29-44, src/cspline.h:26)
__device__ double spline_adv(const double *xs, const double *ys, const double *dd, int n, double x)
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
    return a * ys[klo] + b * ys[khi] + ((a * a * a - a) * dd[klo] + (b * b * b - b) * dd[khi]) * (h * h) / 6.0;
}

// 1/x to a few ulps for positive x of binary32 range: a binary32 seed
// refined by two Newton-Raphson steps r <- r + r (1 - x r), each of which
// squares the relative error (2^-23 -> 2^-46 -> the binary64 rounding)
__device__ __forceinline__ double recip_newton(double x)
{
    double r = (double)__frcp_rn((float)x);
    r = fma(r, fma(-x, r, 1.0), r);
    r = fma(r, fma(-x, r, 1.0), r);
    return r;
}

// The solver's per-cell arrays: the turi's own (global memory) or copies
// in shared memory for the duration of the launch.
struct TtmCells
{
    double *Te, *Te2, *Ti, *srcz, *xi, *Ke, *Ce, *Gc;
    const unsigned *num;
    double *spc;   // staged: the laser's time factor of every substep
};

// type 2 coefficient update (src/ttm.c:154-192)
__device__ void type2_coeffs(Dyn *dyn, const TtmParams &p, const TtmCells &a, const double *Te, int c)
{
    const double te = Te[c];
    if (te < 0.) return;
    if (te < p.T_C[0] || te > p.T_C[p.nC - 1]) atomic_or_err(dyn, FMDG_ERRBIT_TTM_TABLE);
    a.Ce[c] = spline_adv(p.T_C, p.Ct, p.C_DD, p.nC, te);
    a.Ke[c] = 1. / 3. * a.Ce[c] * p.Kzh_v2 / (p.Kzh_A * (te * te) + p.Kzh_B * a.Ti[c]);
    if (te < p.T_G[0] || te > p.T_G[p.nG - 1]) atomic_or_err(dyn, FMDG_ERRBIT_TTM_TABLE);
    a.Gc[c] = spline_adv(p.T_G, p.Gt, p.G_DD, p.nG, te);
}

// shared bytes of a staged solver launch: eight binary64 arrays and the
// counts per cell, the laser factor per substep
__host__ __device__ inline size_t ttm_stage_bytes(int nz, int ratio)
{
    return (size_t)nz * (8 * sizeof(double) + sizeof(unsigned)) + (size_t)ratio * sizeof(double);
}

// One thread block: cell activation, timestep_ratio FTCS substeps of the
// electron temperature with Neumann reflection at inactive neighbours,
// time-averaged Te and the friction coefficient xi.  staged: the cell
// arrays live in shared memory for the launch (the substeps are a chain of
// dependent reads of neighbouring cells), and the laser's time factor of
// every substep is formed up front, in parallel.
__global__ void k_ttm_solve(Geo g, DTuri t, double dt, int staged)
{
    extern __shared__ double sm[];
    Dyn *dyn = g.dyn;
    const double time = dyn->time;
    if (!turi_window(t, time, dt)) return;
    const TtmParams &p = t.p;
    const int lo = t.itc_lo, hi = t.itc_hi;   // interior cells [lo, hi)
    const int nz = t.dims[2];
    const bool calc_source = fabs(time - p.laser_t0) < p.laser_tdiff;
    const double dte = dt / p.ratio;
    const double dte_C = dte / p.C_gamma, K_dz2 = p.K / p.dz2;   // type 1
    TtmCells a{t.Te, t.Te2, t.Ti, t.srcz, t.xi, t.Ke, t.Ce, t.Gc, t.num, nullptr};
    if (staged)
    {
        a.Te = sm;
        a.Te2 = sm + nz;
        a.Ti = sm + 2 * nz;
        a.srcz = sm + 3 * nz;
        a.xi = sm + 4 * nz;
        a.Ke = sm + 5 * nz;
        a.Ce = sm + 6 * nz;
        a.Gc = sm + 7 * nz;
        a.spc = sm + 8 * nz;
        unsigned *num = reinterpret_cast<unsigned *>(a.spc + p.ratio);
        for (int i = threadIdx.x; i < nz; i += blockDim.x)
        {
            a.Te[i] = t.Te[i];
            a.Te2[i] = t.Te2[i];
            a.Ti[i] = t.Ti[i];
            a.xi[i] = t.xi[i];
            a.Ke[i] = t.Ke[i];
            a.Ce[i] = t.Ce[i];
            a.Gc[i] = t.Gc[i];
            num[i] = t.num[i];
        }
        for (int j = threadIdx.x; j < p.ratio; j += blockDim.x)
        {
            double spc = 0.0;
            if (calc_source)
            {
                const double tt = time + j * dte - p.laser_t0;
                spc = p.laser_factor * exp(p.laser_m_2sig2_inv * (tt * tt));
            }
            a.spc[j] = spc;
        }
        a.num = num;
        __syncthreads();
    }
    double *Te = a.Te, *Te2 = a.Te2;
    // presolve (src/ttm.c:194-231): reads neighbours' Te before this
    // cell's own update, so it runs in cell order on one thread
    if (threadIdx.x == 0)
    {
        for (int i = lo; i < hi; i++)
        {
            a.xi[i] = 0.0;
            if (Te[i] < 0.0 && a.num[i] >= p.min_atoms)
            {
                int count = 0;
                double sum = 0.0;
                const int im1 = (i == lo) ? 0 : i - 1;
                if (Te[im1] >= 0.0) { sum += Te[im1] * a.num[im1]; count += a.num[im1]; }
                if (Te[i + 1] >= 0.0) { sum += Te[i + 1] * a.num[i + 1]; count += a.num[i + 1]; }
                Te[i] = (count > 0) ? sum / count : a.Ti[i];
            }
            if (a.num[i] < p.min_atoms) Te[i] = Te2[i] = -1.0;
        }
    }
    __syncthreads();
    // the field-update event of Te comes between activation and the
    // substeps (src/turi.c:1353-1358): keep that state for it
    for (int i = threadIdx.x; i < nz; i += blockDim.x) t.Te_pre[i] = Te[i];
    if (p.type == 2)
    {
        for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) type2_coeffs(dyn, p, a, Te, i);
        __syncthreads();
    }
    // spatial source factor (time independent)
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x)
    {
        const double z = (i - t.g2l[2] + 0.5) * t.tcellh[2];
        a.srcz[i] = calc_source ? exp(p.laser_m_absdepth_inv * (z - p.frontsurf)) : 0.0;
    }
    __syncthreads();
    for (int j = 0; j < p.ratio; j++)
    {
        double spc = 0.0;
        if (calc_source)
        {
            if (staged) spc = a.spc[j];
            else
            {
                const double tt = time + j * dte - p.laser_t0;
                spc = p.laser_factor * exp(p.laser_m_2sig2_inv * (tt * tt));
            }
        }
        for (int i = lo + threadIdx.x; i < hi; i += blockDim.x)
        {
            const double te = Te[i];
            if (te < 0) continue;
            const double source = calc_source ? spc * a.srcz[i] : 0.0;
            const int im1 = (i == lo) ? 0 : i - 1;
            const int ilo = (Te[im1] < 0) ? i : im1;
            const int ihi = (Te[i + 1] < 0) ? i : i + 1;
            double nv;
            if (p.type == 1)
            {
                // dte / (C_gamma te) * (K lap / dz2 - G (te - Ti) + source)
                // with the constant quotients formed once per launch and one
                // reciprocal: the substeps are a chain of dependent binary64
                // operations, and an IEEE division is the longest link
                const double q = dte_C * recip_newton(te);
                nv = te + q * (K_dz2 * (Te[ihi] - 2 * te + Te[ilo]) - p.G * (te - a.Ti[i]) + source);
            }
            else
            {
                const double KeL = 0.5 * (a.Ke[i] + a.Ke[ilo]);
                const double KeR = 0.5 * (a.Ke[i] + a.Ke[ihi]);
                nv = te + dte / a.Ce[i] *
                     ((KeR * (Te[ihi] - te) - KeL * (te - Te[ilo])) / p.dz2 - a.Gc[i] * (te - a.Ti[i]) + source);
            }
            Te2[i] = nv;
            a.xi[i] += nv;
        }
        __syncthreads();
        double *tmp = Te2;
        Te2 = Te;
        Te = tmp;
        if (p.type == 2 && j < p.ratio - 1)
        {
            for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) type2_coeffs(dyn, p, a, Te, i);
            __syncthreads();
        }
    }
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x)
    {
        if (a.num[i] >= p.min_atoms)
        {
            const double Gi = (p.type == 1) ? p.G : a.Gc[i];
            a.xi[i] = Gi * t.tcell_volume * (a.xi[i] / p.ratio - a.Ti[i]) / (3 * K_BOLTZMANN_D * a.num[i] * a.Ti[i]);
        }
    }
    __syncthreads();
    if (staged)
    {
        // the freshest Te to the turi's Te, the other buffer to Te2 (only
        // its inactive cells, -1, are read before they are rewritten)
        for (int i = threadIdx.x; i < nz; i += blockDim.x)
        {
            t.Te[i] = Te[i];
            t.Te2[i] = Te2[i];
            t.xi[i] = a.xi[i];
            t.Ke[i] = a.Ke[i];
            t.Ce[i] = a.Ce[i];
            t.Gc[i] = a.Gc[i];
        }
    }
    else if (Te != t.Te)
    {
        // the freshest Te lives in `Te`; keep it in t.Te (margins included)
        for (int i = threadIdx.x; i < nz; i += blockDim.x) t.Te[i] = Te[i];
    }
}

int sm_count(int device)
{
    static int cached[64] = {0};
    if (device < 0 || device >= 64) return 152;
    if (!cached[device])
    {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || v <= 0) v = 152;
        cached[device] = v;
    }
    return cached[device];
}

__global__ void k_recip_check(const double *x, int n, double *ours, double *ref)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    ours[i] = recip_newton(x[i]);
    ref[i] = 1.0 / x[i];
}

} // namespace

extern "C" int fmdg_check_recip(fmdg_sys_t *s, const double *x, int n, double *ours, double *ref)
{
    if (n < 0) return fmdg_set_error("fmdg_check_recip: negative count");
    if (n == 0) return FMDG_OK;
    double *d = nullptr;
    cudaError_t e = cudaMalloc(&d, (size_t)n * 24);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d, x, (size_t)n * 8, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
    {
        k_recip_check<<<fmdg_grid(n, 256), 256, 0, s->stream>>>(d, n, d + n, d + 2 * (size_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(ours, d + n, (size_t)n * 8, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ref, d + 2 * (size_t)n, (size_t)n * 8, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    return e == cudaSuccess ? FMDG_OK : fmdg_fail("fmdg_check_recip", e);
}

int fmdg_launch_turi_fields(fmdg_sys_t *s, int k, double dt)
{
    DTuri &t = s->turi[k];
    cudaStream_t st = s->stream;
    const int nbc = fmdg_grid(t.ncells, 256);
    // two blocks of 512 per SM, each looping over the atoms
    const int nba = std::max(1, std::min(2 * sm_count(s->device), fmdg_grid(s->g.cap, TURI_THREADS)));
    k_turi_clear<<<nbc, 256, 0, st>>>(t);
    if (t.ncells <= TURI_SHARED_CELLS)
    {
        k_turi_pass_a<true><<<nba, TURI_THREADS, 5 * t.ncells * sizeof(unsigned long long), st>>>(s->g, t, dt);
        k_turi_finish_a<<<nbc, 256, 0, st>>>(s->g, t, dt);
        k_turi_pass_b<true><<<nba, TURI_THREADS, t.ncells * sizeof(unsigned long long), st>>>(s->g, t, dt);
    }
    else
    {
        k_turi_pass_a<false><<<nba, TURI_THREADS, 0, st>>>(s->g, t, dt);
        k_turi_finish_a<<<nbc, 256, 0, st>>>(s->g, t, dt);
        k_turi_pass_b<false><<<nba, TURI_THREADS, 0, st>>>(s->g, t, dt);
    }
    k_turi_finish_b<<<nbc, 256, 0, st>>>(s->g, t, dt);
    s->launches += 5;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

int fmdg_launch_ttm_solve(fmdg_sys_t *s, int k, double dt)
{
    DTuri &t = s->turi[k];
    if (!t.ttm) return FMDG_OK;
    const size_t bytes = ttm_stage_bytes(t.dims[2], t.p.ratio);
    const int staged = bytes <= 48 * 1024;
    k_ttm_solve<<<1, 128, staged ? bytes : 0, s->stream>>>(s->g, t, dt, staged);
    s->launches++;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

int fmdg_launch_turi(fmdg_sys_t *s, int k, double dt)
{
    int rc = fmdg_launch_turi_fields(s, k, dt);
    return rc ? rc : fmdg_launch_ttm_solve(s, k, dt);
}
