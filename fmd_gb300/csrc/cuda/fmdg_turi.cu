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
// Per-cell sums over atoms are deterministic: lanes of a warp with the same
// cell are combined by shuffles in lane order (binary64), and each group's
// sum is added to the cell as a 64-bit fixed-point integer (integer atomics
// give the same total whatever order the additions arrive in).  Scales:
// mass 2^44, momentum 2^40, thermal kinetic term 2^36 (internal units;
// resolution 6e-14, 9e-13 and 1.5e-11 per group, far below the binary64
// rounding of the reference's own sums relative to the cell totals); a term
// beyond the fixed-point range sets FMDG_ERRBIT_INTERNAL and is skipped.
// The solver runs in one thread block: the grid has tens to hundreds of
// cells and the substeps are sequential; every quantity is binary64.
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
        idx[d] = trunc_div(x[d], t.tcellh[d], t.inv_tcellh[d]) + t.g2l[d];
        if (idx[d] < 0 || idx[d] >= t.dims[d]) { *bad = true; idx[d] = idx[d] < 0 ? 0 : t.dims[d] - 1; }
    }
    return idx[2] + t.dims[2] * (idx[1] + t.dims[1] * idx[0]);
}

// lanes holding the same key add their values; the lowest lane of each
// group returns true and holds the group's sum
template <int NV>
__device__ __forceinline__ bool group_sum(int key, double (&v)[NV])
{
    const unsigned mask = __match_any_sync(0xffffffffu, key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    for (int k = 0; k < NV; k++)
    {
        double s = 0.0;
        unsigned m = mask;
        while (m)
        {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            s += __shfl_sync(mask, v[k], src);
        }
        v[k] = s;
    }
    return lane == leader;
}

// fixed-point scales of the per-cell sums (powers of two: v * scale is exact)
constexpr double FX_MASS = 17592186044416.0;   // 2^44
constexpr double FX_MOM = 1099511627776.0;     // 2^40
constexpr double FX_KIN = 68719476736.0;       // 2^36
constexpr double FX_LIMIT = 4.0e18;            // |v * scale| below 2^62: room for the sums

__device__ __forceinline__ void add_fixed(Dyn *dyn, long long *dst, double v, double scale)
{
    const double q = v * scale;
    if (!(fabs(q) < FX_LIMIT))
    {
        atomic_or_err(dyn, FMDG_ERRBIT_INTERNAL);
        return;
    }
    atomicAdd(reinterpret_cast<unsigned long long *>(dst), (unsigned long long)__double2ll_rn(q));
}

__global__ void k_turi_clear(DTuri t)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < t.ncells; c += gridDim.x * blockDim.x)
    {
        for (int k = 0; k < 5; k++) t.acc[5 * c + k] = 0;
        t.tacc[c] = 0;
    }
}

// pass A: mass, momentum and count per turi cell (src/turi.c:1140-1155, 1213-1230)
__global__ void k_turi_pass_a(Geo g, DTuri t, double dt)
{
    Dyn *dyn = g.dyn;
    if (!turi_window(t, dyn->time, dt)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = dyn->n;
    const Side S = g.side[dyn->cur];
    const int cap = g.cap;
    bool valid = i < n, bad = false;
    int key = -1;
    double v[5] = {0, 0, 0, 0, 0};
    if (valid)
    {
        const double x[3] = {S.x[i], S.x[cap + i], S.x[2 * (size_t)cap + i]};
        key = atom_tcell(t, x, &bad);
        const double m = g.mass[S.kind[i]];
        v[0] = m;
        for (int d = 0; d < 3; d++) v[1 + d] = m * S.v[(size_t)d * cap + i];
        v[4] = 1.0;
    }
    if (bad) atomic_or_err(dyn, FMDG_ERRBIT_TTM);
    if (group_sum<5>(key, v) && key >= 0)
    {
        add_fixed(dyn, &t.acc[5 * key], v[0], FX_MASS);
        for (int d = 0; d < 3; d++) add_fixed(dyn, &t.acc[5 * key + 1 + d], v[1 + d], FX_MOM);
        atomicAdd(reinterpret_cast<unsigned long long *>(&t.acc[5 * key + 4]), (unsigned long long)v[4]);
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
__global__ void k_turi_pass_b(Geo g, DTuri t, double dt)
{
    Dyn *dyn = g.dyn;
    if (!turi_window(t, dyn->time, dt)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = dyn->n;
    const Side S = g.side[dyn->cur];
    const int cap = g.cap;
    bool bad = false;
    int key = -1;
    double v[1] = {0.0};
    if (i < n)
    {
        const double x[3] = {S.x[i], S.x[cap + i], S.x[2 * (size_t)cap + i]};
        key = atom_tcell(t, x, &bad);
        const double m = g.mass[S.kind[i]];
        double vt[3];
        for (int d = 0; d < 3; d++) vt[d] = S.v[(size_t)d * cap + i] - t.vcm[3 * key + d];
        v[0] = m * (vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
    }
    if (group_sum<1>(key, v) && key >= 0) add_fixed(dyn, &t.tacc[key], v[0], FX_KIN);
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

// type 2 coefficient update (src/ttm.c:154-192)
__device__ void type2_coeffs(Dyn *dyn, const DTuri &t, const double *Te, int c)
{
    const TtmParams &p = t.p;
    const double te = Te[c];
    if (te < 0.) return;
    if (te < p.T_C[0] || te > p.T_C[p.nC - 1]) atomic_or_err(dyn, FMDG_ERRBIT_TTM_TABLE);
    t.Ce[c] = spline_adv(p.T_C, p.Ct, p.C_DD, p.nC, te);
    t.Ke[c] = 1. / 3. * t.Ce[c] * p.Kzh_v2 / (p.Kzh_A * (te * te) + p.Kzh_B * t.Ti[c]);
    if (te < p.T_G[0] || te > p.T_G[p.nG - 1]) atomic_or_err(dyn, FMDG_ERRBIT_TTM_TABLE);
    t.Gc[c] = spline_adv(p.T_G, p.Gt, p.G_DD, p.nG, te);
}

// One thread block: cell activation, timestep_ratio FTCS substeps of the
// electron temperature with Neumann reflection at inactive neighbours,
// time-averaged Te and the friction coefficient xi.
__global__ void k_ttm_solve(Geo g, DTuri t, double dt)
{
    Dyn *dyn = g.dyn;
    const double time = dyn->time;
    if (!turi_window(t, time, dt)) return;
    const TtmParams &p = t.p;
    const int lo = t.itc_lo, hi = t.itc_hi;   // interior cells [lo, hi)
    double *Te = t.Te, *Te2 = t.Te2;
    // presolve (src/ttm.c:194-231): reads neighbours' Te before this
    // cell's own update, so it runs in cell order on one thread
    if (threadIdx.x == 0)
    {
        for (int i = lo; i < hi; i++)
        {
            t.xi[i] = 0.0;
            if (Te[i] < 0.0 && t.num[i] >= p.min_atoms)
            {
                int count = 0;
                double sum = 0.0;
                const int im1 = (i == lo) ? 0 : i - 1;
                if (Te[im1] >= 0.0) { sum += Te[im1] * t.num[im1]; count += t.num[im1]; }
                if (Te[i + 1] >= 0.0) { sum += Te[i + 1] * t.num[i + 1]; count += t.num[i + 1]; }
                Te[i] = (count > 0) ? sum / count : t.Ti[i];
            }
            if (t.num[i] < p.min_atoms) Te[i] = Te2[i] = -1.0;
        }
    }
    __syncthreads();
    // the field-update event of Te comes between activation and the
    // substeps (src/turi.c:1353-1358): keep that state for it
    for (int i = threadIdx.x; i < t.dims[2]; i += blockDim.x) t.Te_pre[i] = Te[i];
    if (p.type == 2)
    {
        for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) type2_coeffs(dyn, t, Te, i);
        __syncthreads();
    }
    const bool calc_source = fabs(time - p.laser_t0) < p.laser_tdiff;
    const double dte = dt / p.ratio;
    // spatial source factor (time independent)
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x)
    {
        const double z = (i - t.g2l[2] + 0.5) * t.tcellh[2];
        t.srcz[i] = calc_source ? exp(p.laser_m_absdepth_inv * (z - p.frontsurf)) : 0.0;
    }
    __syncthreads();
    for (int j = 0; j < p.ratio; j++)
    {
        double spc = 0.0;
        if (calc_source)
        {
            const double tt = time + j * dte - p.laser_t0;
            spc = p.laser_factor * exp(p.laser_m_2sig2_inv * (tt * tt));
        }
        for (int i = lo + threadIdx.x; i < hi; i += blockDim.x)
        {
            const double te = Te[i];
            if (te < 0) continue;
            const double source = calc_source ? spc * t.srcz[i] : 0.0;
            const int im1 = (i == lo) ? 0 : i - 1;
            const int ilo = (Te[im1] < 0) ? i : im1;
            const int ihi = (Te[i + 1] < 0) ? i : i + 1;
            double nv;
            if (p.type == 1)
                nv = te + dte / (p.C_gamma * te) *
                     (p.K * (Te[ihi] - 2 * te + Te[ilo]) / p.dz2 - p.G * (te - t.Ti[i]) + source);
            else
            {
                const double KeL = 0.5 * (t.Ke[i] + t.Ke[ilo]);
                const double KeR = 0.5 * (t.Ke[i] + t.Ke[ihi]);
                nv = te + dte / t.Ce[i] *
                     ((KeR * (Te[ihi] - te) - KeL * (te - Te[ilo])) / p.dz2 - t.Gc[i] * (te - t.Ti[i]) + source);
            }
            Te2[i] = nv;
            t.xi[i] += nv;
        }
        __syncthreads();
        double *tmp = Te2;
        Te2 = Te;
        Te = tmp;
        if (p.type == 2 && j < p.ratio - 1)
        {
            for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) type2_coeffs(dyn, t, Te, i);
            __syncthreads();
        }
    }
    // the freshest Te lives in `Te`; keep it in t.Te (margins included)
    if (Te != t.Te)
        for (int i = threadIdx.x; i < t.dims[2]; i += blockDim.x) t.Te[i] = Te[i];
    __syncthreads();
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x)
    {
        if (t.num[i] >= p.min_atoms)
        {
            const double Gi = (p.type == 1) ? p.G : t.Gc[i];
            t.xi[i] = Gi * t.tcell_volume * (t.xi[i] / p.ratio - t.Ti[i]) / (3 * K_BOLTZMANN_D * t.num[i] * t.Ti[i]);
        }
    }
}

} // namespace

int fmdg_launch_turi_fields(fmdg_sys_t *s, int k, double dt)
{
    DTuri &t = s->turi[k];
    cudaStream_t st = s->stream;
    const int nbc = fmdg_grid(t.ncells, 256);
    const int nba = fmdg_grid(s->g.cap, 256);
    k_turi_clear<<<nbc, 256, 0, st>>>(t);
    k_turi_pass_a<<<nba, 256, 0, st>>>(s->g, t, dt);
    k_turi_finish_a<<<nbc, 256, 0, st>>>(s->g, t, dt);
    k_turi_pass_b<<<nba, 256, 0, st>>>(s->g, t, dt);
    k_turi_finish_b<<<nbc, 256, 0, st>>>(s->g, t, dt);
    s->launches += 5;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

int fmdg_launch_ttm_solve(fmdg_sys_t *s, int k, double dt)
{
    DTuri &t = s->turi[k];
    if (!t.ttm) return FMDG_OK;
    k_ttm_solve<<<1, 128, 0, s->stream>>>(s->g, t, dt);
    s->launches++;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

int fmdg_launch_turi(fmdg_sys_t *s, int k, double dt)
{
    int rc = fmdg_launch_turi_fields(s, k, dt);
    return rc ? rc : fmdg_launch_ttm_solve(s, k, dt);
}
