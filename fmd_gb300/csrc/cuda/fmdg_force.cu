// Pair-force, EAM density/embedding and reduction kernels (binary64 path).
//
// Reference loops replaced (FMD 0.4.0):
//   LJ    src/lj.c:28-90    with the pair update of src/lj.h:26-58
//   Morse src/morse.c:30-92 with the pair update of src/morse.h:26-58
//   EAM   src/eam.c:225-322 (density, pass 1), src/eam.c:160-223 (embedding
//         F(rho), F'(rho)), src/eam.c:29-146 (forces, pass 0), pair updates
//         src/eam.h:29-406, cubic spline src/cspline.h:26-27
//   hybrid src/forces.c:33-290 (per-pair category switch)
//   ghost images / partial-force fold-back src/md-ghost.c:711-825 and the
//   PE Allreduce: replaced by periodic image shifts inside the loop and a
//   deterministic two-level block reduction.
//
// The reference visits each pair once (half shell, Newton's third law,
// scattering into both atoms).  Here each thread owns one atom and gathers
// over the full 27-cell stencil: every pair is evaluated from both sides,
// no atomics, deterministic results, and the per-atom energy takes half of
// each pair term.  Image shifts: a neighbour cell index below 0 (above
// nc-1) along a periodic axis is the ghost copy of cell nc-1 (0) shifted by
// -l (+l), exactly the ghost positions of src/md-ghost.c:85-107; along an
// open axis it is empty.
#include "fmdg_internal.cuh"

namespace {

enum { CAT_LJ = 1, CAT_EAM = 2, CAT_MORSE = 3, CAT_HYBRID = 4 };

struct SmemPot
{
    fmdg_pair_t pairs[FMDG_MAXK * FMDG_MAXK];
    double mass[FMDG_MAXK];
    int elem[FMDG_MAXK];
};

__device__ __forceinline__ void load_pot(const Geo &g, SmemPot &sp)
{
    const int nk2 = g.nkinds * g.nkinds;
    for (int k = threadIdx.x; k < nk2; k += blockDim.x) sp.pairs[k] = g.pairs[k];
    for (int k = threadIdx.x; k < g.nkinds; k += blockDim.x)
    {
        sp.mass[k] = g.mass[k];
        sp.elem[k] = g.eam_elem[k];
    }
    __syncthreads();
}

// natural cubic spline on a uniform grid (src/cspline.h:26-27)
__device__ __forceinline__ double spl_val(const double *y, const double *ydd, int lo, double a, double b, double h)
{
    return a * y[lo] + b * y[lo + 1] + ((a * a * a - a) * ydd[lo] + (b * b * b - b) * ydd[lo + 1]) * (h * h) / 6.0;
}

__device__ __forceinline__ double spl_der(const double *y, const double *ydd, int lo, double a, double b, double h)
{
    return (y[lo + 1] - y[lo]) / h + ((3 * b * b - 1) * ydd[lo + 1] - (3 * a * a - 1) * ydd[lo]) * h / 6.0;
}

// Visit every (atom j, image shift) of the 27-cell stencil around cell c.
template <typename F>
__device__ __forceinline__ void for_each_neighbour(const Geo &g, const Side &S, int i, int c, F &&f)
{
    const int cx = c / (g.nc[1] * g.nc[2]), cy = (c / g.nc[2]) % g.nc[1], cz = c % g.nc[2];
    for (int ox = -1; ox <= 1; ox++)
    {
        int jx = cx + ox;
        double sx = 0.0;
        if (jx < 0) { if (!g.pbc[0]) continue; jx += g.nc[0]; sx = -g.l[0]; }
        else if (jx >= g.nc[0]) { if (!g.pbc[0]) continue; jx -= g.nc[0]; sx = g.l[0]; }
        for (int oy = -1; oy <= 1; oy++)
        {
            int jy = cy + oy;
            double sy = 0.0;
            if (jy < 0) { if (!g.pbc[1]) continue; jy += g.nc[1]; sy = -g.l[1]; }
            else if (jy >= g.nc[1]) { if (!g.pbc[1]) continue; jy -= g.nc[1]; sy = g.l[1]; }
            for (int oz = -1; oz <= 1; oz++)
            {
                int jz = cz + oz;
                double sz = 0.0;
                if (jz < 0) { if (!g.pbc[2]) continue; jz += g.nc[2]; sz = -g.l[2]; }
                else if (jz >= g.nc[2]) { if (!g.pbc[2]) continue; jz -= g.nc[2]; sz = g.l[2]; }
                const int nb = jz + g.nc[2] * (jy + g.nc[1] * jx);
                const bool self = (ox == 0 && oy == 0 && oz == 0);
                const int jb = S.cell_start[nb], je = S.cell_start[nb + 1];
                for (int j = jb; j < je; j++)
                {
                    if (self && j == i) continue;
                    f(j, sx, sy, sz);
                }
            }
        }
    }
}

// rv = x_i - (x_j + shift), r2 summed as the reference does (no FMA)
struct PairGeom
{
    double rv[3];
    double r2;
};

__device__ __forceinline__ PairGeom pair_geom(const double xi[3], const Side &S, int cap, int j,
                                              double sx, double sy, double sz)
{
    PairGeom p;
    const double s[3] = {sx, sy, sz};
    for (int d = 0; d < 3; d++)
    {
        double x2 = S.x[d * cap + j];
        if (s[d] != 0.0) x2 = __dadd_rn(x2, s[d]);
        p.rv[d] = __dsub_rn(xi[d], x2);
    }
    p.r2 = __dadd_rn(__dadd_rn(__dmul_rn(p.rv[0], p.rv[0]), __dmul_rn(p.rv[1], p.rv[1])),
                     __dmul_rn(p.rv[2], p.rv[2]));
    return p;
}

// Deterministic block reduction of NV doubles; thread 0 writes out[0..NV).
template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double *out)
{
    __shared__ double red[32][NV];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int k = 0; k < NV; k++)
        for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
    if (lane == 0)
        for (int k = 0; k < NV; k++) red[w][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0)
    {
        const int nw = (blockDim.x + 31) >> 5;
        for (int k = 0; k < NV; k++)
        {
            double t = 0.0;
            for (int q = 0; q < nw; q++) t += red[q][k];
            out[k] = t;
        }
    }
}

// EAM pass 1 + embedding: rho_i = sum_j f_{elem(j)}(r_ij^2), then
// vaream_i = F'(rho_i) and the embedding energy F(rho_i) into the partials.
template <bool HYBRID>
__global__ void __launch_bounds__(128) k_density(Geo g, int group)
{
    __shared__ SmemPot sp;
    load_pot(g, sp);
    Dyn *dyn = g.dyn;
    const int n = dyn->n;
    const Side S = g.side[dyn->cur];
    const int cap = g.cap;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double acc[1] = {0.0};
    if (i < n)
    {
        const int ki = S.kind[i];
        const int ei = sp.elem[ki];
        const bool active = (group < 0 || S.group[i] == group) && (!HYBRID || ei >= 0);
        double rho = 0.0;
        if (active)
        {
            const double xi[3] = {S.x[i], S.x[cap + i], S.x[2 * cap + i]};
            const double h = g.dr2;
            for_each_neighbour(g, S, i, S.cell_of[i], [&](int j, double sx, double sy, double sz) {
                if (group >= 0 && S.group[j] != group) return;
                const int kj = S.kind[j];
                const fmdg_pair_t &pp = sp.pairs[ki * g.nkinds + kj];
                if (HYBRID && pp.cat != FMDG_POT_EAM) return;
                const PairGeom p = pair_geom(xi, S, cap, j, sx, sy, sz);
                if (p.r2 < pp.p[2])
                {
                    const int ir2 = min((int)(p.r2 / h), g.Nr2 - 2);
                    const double a = (ir2 + 1) - p.r2 / h;
                    const double b = 1 - a;
                    const int ej = pp.jloc;
                    rho += spl_val(g.erho + (size_t)ej * g.Nr2, g.erhoDD + (size_t)ej * g.Nr2, ir2, a, b, h);
                }
            });
            // embedding (src/eam.c:160-179)
            const double hr = g.drho;
            int irho = (int)(rho / hr);
            if (irho >= g.Nrho - 1 || irho < 0)
            {
                atomic_or_err(dyn, FMDG_ERRBIT_RHO_RANGE);
                irho = irho < 0 ? 0 : g.Nrho - 2;
            }
            const double a = (irho + 1) - rho / hr;
            const double b = 1 - a;
            const double *Ft = g.eF + (size_t)ei * g.Nrho;
            const double *Fdd = g.eFDD + (size_t)ei * g.Nrho;
            g.vaream[i] = spl_der(Ft, Fdd, irho, a, b, hr);
            acc[0] = spl_val(Ft, Fdd, irho, a, b, hr);
        }
        else
            g.vaream[i] = 0.0;
    }
    block_reduce_store<1>(acc, g.partials + (size_t)gridDim.x * 8 + blockIdx.x);
}

// Pair forces + per-atom half energies; with finish=1 also the
// velocity-Verlet finishStep (src/integrators.c:94-126) and its reductions.
template <int CAT>
__global__ void __launch_bounds__(128) k_force(Geo g, int group, int finish, double dt)
{
    __shared__ SmemPot sp;
    load_pot(g, sp);
    Dyn *dyn = g.dyn;
    const int n = dyn->n;
    const Side S = g.side[dyn->cur];
    const int cap = g.cap;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    // pe, m v^2, m v (3), count
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (i < n)
    {
        const int ki = S.kind[i];
        const bool active = (group < 0 || S.group[i] == group);
        double f[3] = {0.0, 0.0, 0.0};
        double pe = 0.0;
        if (active)
        {
            const double xi[3] = {S.x[i], S.x[cap + i], S.x[2 * cap + i]};
            const double fpi = (CAT == CAT_EAM || CAT == CAT_HYBRID) ? g.vaream[i] : 0.0;
            for_each_neighbour(g, S, i, S.cell_of[i], [&](int j, double sx, double sy, double sz) {
                if (group >= 0 && S.group[j] != group) return;
                const int kj = S.kind[j];
                const fmdg_pair_t &pp = sp.pairs[ki * g.nkinds + kj];
                const int cat = (CAT == CAT_HYBRID) ? pp.cat : CAT;
                const PairGeom p = pair_geom(xi, S, cap, j, sx, sy, sz);
                if (cat == FMDG_POT_LJ)
                {
                    if (p.r2 < pp.p[2])
                    {
                        const double inv_r2 = 1.0 / p.r2;
                        const double inv_rs2 = pp.p[1] * inv_r2;
                        const double inv_rs6 = inv_rs2 * inv_rs2 * inv_rs2;
                        const double inv_rs12 = inv_rs6 * inv_rs6;
                        const double factor = 12.0 * pp.p[0] * inv_r2 * (inv_rs12 - 0.5 * inv_rs6);
                        for (int d = 0; d < 3; d++) f[d] += p.rv[d] * factor;
                        pe += 0.5 * (pp.p[0] * (inv_rs12 - inv_rs6));
                    }
                }
                else if (cat == FMDG_POT_MORSE)
                {
                    if (p.r2 < pp.p[3])
                    {
                        const double r = sqrt(p.r2);
                        const double inv_r = 1.0 / r;
                        const double e1 = exp(-pp.p[1] * (r - pp.p[2]));
                        const double e2 = e1 * e1;
                        const double factor = 2.0 * pp.p[1] * pp.p[0] * inv_r * (e2 - e1);
                        for (int d = 0; d < 3; d++) f[d] += factor * p.rv[d];
                        pe += 0.5 * (pp.p[0] * (e2 - 2.0 * e1));
                    }
                }
                else if (cat == FMDG_POT_EAM)
                {
                    if (p.r2 < pp.p[2])
                    {
                        const double h = g.dr2;
                        const int ir2 = min((int)(p.r2 / h), g.Nr2 - 2);
                        const double a = (ir2 + 1) - p.r2 / h;
                        const double b = 1 - a;
                        const int ei = pp.iloc, ej = pp.jloc;
                        const size_t Nr2 = g.Nr2;
                        const double *ph = g.ephi + ((size_t)ei * g.nelem + ej) * Nr2;
                        const double *phdd = g.ephiDD + ((size_t)ei * g.nelem + ej) * Nr2;
                        const double phi_d = spl_der(ph, phdd, ir2, a, b, h);
                        const double rho_ip = spl_der(g.erho + ei * Nr2, g.erhoDD + ei * Nr2, ir2, a, b, h);
                        const double rho_jp = (ei == ej) ? rho_ip
                                            : spl_der(g.erho + ej * Nr2, g.erhoDD + ej * Nr2, ir2, a, b, h);
                        const double mag = 2 * (fpi * rho_jp + g.vaream[j] * rho_ip + phi_d);
                        for (int d = 0; d < 3; d++) f[d] -= mag * p.rv[d];
                        pe += 0.5 * spl_val(ph, phdd, ir2, a, b, h);
                    }
                }
            });
        }
        for (int d = 0; d < 3; d++) g.F[d * cap + i] = f[d];
        acc[0] = pe;
        if (active)
        {
            const double m = sp.mass[ki];
            double v[3] = {S.v[i], S.v[cap + i], S.v[2 * cap + i]};
            if (finish)
            {
                const double coef = __ddiv_rn(__dmul_rn(dt, 0.5), m);
                for (int d = 0; d < 3; d++)
                {
                    v[d] = __dadd_rn(v[d], __dmul_rn(coef, f[d]));
                    S.v[d * cap + i] = v[d];
                }
            }
            acc[1] = m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            acc[2] = m * v[0];
            acc[3] = m * v[1];
            acc[4] = m * v[2];
            acc[5] = 1.0;
        }
    }
    double tmp[6];
    for (int k = 0; k < 6; k++) tmp[k] = acc[k];
    __shared__ double blk[6];
    block_reduce_store<6>(tmp, blk);
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; k++) g.partials[(size_t)k * gridDim.x + blockIdx.x] = blk[k];
}

// Thermodynamics of the active group from the current velocities
// (src/matter.c:31-68); no energy term.
__global__ void __launch_bounds__(128) k_thermo(Geo g, int group)
{
    Dyn *dyn = g.dyn;
    const int n = dyn->n;
    const Side S = g.side[dyn->cur];
    const int cap = g.cap;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (i < n && (group < 0 || S.group[i] == group))
    {
        const double m = g.mass[S.kind[i]];
        const double v[3] = {S.v[i], S.v[cap + i], S.v[2 * cap + i]};
        acc[1] = m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        acc[2] = m * v[0];
        acc[3] = m * v[1];
        acc[4] = m * v[2];
        acc[5] = 1.0;
    }
    __shared__ double blk[6];
    block_reduce_store<6>(acc, blk);
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; k++) g.partials[(size_t)k * gridDim.x + blockIdx.x] = blk[k];
}

// Second level: sums the per-block partials in a fixed order, writes the
// thermo record (src/integrators.c:78-92) and, when a Berendsen thermostat
// is active, the velocity scale of the next start step
// (src/integrators.c:44-50): lambda = sqrt(1 + dt/tau * (T0/T - 1)).
__global__ void k_reduce_final(Geo g, int nblocks, int keep_pe, int with_emb, int thermostat,
                               double dt, double tau, double T0)
{
    __shared__ double red[256][7];
    const int t = threadIdx.x;
    double s[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int b = t; b < nblocks; b += blockDim.x)
    {
        for (int k = 0; k < 6; k++) s[k] += g.partials[(size_t)k * nblocks + b];
        if (with_emb) s[6] += g.partials[(size_t)nblocks * 8 + b];
    }
    for (int k = 0; k < 7; k++) red[t][k] = s[k];
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1)
    {
        if (t < off)
            for (int k = 0; k < 7; k++) red[t][k] += red[t + off][k];
        __syncthreads();
    }
    if (t == 0)
    {
        fmdg_thermo_t *th = g.thermo;
        const double mv2 = red[0][1];
        const double N = red[0][5];
        th->kinetic = 0.5 * mv2;
        th->temperature = mv2 / (3.0 * N * K_BOLTZMANN_D);
        th->momentum[0] = red[0][2];
        th->momentum[1] = red[0][3];
        th->momentum[2] = red[0][4];
        th->count = N;
        if (!keep_pe) th->potential = red[0][0] + red[0][6];
        if (thermostat)
            g.dyn->lambda = sqrt(1 + dt / tau * (T0 / th->temperature - 1));
    }
}

} // namespace

int fmdg_force_blocks(const fmdg_sys_t *s) { return fmdg_grid(s->g.cap > 0 ? s->g.cap : 1, 128); }

int fmdg_launch_density(fmdg_sys_t *s, int group)
{
    const bool eam = (s->cats & (1 << FMDG_POT_EAM)) != 0;
    if (!eam) return FMDG_OK;
    const int nb = fmdg_force_blocks(s);
    const int ncat = __builtin_popcount(s->cats);
    if (ncat > 1) k_density<true><<<nb, 128, 0, s->stream>>>(s->g, group);
    else k_density<false><<<nb, 128, 0, s->stream>>>(s->g, group);
    s->launches++;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

int fmdg_launch_pair_forces(fmdg_sys_t *s, int group, int finish, double dt)
{
    Geo &g = s->g;
    const int nb = fmdg_force_blocks(s);
    cudaStream_t st = s->stream;
    const int ncat = __builtin_popcount(s->cats);
    if (ncat > 1) k_force<CAT_HYBRID><<<nb, 128, 0, st>>>(g, group, finish, dt);
    else if (s->cats == (1 << FMDG_POT_LJ)) k_force<CAT_LJ><<<nb, 128, 0, st>>>(g, group, finish, dt);
    else if (s->cats == (1 << FMDG_POT_MORSE)) k_force<CAT_MORSE><<<nb, 128, 0, st>>>(g, group, finish, dt);
    else k_force<CAT_EAM><<<nb, 128, 0, st>>>(g, group, finish, dt);
    s->launches++;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

int fmdg_launch_forces(fmdg_sys_t *s, int group, int finish, double dt)
{
    int rc = fmdg_launch_density(s, group);
    if (rc) return rc;
    return fmdg_launch_pair_forces(s, group, finish, dt);
}

// thermo-only reduction (no force evaluation); keeps the potential energy
int fmdg_launch_thermo(fmdg_sys_t *s, int group, int thermostat, double dt, double tau, double T0)
{
    Geo &g = s->g;
    const int nb = fmdg_force_blocks(s);
    k_thermo<<<nb, 128, 0, s->stream>>>(g, group);
    k_reduce_final<<<1, 256, 0, s->stream>>>(g, nb, 1, 0, thermostat, dt, tau, T0);
    s->launches += 2;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

int fmdg_launch_reduce(fmdg_sys_t *s, int thermostat, double dt, double tau, double T0)
{
    Geo &g = s->g;
    const int nb = fmdg_force_blocks(s);
    const bool eam = (s->cats & (1 << FMDG_POT_EAM)) != 0;
    k_reduce_final<<<1, 256, 0, s->stream>>>(g, nb, 0, eam ? 1 : 0, thermostat, dt, tau, T0);
    s->launches++;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}
