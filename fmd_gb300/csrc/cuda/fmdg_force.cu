// Neighbour list, pair-force, EAM density/embedding and reduction kernels.
//
// Reference loops replaced (FMD 0.4.0):
//   LJ    src/lj.c:28-90    with the pair update of src/lj.h:26-58
//   Morse src/morse.c:30-92 with the pair update of src/morse.h:26-58
//   EAM   src/eam.c:225-322 (density, pass 1), src/eam.c:160-223 (embedding
//         F(rho), F'(rho)), src/eam.c:29-146 (forces, pass 0), pair updates
//         src/eam.h:29-406, cubic spline src/cspline.h:26-27
//   hybrid src/forces.c:33-290 (per-pair category switch)
//   ghost images and the partial-force fold-back src/md-ghost.c:711-825,
//   the PE Allreduce src/lj.c:89: replaced by periodic image shifts inside
//   the loops and a deterministic two-level block reduction.
//
// Work decomposition.  The reference visits each pair once (half shell,
// Newton's third law, scattering into both atoms).  Here one thread owns
// one atom and gathers over all its neighbours: every pair is evaluated
// from both sides, there are no atomics and results are deterministic; each
// atom's energy takes half of each pair term.
//
// Per step, after the refresh:
//   k_prep_local  cell-local binary32 coordinates of every atom (float4)
//   k_nlist       27-cell stencil scan in binary32 against the largest
//                 cutoff plus a margin; stores (j, stencil offset) per atom
//   k_density     EAM pass 1 + embedding over the list
//   k_force       pair forces over the list + velocity-Verlet finish step
// An atom with more candidates than the list holds falls back to scanning
// the stencil directly, so the list size is a performance knob only.
//
// Precision modes.  FMDG_PREC_FP64: every pair quantity in binary64, the
// binary32 list only prunes (its margin keeps every pair within the cutoff).
// FMDG_PREC_MIXED: pair geometry from the binary32 cell-local coordinates,
// pair/spline/embedding arithmetic in binary32, forces and energies summed
// in binary64 (binary32 partial sums of at most 8 pair terms are added to
// binary64 accumulators).  Pairs within 1e-4 relative of a cutoff are
// re-tested in binary64 so both modes include exactly the same pairs.
#include "fmdg_internal.cuh"

namespace {

enum { CAT_LJ = 1, CAT_EAM = 2, CAT_MORSE = 3, CAT_HYBRID = 4 };

struct SmemPot
{
    fmdg_pair_t pairs[FMDG_MAXK * FMDG_MAXK];
    float pf[FMDG_MAXK * FMDG_MAXK][4];
    double mass[FMDG_MAXK];
    int elem[FMDG_MAXK];
    float4 off[27];     // image offset of stencil code c: (ox, oy, oz) * cellh (binary32)
};

__device__ __forceinline__ void load_pot(const Geo &g, SmemPot &sp)
{
    const int nk2 = g.nkinds * g.nkinds;
    for (int k = threadIdx.x; k < nk2; k += blockDim.x)
    {
        sp.pairs[k] = g.pairs[k];
        for (int q = 0; q < 4; q++) sp.pf[k][q] = (float)g.pairs[k].p[q];
    }
    for (int k = threadIdx.x; k < g.nkinds; k += blockDim.x)
    {
        sp.mass[k] = g.mass[k];
        sp.elem[k] = g.eam_elem[k];
    }
    for (int c = threadIdx.x; c < 27; c += blockDim.x)
        sp.off[c] = make_float4((float)(c / 9 - 1) * g.cellh_f[0], (float)((c / 3) % 3 - 1) * g.cellh_f[1],
                                (float)(c % 3 - 1) * g.cellh_f[2], 0.f);
    __syncthreads();
}

// stencil offset code: (ox+1)*9 + (oy+1)*3 + (oz+1); 13 is the cell itself
__device__ __forceinline__ int off_x(int code) { return code / 9 - 1; }
__device__ __forceinline__ int off_y(int code) { return (code / 3) % 3 - 1; }
__device__ __forceinline__ int off_z(int code) { return code % 3 - 1; }

struct CellXYZ { int x, y, z; };

__device__ __forceinline__ CellXYZ cell_xyz(const Geo &g, int c)
{
    CellXYZ r;
    r.x = c / (g.nc[1] * g.nc[2]);
    r.y = (c / g.nc[2]) % g.nc[1];
    r.z = c % g.nc[2];
    return r;
}

// Neighbour cell index along one axis for home coordinate h and offset o;
// -1 when the neighbour is outside an open face.  *shift is the image
// translation of src/md-ghost.c:85-107 (ghost copy of the far layer).
__device__ __forceinline__ int nb_axis(const Geo &g, int d, int h, int o, double *shift)
{
    int j = h + o;
    *shift = 0.0;
    if (j < 0)
    {
        if (!g.pbc[d]) return -1;
        j += g.nc[d];
        *shift = -g.l[d];
    }
    else if (j >= g.nc[d])
    {
        if (!g.pbc[d]) return -1;
        j -= g.nc[d];
        *shift = g.l[d];
    }
    return j;
}

// Every (j, stencil code) of the 27-cell stencil of cell c except i itself.
template <typename F>
__device__ __forceinline__ void scan_stencil(const Geo &g, const Side &S, int i, CellXYZ ci, F &&f)
{
    for (int code = 0; code < 27; code++)
    {
        double sx, sy, sz;
        const int jx = nb_axis(g, 0, ci.x, off_x(code), &sx);
        const int jy = nb_axis(g, 1, ci.y, off_y(code), &sy);
        const int jz = nb_axis(g, 2, ci.z, off_z(code), &sz);
        if (jx < 0 || jy < 0 || jz < 0) continue;
        const int nb = jz + g.nc[2] * (jy + g.nc[1] * jx);
        const int jb = S.cell_start[nb], je = S.cell_start[nb + 1];
        for (int j = jb; j < je; j++)
        {
            if (code == 13 && j == i) continue;
            f(j, code);
        }
    }
}

// list walk with stencil fallback; UNROLL: four entries per round, their
// index and coordinate loads independent and in flight together (the walk
// is latency bound; pays where registers do not limit occupancy further)
template <bool UNROLL, typename F>
__device__ __forceinline__ void for_each_pair(const Geo &g, const Side &S, int i, CellXYZ ci, F &&f)
{
    const int cnt = g.nbr_count[i];
    if (cnt <= g.maxnb)
    {
        const int cap = g.cap;
        const int *col = g.nbr + i;
        int k = 0;
        if (UNROLL)
            for (; k + 4 <= cnt; k += 4)
            {
                const int e0 = __ldg(col + (size_t)k * cap), e1 = __ldg(col + (size_t)(k + 1) * cap);
                const int e2 = __ldg(col + (size_t)(k + 2) * cap), e3 = __ldg(col + (size_t)(k + 3) * cap);
                f(e0 & 0x3ffffff, e0 >> 26);
                f(e1 & 0x3ffffff, e1 >> 26);
                f(e2 & 0x3ffffff, e2 >> 26);
                f(e3 & 0x3ffffff, e3 >> 26);
            }
        for (; k < cnt; k++)
        {
            const int e = __ldg(col + (size_t)k * cap);
            f(e & 0x3ffffff, e >> 26);
        }
    }
    else
        scan_stencil(g, S, i, ci, f);
}

// binary64 pair geometry: rv = x_i - (x_j + image shift), r2 summed without
// fused multiply-adds as the reference does (src/forces.h:25-34)
struct Geom64 { double rv[3]; double r2; };

__device__ __forceinline__ Geom64 geom64(const Geo &g, const Side &S, const double xi[3], CellXYZ ci, int j, int code)
{
    Geom64 p;
    const int cap = g.cap;
    const int h[3] = {ci.x, ci.y, ci.z};
    const int o[3] = {off_x(code), off_y(code), off_z(code)};
    for (int d = 0; d < 3; d++)
    {
        double s;
        nb_axis(g, d, h[d], o[d], &s);
        double x2 = S.x[(size_t)d * cap + j];
        if (s != 0.0) x2 = __dadd_rn(x2, s);
        p.rv[d] = __dsub_rn(xi[d], x2);
    }
    p.r2 = __dadd_rn(__dadd_rn(__dmul_rn(p.rv[0], p.rv[0]), __dmul_rn(p.rv[1], p.rv[1])),
                     __dmul_rn(p.rv[2], p.rv[2]));
    return p;
}

// binary32 pair geometry from cell-local coordinates
__device__ __forceinline__ float3 geom32(const SmemPot &sp, float4 xi, float4 xj, int code)
{
    const float4 o = sp.off[code];
    return make_float3(xi.x - xj.x - o.x, xi.y - xj.y - o.y, xi.z - xj.z - o.z);
}

// interval index k = floor(q) (clamped to kmax) and fraction b = q - k of a
// binary32 table coordinate 0 <= q < 2^23, without conversion instructions:
// adding 2^23 rounding towards minus infinity leaves floor(q) in the
// significand
__device__ __forceinline__ int table_index(float q, float kmax, float &b)
{
    const float fl = fminf(__fadd_rd(q, 8388608.f) - 8388608.f, kmax);
    b = q - fl;
    return __float_as_int(fl + 8388608.f) - 0x4B000000;
}

// natural cubic spline on a uniform grid (src/cspline.h:26-27) as a cubic
// in the fraction b of interval k: t = {k0, k1, k2, k3}
__device__ __forceinline__ double spl_val(double4_32a t, double b)
{
    return ((t.w * b + t.z) * b + t.y) * b + t.x;
}
__device__ __forceinline__ double spl_der(double4_32a t, double b, double inv_h)
{
    return ((3.0 * t.w * b + 2.0 * t.z) * b + t.y) * inv_h;
}
__device__ __forceinline__ float spl_val(float4 t, float b)
{
    return ((t.w * b + t.z) * b + t.y) * b + t.x;
}
__device__ __forceinline__ float spl_der(float4 t, float b, float inv_h)
{
    return ((3.f * t.w * b + 2.f * t.z) * b + t.y) * inv_h;
}

// is r2 (binary32) within rc2?  Near the cutoff the decision is taken in
// binary64 from the absolute positions, as the reference does.
__device__ __forceinline__ bool within_cut32(const Geo &g, const Side &S, int i, CellXYZ ci, int j, int code,
                                             float r2f, float rc2f, double rc2)
{
    if (fabsf(r2f - rc2f) > 1e-4f * rc2f) return r2f < rc2f;
    const int cap = g.cap;
    const double xi[3] = {S.x[i], S.x[cap + i], S.x[2 * (size_t)cap + i]};
    return geom64(g, S, xi, ci, j, code).r2 < rc2;
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

// binary32 partial sums flushed into binary64 every 8 terms
template <int NV>
struct Acc32
{
    float part[NV];
    double sum[NV];
    int n;
    __device__ __forceinline__ Acc32() : n(0)
    {
        for (int k = 0; k < NV; k++) { part[k] = 0.f; sum[k] = 0.0; }
    }
    __device__ __forceinline__ void tick()
    {
        if (++n == 8) flush();
    }
    __device__ __forceinline__ void flush()
    {
        for (int k = 0; k < NV; k++) { sum[k] += (double)part[k]; part[k] = 0.f; }
        n = 0;
    }
};

// ---------------------------------------------------------------- kernels

template <class L>
__global__ void k_prep_local(__grid_constant__ const L loc)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    const Dyn *dyn = g.dyn;
    const int i = bx * blockDim.x + threadIdx.x;
    if (i >= dyn->n) return;
    const Side S = g.side[dyn->cur];
    const CellXYZ c = cell_xyz(g, S.cell_of[i]);
    const int cap = g.cap;
    const float lx = (float)(S.x[i] - c.x * g.cellh[0]);
    const float ly = (float)(S.x[cap + i] - c.y * g.cellh[1]);
    const float lz = (float)(S.x[2 * (size_t)cap + i] - c.z * g.cellh[2]);
    g.xf4[i] = make_float4(lx, ly, lz, __int_as_float((int)S.kind[i]));
}

template <class L>
__global__ void __launch_bounds__(L::max_threads, L::min_blocks) k_nlist(__grid_constant__ const L loc)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    const Dyn *dyn = g.dyn;
    const int i = bx * blockDim.x + threadIdx.x;
    if (i >= dyn->n) return;
    const Side S = g.side[dyn->cur];
    const CellXYZ ci = cell_xyz(g, S.cell_of[i]);
    const float4 xi = g.xf4[i];
    const int cap = g.cap, maxnb = g.maxnb;
    const float rl2 = g.rlist2;
    int cnt = 0;
    for (int code = 0; code < 27; code++)
    {
        double sdummy;
        const int jx = nb_axis(g, 0, ci.x, off_x(code), &sdummy);
        const int jy = nb_axis(g, 1, ci.y, off_y(code), &sdummy);
        const int jz = nb_axis(g, 2, ci.z, off_z(code), &sdummy);
        if (jx < 0 || jy < 0 || jz < 0) continue;
        const int c = jz + g.nc[2] * (jy + g.nc[1] * jx);
        const int jb = S.cell_start[c], je = S.cell_start[c + 1];
        // i's position in the neighbour cell's frame
        const float qx = xi.x - (float)off_x(code) * g.cellh_f[0];
        const float qy = xi.y - (float)off_y(code) * g.cellh_f[1];
        const float qz = xi.z - (float)off_z(code) * g.cellh_f[2];
        const int tag = code << 26;
        auto test = [&](int j, float4 xj) {
            const float dx = qx - xj.x, dy = qy - xj.y, dz = qz - xj.z;
            if (dx * dx + dy * dy + dz * dz < rl2)
            {
                if (cnt < maxnb) g.nbr[(size_t)cnt * cap + i] = j | tag;
                cnt++;
            }
        };
        int j = jb;
        if (code != 13)
        {
            // four candidates per round, their loads in flight together
            for (; j + 4 <= je; j += 4)
            {
                const float4 a0 = __ldg(g.xf4 + j), a1 = __ldg(g.xf4 + j + 1);
                const float4 a2 = __ldg(g.xf4 + j + 2), a3 = __ldg(g.xf4 + j + 3);
                test(j, a0);
                test(j + 1, a1);
                test(j + 2, a2);
                test(j + 3, a3);
            }
        }
        for (; j < je; j++)
            if (j != i) test(j, __ldg(g.xf4 + j));
    }
    g.nbr_count[i] = cnt;
}

// EAM pass 1 + embedding: rho_i = sum_j f_{elem(j)}(r_ij^2) (src/eam.h:270-406),
// vaream_i = F'(rho_i), energy F(rho_i) (src/eam.c:160-179).
template <class L, bool MIXED, bool HYBRID>
__global__ void __launch_bounds__(L::max_threads, L::min_blocks) k_density(__grid_constant__ const L loc)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    const int group = g.st.group;
    __shared__ SmemPot sp;
    load_pot(g, sp);
    Dyn *dyn = g.dyn;
    const int n = dyn->n;
    const Side S = g.side[dyn->cur];
    const int cap = g.cap;
    const int i = bx * blockDim.x + threadIdx.x;
    double acc[1] = {0.0};
    if (i < n)
    {
        const int ki = S.kind[i];
        const int ei = sp.elem[ki];
        const bool active = (group < 0 || S.group[i] == group) && (!HYBRID || ei >= 0);
        double rho = 0.0;
        if (active)
        {
            const CellXYZ ci = cell_xyz(g, S.cell_of[i]);
            const int nk = g.nkinds;
            const int nint = g.Nr2 - 1;
            if (!MIXED)
            {
                const double xi[3] = {S.x[i], S.x[cap + i], S.x[2 * (size_t)cap + i]};
                const double inv_h = g.inv_dr2;
                for_each_pair<L::unroll>(g, S, i, ci, [&](int j, int code) {
                    if (group >= 0 && S.group[j] != group) return;
                    const fmdg_pair_t &pp = sp.pairs[ki * nk + S.kind[j]];
                    if (HYBRID && pp.cat != FMDG_POT_EAM) return;
                    const Geom64 p = geom64(g, S, xi, ci, j, code);
                    if (p.r2 < pp.p[2])
                    {
                        const double q = p.r2 * inv_h;
                        const int ir2 = min((int)q, nint - 1);
                        rho += spl_val(g.pk_rho[(size_t)pp.jloc * nint + ir2], q - ir2);
                    }
                });
            }
            else
            {
                const float4 xi = g.xf4[i];
                const float inv_h = (float)g.inv_dr2;
                const float kmax = (float)(nint - 1);
                Acc32<1> ac;
                for_each_pair<L::unroll>(g, S, i, ci, [&](int j, int code) {
                    if (group >= 0 && S.group[j] != group) return;
                    const float4 xj = g.xf4[j];
                    const int kj = __float_as_int(xj.w);
                    const fmdg_pair_t &pp = sp.pairs[ki * nk + kj];
                    if (HYBRID && pp.cat != FMDG_POT_EAM) return;
                    const float3 rv = geom32(sp, xi, xj, code);
                    const float r2 = rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
                    if (within_cut32(g, S, i, ci, j, code, r2, sp.pf[ki * nk + kj][2], pp.p[2]))
                    {
                        float b;
                        const int ir2 = table_index(r2 * inv_h, kmax, b);
                        ac.part[0] += spl_val(g.pkf_rho[(size_t)pp.jloc * nint + ir2], b);
                        ac.tick();
                    }
                });
                ac.flush();
                rho = ac.sum[0];
            }
            // embedding (src/eam.c:160-179)
            const double qr = rho * g.inv_drho;
            int irho = (int)qr;
            if (irho >= g.Nrho - 1 || irho < 0)
            {
                atomic_or_err(dyn, FMDG_ERRBIT_RHO_RANGE);
                irho = irho < 0 ? 0 : g.Nrho - 2;
            }
            const int nrint = g.Nrho - 1;
            if (!MIXED)
            {
                const double b = qr - irho;
                const double4_32a t = g.pk_F[(size_t)ei * nrint + irho];
                g.vaream[i] = spl_der(t, b, g.inv_drho);
                acc[0] = spl_val(t, b);
            }
            else
            {
                const float b = (float)(qr - irho);
                const float4 t = g.pkf_F[(size_t)ei * nrint + irho];
                const float fp = spl_der(t, b, (float)g.inv_drho);
                g.vaream[i] = (double)fp;
                g.fpf[i] = fp;
                acc[0] = (double)spl_val(t, b);
            }
        }
        else
        {
            g.vaream[i] = 0.0;
            if (MIXED) g.fpf[i] = 0.f;
        }
    }
    block_reduce_store<1>(acc, g.partials + (size_t)nb * 8 + bx);
}

// Second level: sums the per-block partials in a fixed order, writes the
// thermo record (src/integrators.c:78-92) and, when a Berendsen thermostat
// is active, the velocity scale of the next start step
// (src/integrators.c:44-50): lambda = sqrt(1 + dt/tau * (T0/T - 1)).
// Run by one whole block of at most 256 threads.
__device__ void final_reduce(const Geo &g, int nblocks, int keep_pe, int with_emb, int thermostat,
                             double dt, double tau, double T0)
{
    __shared__ double red[8][7];
    const int t = threadIdx.x;
    double s[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int b = t; b < nblocks; b += blockDim.x)
    {
        for (int k = 0; k < 6; k++) s[k] += __ldcg(&g.partials[(size_t)k * nblocks + b]);
        if (with_emb) s[6] += __ldcg(&g.partials[(size_t)nblocks * 8 + b]);
    }
    for (int k = 0; k < 7; k++)
        for (int off = 16; off > 0; off >>= 1) s[k] += __shfl_down_sync(0xffffffffu, s[k], off);
    if ((t & 31) == 0)
        for (int k = 0; k < 7; k++) red[t >> 5][k] = s[k];
    __syncthreads();
    if (t == 0)
    {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++)
            for (int k = 0; k < 7; k++) red[0][k] += red[w][k];
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

__global__ void k_reduce_final(Geo g, int nblocks, int keep_pe, int with_emb, int thermostat,
                               double dt, double tau, double T0)
{
    final_reduce(g, nblocks, keep_pe, with_emb, thermostat, dt, tau, T0);
}

// Pair forces + per-atom half energies; with finish=1 also the
// velocity-Verlet finishStep (src/integrators.c:94-126) and its reductions.
template <class L, int CAT, bool MIXED>
__global__ void __launch_bounds__(L::max_threads, L::min_blocks) k_force(__grid_constant__ const L loc, int finish)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    const int group = g.st.group;
    const double dt = g.st.dt;
    __shared__ SmemPot sp;
    load_pot(g, sp);
    Dyn *dyn = g.dyn;
    const int n = dyn->n;
    const Side S = g.side[dyn->cur];
    const int cap = g.cap;
    const int i = bx * blockDim.x + threadIdx.x;
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
            const CellXYZ ci = cell_xyz(g, S.cell_of[i]);
            const int nk = g.nkinds;
            const int nint = g.Nr2 - 1;
            const size_t ne = g.nelem;
            if (!MIXED)
            {
                const double xi[3] = {S.x[i], S.x[cap + i], S.x[2 * (size_t)cap + i]};
                const double fpi = (CAT == CAT_EAM || CAT == CAT_HYBRID) ? g.vaream[i] : 0.0;
                const double inv_h = g.inv_dr2;
                for_each_pair<L::unroll>(g, S, i, ci, [&](int j, int code) {
                    if (group >= 0 && S.group[j] != group) return;
                    const fmdg_pair_t &pp = sp.pairs[ki * nk + S.kind[j]];
                    const int cat = (CAT == CAT_HYBRID) ? pp.cat : CAT;
                    const Geom64 p = geom64(g, S, xi, ci, j, code);
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
                            const double q = p.r2 * inv_h;
                            const int ir2 = min((int)q, nint - 1);
                            const double b = q - ir2;
                            const int ei = pp.iloc, ej = pp.jloc;
                            const double4_32a tph = g.pk_phi[((size_t)ei * ne + ej) * nint + ir2];
                            const double phi_d = spl_der(tph, b, inv_h);
                            const double rho_ip = spl_der(g.pk_rho[(size_t)ei * nint + ir2], b, inv_h);
                            const double rho_jp = (ei == ej) ? rho_ip
                                                : spl_der(g.pk_rho[(size_t)ej * nint + ir2], b, inv_h);
                            const double mag = 2 * (fpi * rho_jp + g.vaream[j] * rho_ip + phi_d);
                            for (int d = 0; d < 3; d++) f[d] -= mag * p.rv[d];
                            pe += 0.5 * spl_val(tph, b);
                        }
                    }
                });
            }
            else
            {
                const float4 xi = g.xf4[i];
                const float fpi = (CAT == CAT_EAM || CAT == CAT_HYBRID) ? g.fpf[i] : 0.f;
                const float inv_h = (float)g.inv_dr2;
                const float kmax = (float)(nint - 1);
                Acc32<4> ac;
                for_each_pair<L::unroll>(g, S, i, ci, [&](int j, int code) {
                    if (group >= 0 && S.group[j] != group) return;
                    const float4 xj = g.xf4[j];
                    const int kj = __float_as_int(xj.w);
                    const int pidx = ki * nk + kj;
                    const fmdg_pair_t &pp = sp.pairs[pidx];
                    const int cat = (CAT == CAT_HYBRID) ? pp.cat : CAT;
                    const float3 rv = geom32(sp, xi, xj, code);
                    const float r2 = rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
                    if (cat == FMDG_POT_LJ)
                    {
                        if (within_cut32(g, S, i, ci, j, code, r2, sp.pf[pidx][2], pp.p[2]))
                        {
                            const float inv_r2 = __fdividef(1.f, r2);
                            const float inv_rs2 = sp.pf[pidx][1] * inv_r2;
                            const float inv_rs6 = inv_rs2 * inv_rs2 * inv_rs2;
                            const float inv_rs12 = inv_rs6 * inv_rs6;
                            const float eps4 = sp.pf[pidx][0];
                            const float factor = 12.f * eps4 * inv_r2 * (inv_rs12 - 0.5f * inv_rs6);
                            ac.part[0] += rv.x * factor;
                            ac.part[1] += rv.y * factor;
                            ac.part[2] += rv.z * factor;
                            ac.part[3] += 0.5f * (eps4 * (inv_rs12 - inv_rs6));
                            ac.tick();
                        }
                    }
                    else if (cat == FMDG_POT_MORSE)
                    {
                        if (within_cut32(g, S, i, ci, j, code, r2, sp.pf[pidx][3], pp.p[3]))
                        {
                            const float D0 = sp.pf[pidx][0], al = sp.pf[pidx][1], r0 = sp.pf[pidx][2];
                            const float inv_r = rsqrtf(r2);
                            const float r = r2 * inv_r;
                            const float e1 = expf(-al * (r - r0));
                            const float e2 = e1 * e1;
                            const float factor = 2.f * al * D0 * inv_r * (e2 - e1);
                            ac.part[0] += factor * rv.x;
                            ac.part[1] += factor * rv.y;
                            ac.part[2] += factor * rv.z;
                            ac.part[3] += 0.5f * (D0 * (e2 - 2.f * e1));
                            ac.tick();
                        }
                    }
                    else if (cat == FMDG_POT_EAM)
                    {
                        if (within_cut32(g, S, i, ci, j, code, r2, sp.pf[pidx][2], pp.p[2]))
                        {
                            float b;
                            const int ir2 = table_index(r2 * inv_h, kmax, b);
                            const int ei = pp.iloc, ej = pp.jloc;
                            const float4 tph = g.pkf_phi[((size_t)ei * ne + ej) * nint + ir2];
                            const float phi_d = spl_der(tph, b, inv_h);
                            const float rho_ip = spl_der(g.pkf_rho[(size_t)ei * nint + ir2], b, inv_h);
                            const float rho_jp = (ei == ej) ? rho_ip
                                               : spl_der(g.pkf_rho[(size_t)ej * nint + ir2], b, inv_h);
                            const float mag = 2.f * (fpi * rho_jp + g.fpf[j] * rho_ip + phi_d);
                            ac.part[0] -= mag * rv.x;
                            ac.part[1] -= mag * rv.y;
                            ac.part[2] -= mag * rv.z;
                            ac.part[3] += 0.5f * spl_val(tph, b);
                            ac.tick();
                        }
                    }
                });
                ac.flush();
                for (int d = 0; d < 3; d++) f[d] = ac.sum[d];
                pe = ac.sum[3];
            }
        }
        if (active && g.ttm_on)
        {
            // TTM friction (src/forces.c:292-330, 1-D): F_z += xi m (v_z - vcm_z)
            const double time = dyn->time, hdt = dyn->dt / 2.0;
            if ((time >= g.ttm_start - hdt) && ((time < g.ttm_stop + hdt) || g.ttm_stop < g.ttm_start))
            {
                const double z = S.x[2 * (size_t)cap + i];
                const double q = z * g.ttm_inv_tcellh_z;
                const double r = rint(q);
                int it = (fabs(q - r) <= 1e-9 * fmax(1.0, fabs(q))) ? (int)__ddiv_rn(z, g.ttm_tcellh_z) : (int)q;
                it += g.ttm_g2l_z;
                if (it >= 0 && it < g.ttm_nz)
                {
                    const double m = sp.mass[ki];
                    f[2] += g.ttm_xi[it] * m * (S.v[2 * (size_t)cap + i] - g.ttm_vcm[3 * it + 2]);
                }
                else
                    atomic_or_err(dyn, FMDG_ERRBIT_TTM);
            }
        }
        for (int d = 0; d < 3; d++) g.F[(size_t)d * cap + i] = f[d];
        acc[0] = pe;
        if (active)
        {
            const double m = sp.mass[ki];
            double v[3] = {S.v[i], S.v[cap + i], S.v[2 * (size_t)cap + i]};
            if (finish)
            {
                const double coef = __ddiv_rn(__dmul_rn(dt, 0.5), m);
                for (int d = 0; d < 3; d++)
                {
                    v[d] = __dadd_rn(v[d], __dmul_rn(coef, f[d]));
                    S.v[(size_t)d * cap + i] = v[d];
                }
            }
            acc[1] = m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            acc[2] = m * v[0];
            acc[3] = m * v[1];
            acc[4] = m * v[2];
            acc[5] = 1.0;
        }
    }
    __shared__ double blk[6];
    __shared__ unsigned ticket;
    block_reduce_store<6>(acc, blk);
    if (threadIdx.x == 0)
    {
        for (int k = 0; k < 6; k++) g.partials[(size_t)k * nb + bx] = blk[k];
        __threadfence();
        ticket = atomicAdd(&g.dyn->blocks_done, 1u);
    }
    __syncthreads();
    // the last block to finish sums every block's partials in a fixed order
    if (ticket == (unsigned)nb - 1)
    {
        __threadfence();
        final_reduce(g, nb, 0, g.has_eam, g.st.thermostat, dt, g.st.tau, g.st.T0);
        if (threadIdx.x == 0)
        {
            g.dyn->blocks_done = 0;
            if (finish && g.dyn->steps_left > 0) g.dyn->steps_left--;
        }
    }
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
        const double v[3] = {S.v[i], S.v[cap + i], S.v[2 * (size_t)cap + i]};
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

} // namespace

int fmdg_force_blocks(const fmdg_sys_t *s) { return fmdg_grid(s->g.cap > 0 ? s->g.cap : 1, s->fblk); }

namespace {

template <class L>
void launch_nlist_t(const L &loc, int n_prep, int prep_threads, int nb, int blk, cudaStream_t st)
{
    k_prep_local<<<n_prep, prep_threads, 0, st>>>(loc);
    k_nlist<<<nb, blk, 0, st>>>(loc);
}

template <class L>
void launch_density_t(const L &loc, bool mixed, bool hyb, int nb, int blk, cudaStream_t st)
{
    if (mixed)
    {
        if (hyb) k_density<L, true, true><<<nb, blk, 0, st>>>(loc);
        else k_density<L, true, false><<<nb, blk, 0, st>>>(loc);
    }
    else
    {
        if (hyb) k_density<L, false, true><<<nb, blk, 0, st>>>(loc);
        else k_density<L, false, false><<<nb, blk, 0, st>>>(loc);
    }
}

template <class L, bool MIXED>
void launch_force_t(const L &loc, int cats, int finish, int nb, int blk, cudaStream_t st)
{
    const int ncat = __builtin_popcount(cats);
    if (ncat > 1) k_force<L, CAT_HYBRID, MIXED><<<nb, blk, 0, st>>>(loc, finish);
    else if (cats == (1 << FMDG_POT_LJ)) k_force<L, CAT_LJ, MIXED><<<nb, blk, 0, st>>>(loc, finish);
    else if (cats == (1 << FMDG_POT_MORSE)) k_force<L, CAT_MORSE, MIXED><<<nb, blk, 0, st>>>(loc, finish);
    else k_force<L, CAT_EAM, MIXED><<<nb, blk, 0, st>>>(loc, finish);
}

} // namespace

int fmdg_launch_nlist(fmdg_sys_t *s)
{
    launch_nlist_t(LocOne{s->g}, fmdg_grid(s->g.cap, 256), 256, fmdg_force_blocks(s), s->fblk, s->stream);
    s->launches += 2;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

int fmdg_launch_density(fmdg_sys_t *s, int group)
{
    const bool eam = (s->cats & (1 << FMDG_POT_EAM)) != 0;
    if (!eam) return FMDG_OK;
    s->g.st.group = group;
    launch_density_t(LocOne{s->g}, s->g.prec == FMDG_PREC_MIXED, __builtin_popcount(s->cats) > 1,
                     fmdg_force_blocks(s), s->fblk, s->stream);
    s->launches++;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

// pair forces; the kernel's last block also writes the thermo record
int fmdg_launch_pair_forces(fmdg_sys_t *s, int group, int finish, double dt, int thermostat, double tau,
                            double T0)
{
    StepArgs &a = s->g.st;
    a.group = group;
    a.dt = dt;
    a.thermostat = thermostat;
    a.tau = tau;
    a.T0 = T0;
    const LocOne L{s->g};
    const int nb = fmdg_force_blocks(s);
    if (s->g.prec == FMDG_PREC_MIXED) launch_force_t<LocOne, true>(L, s->cats, finish, nb, s->fblk, s->stream);
    else launch_force_t<LocOne, false>(L, s->cats, finish, nb, s->fblk, s->stream);
    s->launches++;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

int fmdg_launch_forces(fmdg_sys_t *s, int group, int finish, double dt, int thermostat, double tau, double T0)
{
    int rc = fmdg_launch_nlist(s);
    if (rc) return rc;
    if ((rc = fmdg_launch_density(s, group))) return rc;
    return fmdg_launch_pair_forces(s, group, finish, dt, thermostat, tau, T0);
}

// Neighbour lists, EAM density and pair forces + finish step for every
// system of a pack (one launch per kernel).
// phases: bit 0 neighbour lists, bit 1 EAM density, bit 2 pair forces +
// finish step (all three for a step).  Returns the kernels launched.
int fmdg_pack_launch_forces(const fmdg_pack_launch &P, int phases)
{
    cudaStream_t st = P.stream;
    const int nab = P.la.bstart[P.nsys], nfb = P.lf.bstart[P.nsys];
    int n = 0;
    if (phases & 1)
    {
        k_prep_local<<<nab, 128, 0, st>>>(P.la);
        k_nlist<<<nfb, P.fblk, 0, st>>>(P.lf);
        n += 2;
    }
    const int cats = 1 << P.cat;
    if ((phases & 2) && P.cat == FMDG_POT_EAM)
    {
        launch_density_t(P.lf, P.mixed != 0, false, nfb, P.fblk, st);
        n++;
    }
    if (phases & 4)
    {
        if (P.mixed) launch_force_t<LocPack, true>(P.lf, cats, 1, nfb, P.fblk, st);
        else launch_force_t<LocPack, false>(P.lf, cats, 1, nfb, P.fblk, st);
        n++;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return -fmdg_fail("pack forces", e);
    return n;
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
