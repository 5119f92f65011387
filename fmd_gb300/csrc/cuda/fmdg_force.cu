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
// These kernels serve single systems on the exact per-step list (binary64
// by default, and boxes too small for a skin list); packed systems and
// mixed-precision single systems use the skin-list kernels (fmdg_skin.cu).
//
// Precision modes.  FMDG_PREC_FP64: every pair quantity to binary64
// accuracy, the binary32 list only prunes (its margin keeps every pair
// within the cutoff).  LJ, Morse, EAM and hybrid pairs are evaluated in
// double-float arithmetic (fmdg_df.cuh: about 48 significant bits on the
// binary32 pipe, GB300's binary64 rate being 1/64 of it) from double-float
// cell-local coordinates, parameters and tables, with cutoff decisions
// within 1e-6 relative of the cutoff taken from the reference's binary64
// geometry.  FMDG_PREC_MIXED: pair geometry from the binary32 cell-local
// coordinates, pair/spline/embedding arithmetic in binary32, binary32
// partial sums of at most 8 pair terms accumulated as a TwoSum pair and
// converted to binary64 per atom.  Pairs within 1e-4 relative of a cutoff
// are re-tested in binary64 so both modes include exactly the same pairs.
#include "fmdg_pairs.cuh"

namespace {

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

// list walk with stencil fallback
template <typename F>
__device__ __forceinline__ void for_each_pair(const Geo &g, const Side &S, int i, CellXYZ ci, F &&f)
{
    const int cnt = g.nbr_count[i];
    if (cnt <= g.maxnb)
    {
        const int cap = g.cap;
        const int *col = g.nbr + i;
        for (int k = 0; k < cnt; k++)
        {
            const int e = __ldg(col + (size_t)k * cap);
            f(e & 0x3ffffff, e >> 26);
        }
    }
    else
        scan_stencil(g, S, i, ci, f);
}

// binary64 pair geometry of a stencil entry (Geom64, fmdg_pairs.cuh): the
// reference's ghost shift of the neighbour, then x_i minus it
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
template <bool DF>
__device__ __forceinline__ float3 geom32(const SmemPotT<DF> &sp, float4 xi, float4 xj, int code)
{
    // the offset's binary32 part, then its remainder (the binary32 rounding
    // of (ox, oy, oz) * cellh would shift every pair across a cell face by
    // up to half an ulp of the cell width)
    const float4 o = sp.off[code], ol = sp.offl[code];
    return make_float3(xi.x - xj.x - o.x - ol.x, xi.y - xj.y - o.y - ol.y, xi.z - xj.z - o.z - ol.z);
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

// binary64 cutoff decision from the double-float r^2: within 1e-6 relative
// of the cutoff it is taken from the reference's binary64 geometry
__device__ __forceinline__ bool within_cut_df(const Geo &g, const Side &S, int i, CellXYZ ci, int j, int code,
                                              dfl r2, float rc2f, double rc2)
{
    const float d = __fsub_rn(r2.hi, rc2f);
    if (fabsf(d) > 1e-6f * rc2f) return d < 0.f;
    const int cap = g.cap;
    const double xi[3] = {S.x[i], S.x[cap + i], S.x[2 * (size_t)cap + i]};
    return geom64(g, S, xi, ci, j, code).r2 < rc2;
}

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
    const double4_32a oc = g.corig[S.cell_of[i]];
    const int cap = g.cap;
    const double ux = S.x[i] - oc.x;
    const double uy = S.x[cap + i] - oc.y;
    const double uz = S.x[2 * (size_t)cap + i] - oc.z;
    const float lx = (float)ux, ly = (float)uy, lz = (float)uz;
    const float4 hi = make_float4(lx, ly, lz, __int_as_float((int)S.kind[i]));
    g.xf4[i] = hi;
    // binary64 mode: hi and the remainders side by side, the double-float
    // cell-local position in one 32-byte row
    if (g.prec == FMDG_PREC_FP64)
    {
        g.xdf[2 * (size_t)i] = hi;
        g.xdf[2 * (size_t)i + 1] =
            make_float4((float)(ux - (double)lx), (float)(uy - (double)ly), (float)(uz - (double)lz), 0.f);
    }
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
        // i's position in the neighbour cell's frame (offsets of -1, 0, 1
        // cell selected, not converted: conversions issue at the binary64
        // rate on GB300)
        auto shift = [](int o, float h) { return o == 0 ? 0.f : (o > 0 ? h : -h); };
        const float qx = xi.x - shift(off_x(code), g.cellh_f[0]);
        const float qy = xi.y - shift(off_y(code), g.cellh_f[1]);
        const float qz = xi.z - shift(off_z(code), g.cellh_f[2]);
        const int tag = code << 26;
        // branch-free: a warp's lanes hit at different candidates
        auto test = [&](int j, float4 xj) {
            const float dx = qx - xj.x, dy = qy - xj.y, dz = qz - xj.z;
            const bool hit = dx * dx + dy * dy + dz * dz < rl2;
            if (hit && cnt < maxnb) g.nbr[(size_t)cnt * cap + i] = j | tag;
            cnt += hit;
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
    __shared__ SmemPotT<!MIXED> sp;
    load_pot(g, sp);
    Dyn *dyn = g.dyn;
    const int n = dyn->n;
    const Side S = g.side[dyn->cur];
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
                // double-float pair arithmetic (fmdg_df.cuh)
                float4 ih, il;
                ld_row32(g.xdf + 2 * (size_t)i, ih, il);
                const dfl inv_h = df_of(df_split(g.inv_dr2));
                const float kmax = (float)(nint - 1);
                dfl acc_rho = {0.f, 0.f};
                for_each_pair(g, S, i, ci, [&](int j, int code) {
                    if (group >= 0 && S.group[j] != group) return;
                    float4 jh, jl;
                    ld_row32(g.xdf + 2 * (size_t)j, jh, jl);
                    const int pidx = ki * nk + __float_as_int(jh.w);
                    const fmdg_pair_t &pp = sp.pairs[pidx];
                    if (HYBRID && pp.cat != FMDG_POT_EAM) return;
                    const GeomDF p = geom_df(ih, il, jh, jl, sp.off[code], sp.offl[code]);
                    if (within_cut_df(g, S, i, ci, j, code, p.r2, sp.pf[pidx][2], pp.p[2]))
                        acc_rho = df_add(acc_rho, df_rho(g, pp, p, inv_h, kmax, nint));
                });
                rho = df_to_double(acc_rho);
            }
            else
            {
                const float4 xi = g.xf4[i];
                const float inv_h = (float)g.inv_dr2;
                const float kmax = (float)(nint - 1);
                Acc32<1> ac;
                for_each_pair(g, S, i, ci, [&](int j, int code) {
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
                    }
                    ac.tick();
                });
                ac.flush();
                rho = ac.total(0);
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
                const double fp = spl_der(t, b, g.inv_drho);
                g.vaream[i] = fp;
                g.fpdf[i] = df_split(fp);
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
            else g.fpdf[i] = make_float2(0.f, 0.f);
        }
    }
    block_reduce_store<1>(acc, g.partials + (size_t)nb * 8 + bx);
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
    __shared__ SmemPotT<!MIXED> sp;
    load_pot(g, sp);
    Dyn *dyn = g.dyn;
    const int n = dyn->n;
    const Side S = g.side[dyn->cur];
    const int cap = g.cap;
    const int i = bx * blockDim.x + threadIdx.x;
    // pe, m v^2, m v (3), count, pair virial
    double acc[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    if (i < n)
    {
        const int ki = S.kind[i];
        const bool active = (group < 0 || S.group[i] == group);
        double f[3] = {0.0, 0.0, 0.0};
        double pe = 0.0, vir = 0.0;
        if (active)
        {
            const CellXYZ ci = cell_xyz(g, S.cell_of[i]);
            const int nk = g.nkinds;
            const int nint = g.Nr2 - 1;
            const size_t ne = g.nelem;
            if (!MIXED)
            {
                // binary64 mode: double-float pair arithmetic (fmdg_df.cuh)
                // in the reference's formulas -- LJ src/lj.h:35-56, Morse
                // src/morse.h:35-56, EAM src/eam.h:186-226 -- the category
                // chosen per pair for hybrid tables (src/forces.c:33-290)
                float4 ih, il;
                ld_row32(g.xdf + 2 * (size_t)i, ih, il);
                const dfl fpi = (CAT == CAT_EAM || CAT == CAT_HYBRID) ? df_of(g.fpdf[i]) : dfl{0.f, 0.f};
                const dfl inv_h = df_of(df_split(g.inv_dr2));
                const float kmax = (float)(nint - 1);
                dfl fs[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}}, pes = {0.f, 0.f}, virs = {0.f, 0.f};
                for_each_pair(g, S, i, ci, [&](int j, int code) {
                    if (group >= 0 && S.group[j] != group) return;
                    float4 jh, jl;
                    ld_row32(g.xdf + 2 * (size_t)j, jh, jl);
                    const int pidx = ki * nk + __float_as_int(jh.w);
                    const fmdg_pair_t &pp = sp.pairs[pidx];
                    const int cat = (CAT == CAT_HYBRID) ? pp.cat : CAT;
                    const int rci = (cat == FMDG_POT_MORSE) ? 3 : 2;
                    const GeomDF p = geom_df(ih, il, jh, jl, sp.off[code], sp.offl[code]);
                    if (!within_cut_df(g, S, i, ci, j, code, p.r2, sp.pf[pidx][rci], pp.p[rci])) return;
                    dfl fa, eh;     // f_i += fa * rv, energy share eh
                    df_pair(g, sp, pidx, pp, cat, p, fpi, inv_h, kmax, nint, ne, [&]() { return df_of(g.fpdf[j]); },
                            fa, eh);
                    for (int d = 0; d < 3; d++) fs[d] = df_add(fs[d], df_mul(fa, p.rv[d]));
                    pes = df_add(pes, eh);
                    virs = df_add(virs, df_mul(fa, p.r2));     // rv . (fa rv), both sides of the pair
                });
                for (int d = 0; d < 3; d++) f[d] = df_to_double(fs[d]);
                pe = df_to_double(pes);
                vir = 0.5 * df_to_double(virs);
            }
            else
            {
                const float4 xi = g.xf4[i];
                const float fpi = (CAT == CAT_EAM || CAT == CAT_HYBRID) ? g.fpf[i] : 0.f;
                const float inv_h = (float)g.inv_dr2;
                const float kmax = (float)(nint - 1);
                Acc32<5> ac;
                for_each_pair(g, S, i, ci, [&](int j, int code) {
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
                            ac.part[4] += factor * r2;
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
                            ac.part[4] += factor * r2;
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
                            ac.part[4] -= mag * r2;
                        }
                    }
                    ac.tick();
                });
                ac.flush();
                for (int d = 0; d < 3; d++) f[d] = ac.total(d);
                pe = ac.total(3);
                vir = 0.5 * ac.total(4);
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
        acc[6] = vir;
        if (active)
        {
            const double m = sp.mass[ki];
            double v[3] = {S.v[i], S.v[cap + i], S.v[2 * (size_t)cap + i]};
            if (finish)
            {
                const double coef = sp.hk[ki];   // dt * 0.5 / m, as the reference forms it
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
    __shared__ double blk[7];
    __shared__ unsigned ticket;
    block_reduce_store<7>(acc, blk);
    if (threadIdx.x == 0)
    {
        for (int k = 0; k < 7; k++) g.partials[(size_t)k * nb + bx] = blk[k];
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
    if (s->g.skin_on) return fmdg_skin_launch_nlist(s);
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
    if (s->g.skin_on) return fmdg_skin_launch_density(s);
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
    set_step_dt(s, dt);
    a.thermostat = thermostat;
    a.tau = tau;
    a.T0 = T0;
    if (s->g.skin_on) return fmdg_skin_launch_pair_forces(s, finish);
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
