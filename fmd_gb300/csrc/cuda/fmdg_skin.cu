// Pair kernels over a Verlet-skin neighbour list: packed (served) systems,
// and single systems in mixed precision whose box allows it.
//
// Systems on the per-step path rebuild their list every step in the
// current (reference cell) order.  Skin-list systems keep a list of radius
// rc + skin indexed by a slot number and rebuild it only when an atom has
// moved more than skin/2 since the last build -- the usual Verlet-list
// criterion, which keeps every pair that can come within the cutoff in the
// list.  Pairs are still tested against the exact cutoff at every
// evaluation, so the list only prunes.
//
// Slots.  A slot starts as the atom's upload position and travels with the
// atom through every re-binning.  Packed systems renumber the slots in the
// current cell order at each rebuild (slot = index), and refresh their
// cells only on rebuild steps, so between rebuilds slot and index coincide.
//
// Packed step:
//   k_skin_start    velocity-Verlet start step, per-step slot positions,
//                   displacement test -> rebuild flag
//   (rebuild steps only) reference-order cell refresh (fmdg_bin.cu),
//   k_prep_skin     slot tables (renumbered), k_nlist_skin stencil scan of
//                   the cells within the list radius
//   k_density_skin  EAM pass 1 + embedding, one thread per slot
//   k_force_skin    pair forces + velocity-Verlet finish step + thermo
//                   record, one thread per slot
// Single-system step: the reference-order refresh every step, then
// k_prep_skin (stable slots), k_nlist_skin (when flagged), density, forces.
//
// Geometry.  An atom's binary32 position is kept relative to the cell it
// had at the last build (unwrapped across periodic faces: it moves less
// than skin/2 before the next build), and a list entry holds the stencil
// offset between the two build cells, so a pair is formed exactly as on the
// per-step path: x_i - x_j - offset * cellh.  Binary64: the minimum image
// as the reference's ghost copy forms it (x_j + shift, then x_i minus that,
// src/md-ghost.c:85-107, src/forces.h:25-34); every periodic box length
// exceeds twice the list radius, so one image at most lies inside it.
// Pair arithmetic and precision modes are those of the per-step kernels
// (fmdg_force.cu); the lean variants (one kind, no group) are described at
// k_force_skin.
#include <type_traits>

#include "fmdg_pairs.cuh"

namespace {

// list entry (read as unsigned): neighbour slot | stencil code << 25; code
// < 125 over a stencil of radius R (width W = 2R + 1):
// ((ox + R) W + (oy + R)) W + (oz + R).  Layout: rounds of four entries,
// int4 row (k / 4) * cap + t holds entries k..k+3 of slot t (one 16-byte
// access per round; a row is contiguous over consecutive slots).
constexpr int SLOT_BITS = 25;
constexpr int SLOT_MASK = (1 << SLOT_BITS) - 1;

// Image offsets of the stencil codes in shared memory, in the scaled frame
// (Geo::xs): off = (ox, oy, oz) * cellh_s is exact in binary32 (|o| <= 2);
// the remainder offl = (ox, oy, oz) * (cellh xs - cellh_s) completes it to
// the binary64 offset (double-float in binary64 mode; in binary32 one more
// subtraction in the general kernels, zero on a cubic grid).
template <bool LO>   // LO: with the remainders (binary64 mode, general binary32 kernels); lean layouts go without
struct SkinOffT
{
    float4 off[125];    // image offset of each stencil code, binary32; .w: the code's bits
    float4 offl[LO ? 125 : 1];   // the remainders (binary64 offset - off)
};

template <bool LO>
__device__ __forceinline__ void load_offsets(const Geo &g, SkinOffT<LO> &so)
{
    const int R = g.srad, W = 2 * R + 1;
    // remainders cellh xs - cellh_s (3 binary64 operations per block)
    const float lx = (float)(g.cellh[0] * g.xs - (double)g.cellh_s[0]),
                ly = (float)(g.cellh[1] * g.xs - (double)g.cellh_s[1]),
                lz = (float)(g.cellh[2] * g.xs - (double)g.cellh_s[2]);
    for (int c = threadIdx.x; c < W * W * W; c += blockDim.x)
    {
        const float ox = small_int_f(c / (W * W) - R), oy = small_int_f((c / W) % W - R), oz = small_int_f(c % W - R);
        so.off[c] = make_float4(ox * g.cellh_s[0], oy * g.cellh_s[1], oz * g.cellh_s[2], __int_as_float(c));
        if (LO) so.offl[c] = make_float4(ox * lx, oy * ly, oz * lz, 0.f);
    }
    __syncthreads();
}

// the scaled frame (Geo::xs): binary32 xs^2 (force constants) and the EAM
// r^2-grid index factor of a scaled r^2
__device__ __forceinline__ float scaled_xs2(const Geo &g) { return (float)(g.xs * g.xs); }
__device__ __forceinline__ float scaled_index_factor(const Geo &g) { return (float)(g.inv_dr2 * (g.inv_xs * g.inv_xs)); }

// binary32 pair vector x_i - x_j - offset without the offset's remainder
// (list-radius prefilters)
__device__ __forceinline__ float3 rv_of(float4 xi, float4 xj, float4 o)
{
    return make_float3(xi.x - xj.x - o.x, xi.y - xj.y - o.y, xi.z - xj.z - o.z);
}

// binary32 pair vector of a list entry with the offset's remainder: the
// binary32 rounding of (ox, oy, oz) * cellh would otherwise shift every
// pair across a cell face by up to half an ulp of the cell width
// (5e-7 A), as much as the rounding of the coordinates themselves.  o.w
// holds the stencil code (an overflow-fallback occurrence: -1 - code).
template <bool DF>
__device__ __forceinline__ float3 rv_lo(const SkinOffT<DF> &so, float4 xi, float4 xj, float4 o)
{
    const int code = __float_as_int(o.w);
    const float4 ol = so.offl[code ^ (code >> 31)];
    return make_float3(xi.x - xj.x - o.x - ol.x, xi.y - xj.y - o.y - ol.y, xi.z - xj.z - o.z - ol.z);
}

// binary64 minimum-image geometry rv = x_a - (x_b + shift)
__device__ __forceinline__ Geom64 geom64_mi(const Geo &g, double4_32a a, double4_32a b)
{
    const double xa[3] = {a.x, a.y, a.z}, xb[3] = {b.x, b.y, b.z};
    Geom64 p;
    for (int d = 0; d < 3; d++)
    {
        double x2 = xb[d];
        if (g.pbc[d])
        {
            const double dd = xa[d] - x2;
            if (dd > 0.5 * g.l[d]) x2 = __dadd_rn(x2, g.l[d]);
            else if (dd < -0.5 * g.l[d]) x2 = __dadd_rn(x2, -g.l[d]);
        }
        p.rv[d] = __dsub_rn(xa[d], x2);
    }
    p.r2 = __dadd_rn(__dadd_rn(__dmul_rn(p.rv[0], p.rv[0]), __dmul_rn(p.rv[1], p.rv[1])),
                     __dmul_rn(p.rv[2], p.rv[2]));
    return p;
}

// binary32 cutoff test; within 1e-4 relative of the cutoff the decision is
// taken in binary64 from the binary64 positions
__device__ __forceinline__ bool within_cut_skin(const Geo &g, int ta, int tb, float r2f, float rc2f, double rc2)
{
    if (fabsf(r2f - rc2f) > 1e-4f * rc2f) return r2f < rc2f;
    return geom64_mi(g, g.xd[ta], g.xd[tb]).r2 < rc2;
}

// Gap along one axis between a point at u inside its cell box [0, h) and
// the cell at offset o (0 for the cell itself).
__device__ __forceinline__ float axis_gap(int o, float u, float h)
{
    return o > 0 ? fmaxf(0.f, (float)o * h - u) : (o < 0 ? fmaxf(0.f, u + (float)(-o - 1) * h) : 0.f);
}

// Binary64 mode: double-float geometry of a list entry (build frame: slot
// positions xl + xll and the entry's stencil offset) or of an overflow
// fallback occurrence (code < 0 in o.w: current-cell frame, formed from the
// binary64 positions); the cutoff decision within 1e-6 relative of the
// cutoff is the binary64 minimum-image one.
template <bool DF>
__device__ __forceinline__ GeomDF skin_geom_df(const Geo &g, const SkinOffT<DF> &so, int t, float4 ih, float4 il, int js,
                                               float4 xj, float4 o)
{
    const int code = __float_as_int(o.w);
    if (code >= 0) return geom_df(ih, il, xj, g.xll[js], o, so.offl[code]);
    return geom_df_of64(geom64_mi(g, g.xd[t], g.xd[js]));
}

__device__ __forceinline__ bool within_cut_df_mi(const Geo &g, int t, int js, dfl r2, float rc2f, double rc2)
{
    const float d = __fsub_rn(r2.hi, rc2f);
    if (fabsf(d) > 1e-6f * rc2f) return d < 0.f;
    return geom64_mi(g, g.xd[t], g.xd[js]).r2 < rc2;
}

// Every cell c of the stencil of radius R around cell ci, with its stencil
// code, in a fixed order: f(code, c).  On a periodic axis shorter than the
// stencil a cell recurs with another image (at most one image of a pair
// lies within the list radius).  xi: the atom's binary32 position relative
// to the centre of cell ci; a cell whose box lies farther than the list
// radius from xi (plus 1e-4 relative) holds no candidate and is skipped.
template <typename F>
__device__ __forceinline__ void for_each_stencil_cell(const Geo &g, CellXYZ ci, float4 xi, F &&f)
{
    const int R = g.srad, W = 2 * R + 1;
    const float lim2 = g.rskin2 * 1.0001f;
    // position inside the cell box [0, h) (up to the drift since the build)
    const float ux = xi.x + 0.5f * g.cellh_s[0], uy = xi.y + 0.5f * g.cellh_s[1], uz = xi.z + 0.5f * g.cellh_s[2];
    for (int ox = -R; ox <= R; ox++)
    {
        const float gx = axis_gap(ox, ux, g.cellh_s[0]);
        if (gx * gx > lim2) continue;
        int cx = ci.x + ox;
        if (cx < 0 || cx >= g.nc[0])
        {
            if (!g.pbc[0]) continue;
            cx = (cx + 2 * g.nc[0]) % g.nc[0];
        }
        for (int oy = -R; oy <= R; oy++)
        {
            const float gy = axis_gap(oy, uy, g.cellh_s[1]);
            if (gx * gx + gy * gy > lim2) continue;
            int cy = ci.y + oy;
            if (cy < 0 || cy >= g.nc[1])
            {
                if (!g.pbc[1]) continue;
                cy = (cy + 2 * g.nc[1]) % g.nc[1];
            }
            for (int oz = -R; oz <= R; oz++)
            {
                const float gz = axis_gap(oz, uz, g.cellh_s[2]);
                if (gx * gx + gy * gy + gz * gz > lim2) continue;
                int cz = ci.z + oz;
                if (cz < 0 || cz >= g.nc[2])
                {
                    if (!g.pbc[2]) continue;
                    cz = (cz + 2 * g.nc[2]) % g.nc[2];
                }
                f(((ox + R) * W + (oy + R)) * W + (oz + R), cz + g.nc[2] * (cy + g.nc[1] * cx));
            }
        }
    }
}

// the stencil code of the atom's own cell
__device__ __forceinline__ int home_code(const Geo &g)
{
    const int R = g.srad, W = 2 * R + 1;
    return (R * W + R) * W + R;
}

// every (j, code) of the stencil around i's current cell, j the current
// index, i itself left out
template <typename F>
__device__ __forceinline__ void for_each_candidate(const Geo &g, const Side &S, int i, float4 xi, F &&f)
{
    const int home = home_code(g);
    for_each_stencil_cell(g, cell_xyz(g, S.cell_of[i]), xi, [&](int code, int c) {
        const int je = S.cell_start[c + 1];
        for (int j = S.cell_start[c]; j < je; j++)
            if (!(code == home && j == i)) f(j, code);
    });
}

struct NoRound
{
    __device__ __forceinline__ void operator()(int) const {}
};

// List walk of slot t (four entries per round): f(neighbour slot, its
// binary32 position, image offset); r(k) after every k entries visited (a
// round of four, or one).  PF: the next round's list rows are prefetched
// into L1 while this round is processed (the rows stream from DRAM).
// An atom whose list overflowed scans the stencil of its cell directly:
// positions are the current binary64 ones relative to the cells of the
// last refresh (packed systems refresh their cells only at a rebuild; an
// atom has moved less than skin/2 since, so the stencil still covers the
// list radius), and of the occurrences of a neighbour (a cell recurs in the
// stencil when an axis has fewer than 2R + 1 cells) only the image within
// the list radius is passed on.
template <bool PF = false, typename F, typename R, bool DF>
__device__ __forceinline__ void for_each_slot_pair(const Geo &g, const Side &S, const SkinOffT<DF> &so, int t, int i,
                                                   float4 &xi, F &&f, R &&r)
{
    const int cnt = g.nbr_count[t];
    if (cnt <= g.maxnb)
    {
        const int cap = g.cap;
        const int4 *col = reinterpret_cast<const int4 *>(g.nbr) + t;
        int k = 0;
        for (; k + 4 <= cnt; k += 4)
        {
            if (PF && k + 8 <= cnt) asm volatile("prefetch.global.L1 [%0];" ::"l"(col + (size_t)((k >> 2) + 1) * cap));
            const int4 e4 = __ldg(col + (size_t)(k >> 2) * cap);
            const int e0 = e4.x, e1 = e4.y, e2 = e4.z, e3 = e4.w;
            const float4 x0 = g.xl[e0 & SLOT_MASK], x1 = g.xl[e1 & SLOT_MASK];
            const float4 x2 = g.xl[e2 & SLOT_MASK], x3 = g.xl[e3 & SLOT_MASK];
            f(e0 & SLOT_MASK, x0, so.off[(unsigned)e0 >> SLOT_BITS]);
            f(e1 & SLOT_MASK, x1, so.off[(unsigned)e1 >> SLOT_BITS]);
            f(e2 & SLOT_MASK, x2, so.off[(unsigned)e2 >> SLOT_BITS]);
            f(e3 & SLOT_MASK, x3, so.off[(unsigned)e3 >> SLOT_BITS]);
            r(4);
        }
        if (k < cnt)
        {
            // the last, partial round (1-3 entries)
            const int4 e4 = __ldg(col + (size_t)(k >> 2) * cap);
            const int ee[3] = {e4.x, e4.y, e4.z};
            for (int q = 0; q < 3 && k + q < cnt; q++)
            {
                const int e = ee[q];
                f(e & SLOT_MASK, g.xl[e & SLOT_MASK], so.off[(unsigned)e >> SLOT_BITS]);
                r(1);
            }
        }
    }
    else
    {
        const double4_32a xdi = g.xd[t], oi = g.corig[S.cell_of[i]];
        const double xs = g.xs;
        xi = make_float4((float)((xdi.x - oi.x) * xs), (float)((xdi.y - oi.y) * xs), (float)((xdi.z - oi.z) * xs),
                         xi.w);
        const float lim2 = g.rskin2 * 1.0001f;
        for_each_candidate(g, S, i, xi, [&](int j, int code) {
            const int js = S.slot[j];
            const double4_32a xdj = g.xd[js], oj = g.corig[S.cell_of[j]];
            const float4 xj = make_float4((float)((xdj.x - oj.x) * xs), (float)((xdj.y - oj.y) * xs),
                                          (float)((xdj.z - oj.z) * xs), g.xf4[j].w);
            float4 o = so.off[code];
            const float3 d = rv_of(xi, xj, o);
            if (d.x * d.x + d.y * d.y + d.z * d.z > lim2) return;
            o.w = __int_as_float(-1 - code);    // current-cell frame, not the build frame
            f(js, xj, o);
            r(1);
        });
    }
}

template <typename F, bool DF>
__device__ __forceinline__ void for_each_slot_pair(const Geo &g, const Side &S, const SkinOffT<DF> &so, int t, int i,
                                                   float4 &xi, F &&f)
{
    for_each_slot_pair(g, S, so, t, i, xi, f, NoRound{});
}

// ---------------------------------------------------------------- kernels

// Slot t's binary32 position relative to the cell it had at the last build
// (unwrapped across periodic faces) and the displacement test against its
// build position: sets the rebuild flag beyond skin/2.
__device__ __forceinline__ void slot_rel_build(const Geo &g, Dyn *dyn, int t, const double (&x)[3], float kb)
{
    const double4_32a ob = g.corig[g.cb[t]];
    const double o3[3] = {ob.x, ob.y, ob.z};
    float l3[3];
    double u3[3];
    const double xs = g.xs;     // (1 in binary64 mode: xll below holds remainders of unscaled values)
    for (int d = 0; d < 3; d++)
    {
        double u = x[d] - o3[d];
        float uf = d2f_rn(u * xs);
        // unwrap across a periodic face (binary64 test near half a box)
        if (g.pbc[d] && fabsf(uf) > 0.49f * g.l_f[d])
        {
            if (u > 0.5 * g.l[d]) u -= g.l[d];
            else if (u < -0.5 * g.l[d]) u += g.l[d];
            uf = d2f_rn(u * xs);
        }
        l3[d] = uf;
        u3[d] = u;
    }
    g.xl[t] = make_float4(l3[0], l3[1], l3[2], kb);
    if (g.prec == FMDG_PREC_FP64)
        g.xll[t] = make_float4((float)(u3[0] - (double)l3[0]), (float)(u3[1] - (double)l3[1]),
                               (float)(u3[2] - (double)l3[2]), 0.f);
    const float4 o = g.xb[t];
    const float dx = l3[0] - o.x, dy = l3[1] - o.y, dz = l3[2] - o.z;
    if (!(dx * dx + dy * dy + dz * dz <= g.half_skin2)) dyn->rebuild = 1;
}

// Packed systems, every step (one thread per current atom index): the
// velocity-Verlet start step (src/integrators.c:40-75, the operations of
// k_bin_classify), the slot tables that change every step and the
// displacement test; advances the device time by one step.  The cells and
// the remaining slot tables are refreshed on rebuild steps only.
template <class L>
__global__ void k_skin_start(__grid_constant__ const L loc)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    const double dt = g.st.dt;
    const int group = g.st.group, thermostat = g.st.thermostat;
    __shared__ double hk[FMDG_MAXK];
    if (threadIdx.x < g.nkinds) hk[threadIdx.x] = g.st.hk[threadIdx.x];
    __syncthreads();
    Dyn *dyn = g.dyn;
    if (bx == 0 && threadIdx.x == 0) dyn->time += dt;
    const int i = bx * blockDim.x + threadIdx.x;
    if (i >= dyn->n) return;
    const Side S = g.side[dyn->cur];
    const size_t cap = g.cap;
    const int kind = (int)S.kind[i];
    double x[3] = {S.x[i], S.x[cap + i], S.x[2 * cap + i]};
    if (group < 0 || S.group[i] == group)
    {
        const double lam = dyn->lambda;
        const double coef = hk[kind];
        for (int d = 0; d < 3; d++)
        {
            double vv = S.v[d * cap + i];
            if (thermostat) vv = __dmul_rn(vv, lam);
            vv = __dadd_rn(vv, __dmul_rn(coef, g.F[d * cap + i]));
            S.v[d * cap + i] = vv;
            x[d] = __dadd_rn(x[d], __dmul_rn(dt, vv));
            S.x[d * cap + i] = x[d];
        }
    }
    const int t = S.slot[i];
    g.xd[t] = make_double4_32a(x[0], x[1], x[2], 0.0);
    slot_rel_build(g, dyn, t, x, __int_as_float(kind));
}

// one thread per current atom index.  lazy (packed systems): rebuild steps
// only, after the cell refresh, and the slots are renumbered in the
// current (cell) order -- slot = index, so the rebuild walks and writes
// consecutive atoms of a cell together, and until the next rebuild (no
// refresh in between) every slot-to-index map is the identity
template <class L>
__global__ void k_prep_skin(__grid_constant__ const L loc, int lazy)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    Dyn *dyn = g.dyn;
    if (lazy && !dyn->rebuild) return;
    const int i = bx * blockDim.x + threadIdx.x;
    if (i >= dyn->n)
    {
        if (lazy && i < g.cap) g.pos[i] = -1;
        return;
    }
    const Side S = g.side[dyn->cur];
    const int cap = g.cap;
    const int t = lazy ? i : S.slot[i];
    if (lazy) S.slot[i] = i;
    const double x[3] = {S.x[i], S.x[cap + i], S.x[2 * (size_t)cap + i]};
    const int kind = (int)S.kind[i];
    const float kb = __int_as_float(kind);
    g.pos[t] = i;
    g.xd[t] = make_double4_32a(x[0], x[1], x[2], 0.0);
    g.gslot[t] = S.group[i];
    // relative to the current cell (a rebuild starts from these)
    const double4_32a oc = g.corig[S.cell_of[i]];
    const double ux = x[0] - oc.x, uy = x[1] - oc.y, uz = x[2] - oc.z;
    const double xs = g.xs;     // (1 in binary64 mode: the remainders below are of unscaled values)
    const float lx = (float)(ux * xs), ly = (float)(uy * xs), lz = (float)(uz * xs);
    g.xf4[i] = make_float4(lx, ly, lz, kb);
    if (g.prec == FMDG_PREC_FP64)
    {
        g.xdf[2 * (size_t)i] = make_float4(lx, ly, lz, kb);
        g.xdf[2 * (size_t)i + 1] =
            make_float4((float)(ux - (double)lx), (float)(uy - (double)ly), (float)(uz - (double)lz), 0.f);
    }
    // (renumbered, or a rebuild already due: the build cell and position of
    // slot t are rewritten by the list build that follows)
    if (!lazy && !dyn->rebuild) slot_rel_build(g, dyn, t, x, kb);
}

// The stencil walk of a list build: f(code, c, ax, ay, az) for every cell
// of for_each_stencil_cell, with the cell's image offset folded into the
// atom's position once per cell (ax, ay, az).
template <typename F>
__device__ __forceinline__ void for_each_build_cell(const Geo &g, const SkinOffT<false> &so, CellXYZ ci, float4 xi,
                                                    F &&f)
{
    for_each_stencil_cell(g, ci, xi, [&](int code, int c) {
        const float4 o = so.off[code];
        f(code, c, xi.x - o.x, xi.y - o.y, xi.z - o.z);
    });
}

// per-slot state recorded with a new list: build cell and build-frame
// position (+ its double-float remainder in binary64 mode)
__device__ __forceinline__ void record_build(const Geo &g, const Side &S, int t, int i, float4 xi)
{
    g.cb[t] = S.cell_of[i];
    g.xl[t] = xi;
    g.xb[t] = xi;
    if (g.prec == FMDG_PREC_FP64) g.xll[t] = g.xdf[2 * (size_t)i + 1];
}

// the last block of a build to finish clears the system's rebuild flag
__device__ __forceinline__ void finish_build(Dyn *dyn, int nb)
{
    __shared__ unsigned ticket;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        __threadfence();
        ticket = atomicAdd(&dyn->nl_done, 1u);
    }
    __syncthreads();
    if (ticket == (unsigned)nb - 1 && threadIdx.x == 0)
    {
        dyn->nl_done = 0;
        dyn->rebuild = 0;
    }
}

// one thread per slot; every block leaves at once when no rebuild is due
template <class L>
__global__ void __launch_bounds__(L::max_threads, L::min_blocks) k_nlist_skin(__grid_constant__ const L loc)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    Dyn *dyn = g.dyn;
    if (!dyn->rebuild) return;
    __shared__ SkinOffT<false> so;
    load_offsets(g, so);
    const int cap = g.cap, maxnb = g.maxnb;
    const int t = bx * blockDim.x + threadIdx.x;
    if (t < cap)
    {
        int cnt = 0;
        const int i = g.pos[t];
        if (i >= 0)
        {
            const Side S = g.side[dyn->cur];
            const float4 xi = g.xf4[i];
            const float rl2 = g.rskin2;
            int4 *row = reinterpret_cast<int4 *>(g.nbr) + t;
            // hits shift through a four-entry register buffer (in order:
            // x oldest); every fourth hit writes one 16-byte row; the
            // buffer update is branch-free (a warp's lanes hit at different
            // candidates).  The self test is only in the atom's own cell;
            // the radius is widened by 1e-5 relative so the folded rounding
            // of the cell offsets can only add entries.
            int4 buf = make_int4(0, 0, 0, 0);
            const float rb2 = rl2 * 1.00001f;
            auto take = [&](int j, int code, float ax, float ay, float az) {
                const float4 xj = __ldg(g.xf4 + j);
                const float dx = ax - xj.x, dy = ay - xj.y, dz = az - xj.z;
                const bool hit = dx * dx + dy * dy + dz * dz < rb2;
                const int sj = L::renumbered ? j : (hit ? S.slot[j] : 0);
                const int e = (int)((unsigned)sj | ((unsigned)code << SLOT_BITS));
                buf.x = hit ? buf.y : buf.x;
                buf.y = hit ? buf.z : buf.y;
                buf.z = hit ? buf.w : buf.z;
                buf.w = hit ? e : buf.w;
                cnt += hit;
                if (hit && (cnt & 3) == 0 && cnt <= maxnb) row[(size_t)((cnt >> 2) - 1) * cap] = buf;
            };
            const int center = home_code(g);
            for_each_build_cell(g, so, cell_xyz(g, S.cell_of[i]), xi, [&](int code, int c, float ax, float ay, float az) {
                const int jb = S.cell_start[c], je = S.cell_start[c + 1];
                if (code == center)
                {
                    for (int j = jb; j < i; j++) take(j, code, ax, ay, az);
                    for (int j = i + 1; j < je; j++) take(j, code, ax, ay, az);
                }
                else
                    for (int j = jb; j < je; j++) take(j, code, ax, ay, az);
            });
            const int rem = cnt & 3;
            if (rem && cnt <= maxnb)
            {
                const int4 last = (rem == 1) ? make_int4(buf.w, 0, 0, 0)
                                : (rem == 2) ? make_int4(buf.z, buf.w, 0, 0) : make_int4(buf.y, buf.z, buf.w, 0);
                row[(size_t)(cnt >> 2) * cap] = last;
            }
            record_build(g, S, t, i, xi);
        }
        g.nbr_count[t] = cnt;
    }
    finish_build(dyn, nb);
}

// Single-system build (a served job's admission, the fmd.h path) with G
// lanes per slot: a system of 10^4-10^5 atoms gives one thread per slot too
// few warps to hide the gather latency of its long candidate walk.  The G
// lanes of a slot test G consecutive candidates of a cell together and
// place their hits in candidate order (ballot + prefix count), so the list
// is the one-thread build's, entry for entry.
// The list of slot t built by the G lanes of a group (gl: this lane's
// index in it, gbase: the group's first lane in the warp): the lanes test
// G consecutive candidates of a cell together and place their hits in
// candidate order (ballot + prefix count), so the list is the one-thread
// build's, entry for entry.  Every lane of the group must call it (its
// control flow depends on the slot only).
__device__ __forceinline__ void build_slot_grouped(const Geo &g, const Side &S, const SkinOffT<false> &so, int t,
                                                   int G, int gl, int gbase)
{
    const int cap = g.cap, maxnb = g.maxnb;
    const unsigned gmask = (G == 32) ? 0xffffffffu : ((1u << G) - 1u) << gbase;
    int cnt = 0;
    const int i = g.pos[t];
    if (i >= 0)
    {
        const float4 xi = g.xf4[i];
        const float rb2 = g.rskin2 * 1.00001f;   // as in k_nlist_skin
        int *ent = g.nbr;   // entry k of slot t: int4 row (k / 4) * cap + t, component k % 4
        const int center = home_code(g);
        for_each_build_cell(g, so, cell_xyz(g, S.cell_of[i]), xi, [&](int code, int c, float ax, float ay, float az) {
            const int jb = S.cell_start[c], je = S.cell_start[c + 1];
            const bool self = code == center;
            for (int base = jb; base < je; base += G)
            {
                const int j = base + gl;
                bool hit = false;
                if (j < je && !(self && j == i))
                {
                    const float4 xj = __ldg(g.xf4 + j);
                    const float dx = ax - xj.x, dy = ay - xj.y, dz = az - xj.z;
                    hit = dx * dx + dy * dy + dz * dz < rb2;
                }
                const unsigned m = __ballot_sync(gmask, hit) >> gbase;
                if (hit)
                {
                    const int k = cnt + __popc(m & ((1u << gl) - 1u));
                    if (k < maxnb)
                        ent[((size_t)(k >> 2) * cap + t) * 4 + (k & 3)] =
                            (int)((unsigned)S.slot[j] | ((unsigned)code << SLOT_BITS));
                }
                cnt += __popc(m);
            }
        });
        if (gl == 0) record_build(g, S, t, i, xi);
    }
    if (gl == 0) g.nbr_count[t] = cnt;
}

// Single-system build (a served job's admission, the fmd.h path) with G
// lanes per slot: a system of 10^3-10^5 atoms gives one thread per slot too
// few warps to hide the gather latency of its long candidate walk.
template <int G>
__global__ void __launch_bounds__(128) k_nlist_skin_grp(__grid_constant__ const LocOne loc)
{
    static_assert(G >= 2 && G <= 32 && (G & (G - 1)) == 0, "G: a power of two up to the warp");
    const Geo &g = loc.g;
    Dyn *dyn = g.dyn;
    if (!dyn->rebuild) return;
    __shared__ SkinOffT<false> so;
    load_offsets(g, so);
    const int t = (blockIdx.x * blockDim.x + threadIdx.x) / G;   // uniform over a group
    if (t < g.cap) build_slot_grouped(g, g.side[dyn->cur], so, t, G, threadIdx.x & (G - 1), threadIdx.x & 31 & ~(G - 1));
    finish_build(dyn, gridDim.x);
}

// EAM pass 1 + embedding (src/eam.h:270-406, src/eam.c:160-179), one
// thread per slot.  LEAN (binary32, one kind, no group): the pair's table
// row and cutoff in registers, no per-entry kind or group lookups.
template <class L, bool MIXED, bool HYBRID, bool LEAN>
__global__ void __launch_bounds__(L::max_threads, L::min_blocks) k_density_skin(__grid_constant__ const L loc)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    const int group = g.st.group;
    __shared__ SmemPotT<!MIXED, LEAN> sp;
    __shared__ SkinOffT<!MIXED || !LEAN> so;   // lean binary32 kernels: no remainders (exact on a cubic grid)
    load_pot(g, sp, skin_params(g));
    load_offsets(g, so);
    Dyn *dyn = g.dyn;
    const Side S = g.side[dyn->cur];
    const int t = bx * blockDim.x + threadIdx.x;
    double acc[1] = {0.0};
    const int i = (t < g.cap) ? g.pos[t] : -1;
    if (i >= 0)
    {
        float4 xi = g.xl[t];
        const int ki = __float_as_int(xi.w);
        const int ei = sp.elem[ki];
        const bool active = (group < 0 || g.gslot[t] == group) && ei >= 0;   // hybrid: EAM kinds only
        const int nk = g.nkinds, nint = g.Nr2 - 1;
        double rho = 0.0;
        if (active)
        {
            if (!MIXED)
            {
                // double-float pair arithmetic (fmdg_df.cuh)
                const float4 ih = g.xl[t], il = g.xll[t];
                const dfl inv_h = df_of(df_split(g.inv_dr2));
                const float kmax = (float)(nint - 1);
                dfl acc_rho = {0.f, 0.f};
                for_each_slot_pair(g, S, so, t, i, xi, [&](int js, float4 xjf, float4 o) {
                    if (group >= 0 && g.gslot[js] != group) return;
                    const int pidx = ki * nk + __float_as_int(xjf.w);
                    const fmdg_pair_t &pp = sp.pairs[pidx];
                    if (HYBRID && pp.cat != FMDG_POT_EAM) return;
                    const GeomDF p = skin_geom_df(g, so, t, ih, il, js, xjf, o);
                    if (within_cut_df_mi(g, t, js, p.r2, sp.pf[pidx][2], pp.p[2]))
                        acc_rho = df_add(acc_rho, df_rho(g, pp, p, inv_h, kmax, nint));
                });
                rho = df_to_double(acc_rho);
            }
            else if constexpr (LEAN)
            {
                // branch-free walk (table rows read for every entry, entries
                // beyond the cutoff add zero); near-cutoff entries decided in
                // binary64 after the walk, as in the lean force kernel
                const float inv_h = scaled_index_factor(g);   // (scaled r^2: index only)
                const float kmax = (float)(nint - 1);
                const float4 *trho = g.pkf_rho + (size_t)sp.pairs[0].jloc * nint;
                const float rc2f = sp.pf[0][2], band = 2e-5f * rc2f;
                const double rc2 = sp.pairs[0].p[2];
                Acc32<1> ac;
                int npend = 0, pend = 0;
                float pr2 = 0.f;
                for_each_slot_pair<true>(g, S, so, t, i, xi, [&](int js, float4 xj, float4 o) {
                    const float3 rv = rv_of(xi, xj, o);
                    const float r2 = rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
                    const bool near = fabsf(r2 - rc2f) <= band;
                    const bool in = (r2 < rc2f) && !near;
                    npend += near;
                    pend = near ? js : pend;
                    pr2 = near ? r2 : pr2;
                    float b;
                    const int ir2 = table_index(r2 * inv_h, kmax, b);
                    const float v = spl_val(trho[ir2], b);
                    ac.part[0] += in ? v : 0.f;
                }, [&](int k) { ac.entries(k); });
                ac.flush();
                if (npend == 1)
                {
                    if (geom64_mi(g, g.xd[t], g.xd[pend]).r2 < rc2)
                    {
                        float b;
                        const int ir2 = table_index(pr2 * inv_h, kmax, b);
                        ac.part[0] += spl_val(trho[ir2], b);
                        ac.flush();
                    }
                }
                else if (npend > 1)
                {
                    for_each_slot_pair<false>(g, S, so, t, i, xi, [&](int js, float4 xj, float4 o) {
                        const float3 rv = rv_of(xi, xj, o);
                        const float r2 = rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
                        if (!(fabsf(r2 - rc2f) <= band)) return;
                        if (!(geom64_mi(g, g.xd[t], g.xd[js]).r2 < rc2)) return;
                        float b;
                        const int ir2 = table_index(r2 * inv_h, kmax, b);
                        ac.part[0] += spl_val(trho[ir2], b);
                    }, [&](int k) { ac.entries(k); });
                    ac.flush();
                }
                rho = ac.total(0);
            }
            else
            {
                const float inv_h = scaled_index_factor(g);   // (scaled r^2: index only)
                const float kmax = (float)(nint - 1);
                Acc32<1> ac;
                for_each_slot_pair(g, S, so, t, i, xi, [&](int js, float4 xj, float4 o) {
                    if (group >= 0 && g.gslot[js] != group) return;
                    const int pidx = ki * nk + __float_as_int(xj.w);
                    const fmdg_pair_t &pp = sp.pairs[pidx];
                    const float3 rv = rv_lo(so, xi, xj, o);
                    const float r2 = rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
                    if ((!HYBRID || pp.cat == FMDG_POT_EAM) &&
                        within_cut_skin(g, t, js, r2, sp.pf[pidx][2], pp.p[2]))
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
            const double qr = rho * g.inv_drho;
            int irho = (int)qr;
            if (irho >= g.Nrho - 1 || irho < 0)
            {
                atomic_or_err(dyn, FMDG_ERRBIT_RHO_RANGE);
                irho = irho < 0 ? 0 : g.Nrho - 2;
            }
            const int nrint = g.Nrho - 1;
            double fp;
            if (!MIXED)
            {
                const double b = qr - irho;
                const double4_32a tf = g.pk_F[(size_t)ei * nrint + irho];
                fp = spl_der(tf, b, g.inv_drho);
                acc[0] = spl_val(tf, b);
            }
            else
            {
                const float b = (float)(qr - irho);
                const float4 tf = g.pkf_F[(size_t)ei * nrint + irho];
                const float f32 = spl_der(tf, b, (float)g.inv_drho);
                g.fpb[t] = f32;
                // lean (one kind: the kind bits are unused): F'(rho) also
                // rides in the w of the slot's list position, so the force
                // walk reads it with the neighbour's position (one gather
                // per pair instead of two); the next step start rewrites w
                if (LEAN) reinterpret_cast<float *>(g.xl + t)[3] = f32;
                fp = (double)f32;
                acc[0] = (double)spl_val(tf, b);
            }
            g.vaream[i] = fp;
            g.fpd[t] = fp;
            if (!MIXED) g.fpdf[t] = df_split(fp);
        }
        else
        {
            g.vaream[i] = 0.0;
            g.fpd[t] = 0.0;
            g.fpb[t] = 0.f;
            if (LEAN) reinterpret_cast<float *>(g.xl + t)[3] = 0.f;
            if (!MIXED) g.fpdf[t] = make_float2(0.f, 0.f);
        }
    }
    if (loc_thermo(loc, g)) block_reduce_store<1>(acc, g.partials + (size_t)nb * 8 + bx);
}

// Pair forces + velocity-Verlet finish step (src/integrators.c:94-126) and
// the thermo record, one thread per slot; the forces are stored in the
// current order for the next start step.  LEAN (binary32, one kind, no
// group): pair parameters in registers, no per-entry kind or group
// lookups, hardware exp2 / rsqrt / rcp approximations.
template <class L, int CAT, bool MIXED, bool LEAN>
__global__ void __launch_bounds__(L::max_threads, LEAN ? L::lean_min_blocks : L::min_blocks) k_force_skin(__grid_constant__ const L loc, int finish)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    const int group = g.st.group;
    const double dt = g.st.dt;
    __shared__ SmemPotT<!MIXED, LEAN> sp;
    __shared__ SkinOffT<!MIXED || !LEAN> so;   // lean binary32 kernels: no remainders (exact on a cubic grid)
    load_pot(g, sp, skin_params(g));
    load_offsets(g, so);
    Dyn *dyn = g.dyn;
    const Side S = g.side[dyn->cur];
    const int cap = g.cap;
    const int t = bx * blockDim.x + threadIdx.x;
    const bool thermo = loc_thermo(loc, g);
    // pe, m v^2, m v (3), count, pair virial
    double acc[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    const int i = (t < cap) ? g.pos[t] : -1;
    if (i >= 0)
    {
        float4 xi = g.xl[t];
        const int ki = LEAN ? 0 : __float_as_int(xi.w);   // (lean EAM: w holds F'(rho))
        const bool active = (group < 0 || g.gslot[t] == group);
        const int nk = g.nkinds;
        double f[3] = {0.0, 0.0, 0.0};
        double pe = 0.0, vir = 0.0;
        if (active)
        {
            const int nint = g.Nr2 - 1;
            const size_t ne = g.nelem;
            if (!MIXED)
            {
                // double-float pair arithmetic (fmdg_df.cuh, df_pair)
                const float4 ih = g.xl[t], il = g.xll[t];
                const dfl fpi = (CAT == CAT_EAM || CAT == CAT_HYBRID) ? df_of(g.fpdf[t]) : dfl{0.f, 0.f};
                const dfl inv_h = df_of(df_split(g.inv_dr2));
                const float kmax = (float)(nint - 1);
                dfl fs[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}}, pes = {0.f, 0.f}, virs = {0.f, 0.f};
                for_each_slot_pair(g, S, so, t, i, xi, [&](int js, float4 xjf, float4 o) {
                    if (group >= 0 && g.gslot[js] != group) return;
                    const int pidx = ki * nk + __float_as_int(xjf.w);
                    const fmdg_pair_t &pp = sp.pairs[pidx];
                    const int cat = (CAT == CAT_HYBRID) ? pp.cat : CAT;
                    const int rci = (cat == FMDG_POT_MORSE) ? 3 : 2;
                    const GeomDF p = skin_geom_df(g, so, t, ih, il, js, xjf, o);
                    if (!within_cut_df_mi(g, t, js, p.r2, sp.pf[pidx][rci], pp.p[rci])) return;
                    dfl fa, eh;
                    df_pair(g, sp, pidx, pp, cat, p, fpi, inv_h, kmax, nint, ne, [&]() { return df_of(g.fpdf[js]); },
                            fa, eh);
                    for (int d = 0; d < 3; d++) fs[d] = df_add(fs[d], df_mul(fa, p.rv[d]));
                    pes = df_add(pes, eh);
                    virs = df_add(virs, df_mul(fa, p.r2));     // rv . (fa rv), both sides of the pair
                });
                for (int d = 0; d < 3; d++) f[d] = df_to_double(fs[d]);
                pe = df_to_double(pes);
                vir = 0.5 * df_to_double(virs);
            }
            else if constexpr (LEAN)
            {
                const float4 pq = make_float4(sp.pf[0][0], sp.pf[0][1], sp.pf[0][2], sp.pf[0][3]);
                const float rc2f = (CAT == CAT_MORSE) ? pq.w : pq.z;
                const double rc2 = (CAT == CAT_MORSE) ? sp.pairs[0].p[3] : sp.pairs[0].p[2];
                // scaled frame (Geo::xs; pq holds scaled parameters): real
                // force factors from scaled geometry.  Morse: 2^((r0' - r')
                // alpha' log2 e) with alpha' = alpha / xs, r0' = r0 xs, factor
                // 2 alpha D0 xs = 2 alpha' D0 xs^2; LJ: 12 eps4 xs^2 / r'^2
                const float xs2 = scaled_xs2(g);
                const float m_c1 = pq.y * 1.44269504f, m_c2 = 2.f * pq.y * pq.x * xs2;
                const float lj_c = 12.f * pq.x * xs2;
                const float fpi = (CAT == CAT_EAM) ? g.fpb[t] : 0.f;
                const float inv_h = (float)g.inv_dr2;         // derivatives with respect to the real r^2
                const float inv_hi = scaled_index_factor(g);  // table index of the scaled r^2
                const float kmax = (float)(nint - 1);
                const int ee = sp.pairs[0].iloc;
                const float4 *tpr = g.pkf_pr + (size_t)ee * nint * 2;
                // LJ / Morse pair: force factor and half energy
                auto pair_lm = [&](float r2, float &fa, float &e) {
                    if (CAT == CAT_LJ)
                    {
                        const float inv_r2 = rcp_approx(r2);
                        const float s2 = pq.y * inv_r2;
                        const float s6 = s2 * s2 * s2;
                        const float s12 = s6 * s6;
                        fa = lj_c * inv_r2 * (s12 - 0.5f * s6);
                        e = 0.5f * (pq.x * (s12 - s6));
                    }
                    else
                    {
                        const float inv_r = rsqrt_approx(r2);
                        const float r = r2 * inv_r;
                        const float e1 = ex2_approx((pq.z - r) * m_c1);
                        const float e2 = e1 * e1;
                        fa = m_c2 * inv_r * (e2 - e1);
                        e = 0.5f * (pq.x * (e2 - 2.f * e1));
                    }
                };
                // E: the walk sums the energy, V: the pair virial (rv . F =
                // fa r^2); both on steps that form the thermo record only
                // (the EAM walk keeps its energy term on every step)
                auto walk = [&](auto with_e, auto with_v) {
                    constexpr bool E = decltype(with_e)::value;
                    constexpr bool V = decltype(with_v)::value;
                    constexpr int NA = V ? 5 : (E ? 4 : 3);
                    Acc32<NA> ac;
                    if constexpr (CAT == CAT_EAM)
                    {
                        const float band = 1e-4f * rc2f;
                        for_each_slot_pair<false>(g, S, so, t, i, xi, [&](int js, float4 xj, float4 o) {
                            const float3 rv = rv_of(xi, xj, o);
                            const float r2 = rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
                            bool in = r2 < rc2f;
                            if (fabsf(r2 - rc2f) <= band) in = geom64_mi(g, g.xd[t], g.xd[js]).r2 < rc2;
                            if (!in) return;
                            float b;
                            const int ir2 = table_index(r2 * inv_hi, kmax, b);
                            float4 tph, trh;
                            ld_row32(tpr + 2 * ir2, tph, trh);
                            const float phi_d = spl_der(tph, b, inv_h);
                            const float rho_d = spl_der(trh, b, inv_h);
                            // F'(rho_j): w of the list position; an overflow
                            // fallback occurrence (code < 0) carries kind bits
                            const float fpj = __float_as_int(o.w) >= 0 ? xj.w : g.fpb[js];
                            const float fa = -2.f * (fpi * rho_d + fpj * rho_d + phi_d);
                            ac.part[0] += fa * rv.x;
                            ac.part[1] += fa * rv.y;
                            ac.part[2] += fa * rv.z;
                            if constexpr (E) ac.part[3] += 0.5f * spl_val(tph, b);
                            if constexpr (V) ac.part[NA - 1] += fa * r2;
                        }, [&](int k) { ac.entries(k); });
                        ac.flush();
                    }
                    else
                    {
                        // Branch-free walk: the arithmetic runs for every entry and
                        // entries beyond the cutoff add zero.  An entry within
                        // 2e-5 relative of the cutoff (several times the binary32
                        // error of r^2) is decided in binary64 after the walk: one
                        // such entry per atom is kept in registers, more (rare)
                        // send the atom through a second walk over its near
                        // entries only.
                        const float band = 2e-5f * rc2f;
                        int npend = 0, pend = 0;
                        float3 prv = make_float3(0.f, 0.f, 0.f);
                        for_each_slot_pair<true>(g, S, so, t, i, xi, [&](int js, float4 xj, float4 o) {
                            const float3 rv = rv_of(xi, xj, o);
                            const float r2 = rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
                            const bool near = fabsf(r2 - rc2f) <= band;
                            const bool in = (r2 < rc2f) && !near;
                            npend += near;
                            pend = near ? js : pend;
                            prv = near ? rv : prv;
                            float fa, e;
                            pair_lm(r2, fa, e);
                            fa = in ? fa : 0.f;
                            e = in ? e : 0.f;
                            ac.part[0] += fa * rv.x;
                            ac.part[1] += fa * rv.y;
                            ac.part[2] += fa * rv.z;
                            if constexpr (E) ac.part[3] += e;
                            if constexpr (V) ac.part[NA - 1] += fa * r2;
                        }, [&](int k) { ac.entries(k); });
                        ac.flush();
                        if (npend == 1)
                        {
                            if (geom64_mi(g, g.xd[t], g.xd[pend]).r2 < rc2)
                            {
                                const float r2 = prv.x * prv.x + prv.y * prv.y + prv.z * prv.z;
                                float fa, e;
                                pair_lm(r2, fa, e);
                                ac.part[0] += fa * prv.x;
                                ac.part[1] += fa * prv.y;
                                ac.part[2] += fa * prv.z;
                                if constexpr (E) ac.part[3] += e;
                                if constexpr (V) ac.part[NA - 1] += fa * r2;
                                ac.flush();
                            }
                        }
                        else if (npend > 1)
                        {
                            for_each_slot_pair<false>(g, S, so, t, i, xi, [&](int js, float4 xj, float4 o) {
                                const float3 rv = rv_of(xi, xj, o);
                                const float r2 = rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
                                if (!(fabsf(r2 - rc2f) <= band)) return;
                                if (!(geom64_mi(g, g.xd[t], g.xd[js]).r2 < rc2)) return;
                                float fa, e;
                                pair_lm(r2, fa, e);
                                ac.part[0] += fa * rv.x;
                                ac.part[1] += fa * rv.y;
                                ac.part[2] += fa * rv.z;
                                if constexpr (E) ac.part[3] += e;
                                if constexpr (V) ac.part[NA - 1] += fa * r2;
                            }, [&](int k) { ac.entries(k); });
                            ac.flush();
                        }
                    }
                    for (int d = 0; d < 3; d++) f[d] = ac.total(d);
                    if constexpr (E) pe = ac.total(3);
                    if constexpr (V) vir = 0.5 * ac.total(NA - 1);
                };
                // (the EAM walk keeps its energy term: dropping it measured
                // slower for that kernel)
                if (thermo)
                    walk(std::true_type{}, std::true_type{});
                else if constexpr (CAT == CAT_EAM)
                    walk(std::true_type{}, std::false_type{});
                else
                    walk(std::false_type{}, std::false_type{});
            }
            else
            {
                const float fpi = (CAT == CAT_EAM || CAT == CAT_HYBRID) ? g.fpb[t] : 0.f;
                const float inv_h = (float)g.inv_dr2;         // derivatives with respect to the real r^2
                const float inv_hi = scaled_index_factor(g);  // table index of the scaled r^2
                const float kmax = (float)(nint - 1);
                const float xs2 = scaled_xs2(g);
                Acc32<5> ac;
                for_each_slot_pair(g, S, so, t, i, xi, [&](int js, float4 xj, float4 o) {
                    if (group >= 0 && g.gslot[js] != group) return;
                    const int pidx = ki * nk + __float_as_int(xj.w);
                    const fmdg_pair_t &pp = sp.pairs[pidx];
                    const int cat = (CAT == CAT_HYBRID) ? pp.cat : CAT;
                    const float3 rv = rv_lo(so, xi, xj, o);
                    const float r2 = rv.x * rv.x + rv.y * rv.y + rv.z * rv.z;
                    if (cat == FMDG_POT_LJ)
                    {
                        if (within_cut_skin(g, t, js, r2, sp.pf[pidx][2], pp.p[2]))
                        {
                            float fa, e;
                            lj_pair(r2, sp.pf[pidx][0], sp.pf[pidx][1], fa, e);
                            fa *= xs2;         // the real force factor (scaled frame)
                            ac.part[0] += rv.x * fa;
                            ac.part[1] += rv.y * fa;
                            ac.part[2] += rv.z * fa;
                            ac.part[3] += e;
                            ac.part[4] += fa * r2;
                        }
                    }
                    else if (cat == FMDG_POT_MORSE)
                    {
                        if (within_cut_skin(g, t, js, r2, sp.pf[pidx][3], pp.p[3]))
                        {
                            float fa, e;
                            morse_pair(r2, sp.pf[pidx][0], sp.pf[pidx][1], sp.pf[pidx][2], fa, e);
                            fa *= xs2;         // the real force factor (scaled frame)
                            ac.part[0] += fa * rv.x;
                            ac.part[1] += fa * rv.y;
                            ac.part[2] += fa * rv.z;
                            ac.part[3] += e;
                            ac.part[4] += fa * r2;
                        }
                    }
                    else if (cat == FMDG_POT_EAM)
                    {
                        if (within_cut_skin(g, t, js, r2, sp.pf[pidx][2], pp.p[2]))
                        {
                            float b;
                            const int ir2 = table_index(r2 * inv_hi, kmax, b);
                            const int ei = pp.iloc, ej = pp.jloc;
                            const float4 tph = g.pkf_phi[((size_t)ei * ne + ej) * nint + ir2];
                            const float phi_d = spl_der(tph, b, inv_h);
                            const float rho_ip = spl_der(g.pkf_rho[(size_t)ei * nint + ir2], b, inv_h);
                            const float rho_jp = (ei == ej) ? rho_ip
                                               : spl_der(g.pkf_rho[(size_t)ej * nint + ir2], b, inv_h);
                            const float mag = 2.f * (fpi * rho_jp + g.fpb[js] * rho_ip + phi_d);
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
        if (MIXED)
        {
            // binary32 pairs were summed in the scaled frame (Geo::xs): the
            // real force is the sum over xs, the real virial over xs^2
            for (int d = 0; d < 3; d++) f[d] *= g.inv_xs;
            vir *= g.inv_xs * g.inv_xs;
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
                    f[2] += g.ttm_xi[it] * sp.mass[ki] * (S.v[2 * (size_t)cap + i] - g.ttm_vcm[3 * it + 2]);
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
            if (thermo)
            {
                acc[1] = m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                acc[2] = m * v[0];
                acc[3] = m * v[1];
                acc[4] = m * v[2];
                acc[5] = 1.0;
            }
        }
    }
    __shared__ double blk[7];
    __shared__ unsigned ticket;
    if (thermo) block_reduce_store<7>(acc, blk);
    if (threadIdx.x == 0)
    {
        if (thermo)
            for (int k = 0; k < 7; k++) g.partials[(size_t)k * nb + bx] = blk[k];
        __threadfence();
        ticket = atomicAdd(&dyn->blocks_done, 1u);
    }
    __syncthreads();
    if (ticket == (unsigned)nb - 1)
    {
        __threadfence();
        if (thermo) final_reduce(g, nb, 0, g.has_eam, g.st.thermostat, dt, g.st.tau, g.st.T0);
        if (threadIdx.x == 0)
        {
            dyn->blocks_done = 0;
            if (finish && dyn->steps_left > 0) dyn->steps_left--;
        }
    }
}

// lean: one kind and no group (used in binary32 only)
template <class L, bool MIXED>
void launch_force_skin(const L &loc, int cats, int finish, int nb, int blk, cudaStream_t st, bool lean)
{
    const int ncat = __builtin_popcount(cats);
    if (ncat > 1) k_force_skin<L, CAT_HYBRID, MIXED, false><<<nb, blk, 0, st>>>(loc, finish);
    else if (MIXED && lean)
    {
        if (cats == (1 << FMDG_POT_LJ)) k_force_skin<L, CAT_LJ, true, true><<<nb, blk, 0, st>>>(loc, finish);
        else if (cats == (1 << FMDG_POT_MORSE)) k_force_skin<L, CAT_MORSE, true, true><<<nb, blk, 0, st>>>(loc, finish);
        else k_force_skin<L, CAT_EAM, true, true><<<nb, blk, 0, st>>>(loc, finish);
    }
    else if (cats == (1 << FMDG_POT_LJ)) k_force_skin<L, CAT_LJ, MIXED, false><<<nb, blk, 0, st>>>(loc, finish);
    else if (cats == (1 << FMDG_POT_MORSE)) k_force_skin<L, CAT_MORSE, MIXED, false><<<nb, blk, 0, st>>>(loc, finish);
    else k_force_skin<L, CAT_EAM, MIXED, false><<<nb, blk, 0, st>>>(loc, finish);
}

template <class L>
void launch_density_skin(const L &loc, bool mixed, bool hyb, int nb, int blk, cudaStream_t st, bool lean)
{
    if (mixed)
    {
        if (hyb) k_density_skin<L, true, true, false><<<nb, blk, 0, st>>>(loc);
        else if (lean) k_density_skin<L, true, false, true><<<nb, blk, 0, st>>>(loc);
        else k_density_skin<L, true, false, false><<<nb, blk, 0, st>>>(loc);
    }
    else
    {
        if (hyb) k_density_skin<L, false, true, false><<<nb, blk, 0, st>>>(loc);
        else k_density_skin<L, false, false, false><<<nb, blk, 0, st>>>(loc);
    }
}

} // namespace

int fmdg_pack_launch_start(const fmdg_pack_launch &P)
{
    k_skin_start<<<P.la.bstart[P.nsys], 128, 0, P.stream>>>(P.la);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return -fmdg_fail("pack start", e);
    return 1;
}

// phases: bit 0 slot tables + list (re)build, bit 1 EAM density, bit 2
// pair forces + finish step (all three for a step).  Returns the kernels
// launched, or minus a status.
int fmdg_pack_launch_forces(const fmdg_pack_launch &P, int phases)
{
    cudaStream_t st = P.stream;
    const int nab = P.la.bstart[P.nsys], nfb = P.lf.bstart[P.nsys];
    int n = 0;
    if (phases & 1)
    {
        k_prep_skin<<<nab, 128, 0, st>>>(P.la, 1);
        k_nlist_skin<<<nfb, P.fblk, 0, st>>>(P.lf);
        n += 2;
    }
    if ((phases & 2) && (P.cats & (1 << FMDG_POT_EAM)))
    {
        launch_density_skin(P.lf, P.mixed != 0, __builtin_popcount(P.cats) > 1, nfb, P.fblk, st, P.lean != 0);
        n++;
    }
    if (phases & 4)
    {
        if (P.mixed) launch_force_skin<LocPack, true>(P.lf, P.cats, 1, nfb, P.fblk, st, P.lean != 0);
        else launch_force_skin<LocPack, false>(P.lf, P.cats, 1, nfb, P.fblk, st, false);
        n++;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return -fmdg_fail("pack forces", e);
    return n;
}

// The single-system path on a skin list (fmdg_launch_nlist/density/
// pair_forces dispatch here when the system has one): slot tables + list
// (re)build; EAM density; pair forces (+ finish step).
int fmdg_skin_launch_nlist(fmdg_sys_t *s)
{
    const LocOne L{s->g};
    k_prep_skin<<<fmdg_grid(s->g.cap, 128), 128, 0, s->stream>>>(L, 0);
    // lanes per slot by size, from build times measured on GB300 (LJ,
    // Morse, EAM jobs of 2k-190k atoms): 16 up to 2^14 slots, 8 up to 2^16,
    // then one thread per slot (enough warps; a group's ballots cost more
    // than they hide).  Groups of 2 or 4 lanes never won: the lanes of
    // different groups in a warp diverge and serialise.
    const int cap = s->g.cap;
    int G = s->build_lanes;
    if (G == 0) G = cap <= (1 << 14) ? 16 : (cap <= (1 << 16) ? 8 : 1);
    const int nbg = fmdg_grid(cap > 0 ? cap * G : 1, 128);
    switch (G)
    {
    case 2: k_nlist_skin_grp<2><<<nbg, 128, 0, s->stream>>>(L); break;
    case 4: k_nlist_skin_grp<4><<<nbg, 128, 0, s->stream>>>(L); break;
    case 8: k_nlist_skin_grp<8><<<nbg, 128, 0, s->stream>>>(L); break;
    case 16: k_nlist_skin_grp<16><<<nbg, 128, 0, s->stream>>>(L); break;
    case 32: k_nlist_skin_grp<32><<<nbg, 128, 0, s->stream>>>(L); break;
    default: k_nlist_skin<<<fmdg_force_blocks(s), s->fblk, 0, s->stream>>>(L); break;
    }
    s->launches += 2;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

// one kind and every atom in the step's group: the lean kernels
static bool lean_system(const fmdg_sys_t *s) { return s->nkinds == 1 && s->g.st.group < 0; }

int fmdg_skin_launch_density(fmdg_sys_t *s)
{
    launch_density_skin(LocOne{s->g}, s->g.prec == FMDG_PREC_MIXED, __builtin_popcount(s->cats) > 1,
                        fmdg_force_blocks(s), s->fblk, s->stream, lean_system(s));
    s->launches++;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

int fmdg_skin_launch_pair_forces(fmdg_sys_t *s, int finish)
{
    const LocOne L{s->g};
    const int nb = fmdg_force_blocks(s);
    if (s->g.prec == FMDG_PREC_MIXED)
        launch_force_skin<LocOne, true>(L, s->cats, finish, nb, s->fblk, s->stream, lean_system(s));
    else launch_force_skin<LocOne, false>(L, s->cats, finish, nb, s->fblk, s->stream, false);
    s->launches++;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}
