// Cell-list refresh on the GPU with the reference's cell assignment and
// in-cell atom order.
//
// Reference behaviour being reproduced (FMD 0.4.0, one subdomain):
//  * src/misc.c:268-308 `_fmd_refreshGrid`: interior cells are visited in
//    storage order; inside a cell, atom i is re-binned with
//    floor(x/cellh)+1 (local index incl. the one-cell ghost margin); a
//    departing atom is appended to its destination cell and removed from
//    its source by swap-with-last (src/cell.c:151-160, src/cell.h:84-95), so
//    the atom moved into slot i is examined next.
//  * src/md-ghost.c:827-869 `_fmd_particles_migrate`: for d = 0,1,2, the
//    lower ghost layer then the upper one hand their whole lists (appended,
//    x[d] -/+ l[d]) to the opposite interior layer (periodic) or are
//    discarded (open boundary).
//
// Parallel restatement.  Destinations do not depend on order, so they are
// computed per atom first.  The order then follows from three facts:
//  (1) a cell's departure sequence depends only on its own list and on the
//      NUMBER A of atoms that arrived from lower-index cells before it was
//      visited (arrivals never depart again) -- one thread per cell replays
//      the swap-remove walk with A placeholder tokens in O(1) state, because
//      only the scan position can hold a moved element;
//  (2) arrivals into a cell D are ordered by (source cell, departure rank);
//      the first A of them fill the placeholder slots, the rest are appended;
//  (3) atoms that passed through ghost cells arrive after all interior
//      arrivals, ordered by the pass of their last hop, then by their
//      position in that ghost cell's list, which is itself (direct arrivals
//      by (source, rank)) followed by earlier-pass arrivals -- a fixed-width
//      key of the pass sequence read from the last hop backwards.
// Each destination cell sorts its (few) arrivals by that key, after which
// every atom knows its new index and one scatter writes the next side.
#include "fmdg_internal.cuh"

namespace {

__device__ __forceinline__ int cell_flat(const Geo &g, int x, int y, int z)
{
    return z + g.nc[2] * (y + g.nc[1] * x);
}

// Start-of-step update fused with the binning decision.
//  mode VV: src/integrators.c:40-75 (v *= lambda; v += dt*0.5/m*F; x += dt*v)
//  mode SE: src/integrators.c:129-152 (v += dt*F/m; x += dt*v)
// Explicit _rn intrinsics keep the reference's operation order with no
// fused multiply-add, so positions and velocities match bit for bit given
// the same forces.  lazy (packed systems, mode REFRESH_ONLY): the cells are
// refreshed only on a step that rebuilds the skin list.
template <class L>
__global__ void k_bin_classify(__grid_constant__ const L loc, int mode, int lazy)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    if (lazy && !g.dyn->rebuild) return;
    const double dt = g.st.dt;
    const int group = g.st.group, thermostat = g.st.thermostat;
    // half kick dt * 0.5 / m per kind, formed on the host (set_step_dt):
    // the reference's operations, so the same bits as per atom
    __shared__ double hk[FMDG_MAXK];
    if (threadIdx.x < g.nkinds) hk[threadIdx.x] = g.st.hk[threadIdx.x];
    __syncthreads();
    Dyn *dyn = g.dyn;
    const int n = dyn->n;
    const int i = bx * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Side S = g.side[dyn->cur];
    const int cap = g.cap;

    double x[3], v[3];
    for (int d = 0; d < 3; d++) { x[d] = S.x[d * cap + i]; v[d] = S.v[d * cap + i]; }

    if (mode != FMDG_REFRESH_ONLY && (group < 0 || S.group[i] == group))
    {
        const int k = S.kind[i];
        const double m = g.mass[k];
        if (mode == FMDG_REFRESH_VV)
        {
            const double lam = dyn->lambda;
            const double coef = hk[k];
            for (int d = 0; d < 3; d++)
            {
                double vv = v[d];
                if (thermostat) vv = __dmul_rn(vv, lam);
                vv = __dadd_rn(vv, __dmul_rn(coef, g.F[d * cap + i]));
                v[d] = vv;
                x[d] = __dadd_rn(x[d], __dmul_rn(dt, vv));
            }
        }
        else
        {
            for (int d = 0; d < 3; d++)
            {
                double vv = __dadd_rn(v[d], __ddiv_rn(__dmul_rn(dt, g.F[d * cap + i]), m));
                v[d] = vv;
                x[d] = __dadd_rn(x[d], __dmul_rn(dt, vv));
            }
        }
        for (int d = 0; d < 3; d++) S.v[d * cap + i] = v[d];
    }

    const int c = S.cell_of[i];
    const int cc[3] = { c / (g.nc[1] * g.nc[2]), (c / g.nc[2]) % g.nc[1], c % g.nc[2] };
    int jc[3];
    bool departs = false, outside = false;
    for (int d = 0; d < 3; d++)
    {
        const int q = cell_floor(x[d], g.cellh[d], g.inv_cellh[d], g.inv_cellh_f[d]);
        // local index including the ghost margin (ic_start = 1)
        if (!(q >= -1 && q <= g.nc[d])) outside = true;
        jc[d] = outside ? 0 : q + 1;
        if (jc[d] - 1 != cc[d]) departs = true;
    }
    if (outside)
    {
        // src/misc.c:286-290 raises FMD_ERR_UNEXPECTED_POSITION; the atom is
        // left where it is so no index leaves the grid
        atomic_or_err(dyn, FMDG_ERRBIT_POSITION);
        for (int d = 0; d < 3; d++) S.x[d * cap + i] = x[d];
        g.bdest[i] = -2;
        return;
    }
    if (!departs)
    {
        for (int d = 0; d < 3; d++) S.x[d * cap + i] = x[d];
        g.bdest[i] = -2;
        return;
    }

    // migration path through the ghost margin (src/md-ghost.c:827-869)
    int q[3] = {0, 0, 0};
    int nq = 0;
    bool deleted = false;
    for (int d = 0; d < 3; d++)
    {
        if (jc[d] == 0 || jc[d] == g.nc[d] + 1)
        {
            const bool upper = (jc[d] != 0);
            if (!g.pbc[d]) deleted = true;
            q[nq++] = 1 + 2 * d + (upper ? 1 : 0);
            if (upper) { jc[d] = 1;          x[d] = __dadd_rn(x[d], -g.l[d]); }
            else       { jc[d] = g.nc[d];    x[d] = __dadd_rn(x[d],  g.l[d]); }
        }
    }
    atomicAdd(&g.dep_count[c], 1);
    dyn->any_move = 1;
    if (deleted)
    {
        g.bdest[i] = -1;
        if (g.skin_on)
        {
            // the slot is gone: its list entries must go too
            g.pos[S.slot[i]] = -1;
            dyn->rebuild = 1;
        }
        return;
    }
    for (int d = 0; d < 3; d++) S.x[d * cap + i] = x[d];
    const int D = cell_flat(g, jc[0] - 1, jc[1] - 1, jc[2] - 1);
    // key bits: [9] migrated, [8:6] last pass, [5:3] previous, [2:0] first
    int path = 0;
    if (nq > 0)
    {
        path = 1 << 9;
        int shift = 6;
        for (int k = nq - 1; k >= 0; k--, shift -= 3) path |= q[k] << shift;
    }
    g.bpath[i] = path;
    g.bdest[i] = D;
    atomicAdd(&g.arr_total[D], 1);
    if (nq == 0 && c < D) atomicAdd(&g.arr_lower[D], 1);
}

// Exclusive scans over cells (one block): arrival bases and the next side's
// cell_start, plus the atom count after the refresh.
template <class L>
__global__ void k_bin_scan(__grid_constant__ const L loc)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    Dyn *dyn = g.dyn;
    if (!dyn->any_move) return;
    const Side S = g.side[dyn->cur];
    const Side T = g.side[dyn->cur ^ 1];
    const int nc = g.ncell;
    __shared__ int sa[1024], sn[1024];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int per = (nc + nt - 1) / nt;
    const int lo = min(nc, tid * per), hi = min(nc, lo + per);
    int ta = 0, tn = 0;
    for (int c = lo; c < hi; c++)
    {
        ta += g.arr_total[c];
        tn += S.cell_start[c + 1] - S.cell_start[c] - g.dep_count[c] + g.arr_total[c];
    }
    sa[tid] = ta; sn[tid] = tn;
    __syncthreads();
    for (int off = 1; off < nt; off <<= 1)
    {
        int va = 0, vn = 0;
        if (tid >= off) { va = sa[tid - off]; vn = sn[tid - off]; }
        __syncthreads();
        sa[tid] += va; sn[tid] += vn;
        __syncthreads();
    }
    int ra = sa[tid] - ta, rn = sn[tid] - tn;
    for (int c = lo; c < hi; c++)
    {
        g.arr_base[c] = ra;
        T.cell_start[c] = rn;
        ra += g.arr_total[c];
        rn += S.cell_start[c + 1] - S.cell_start[c] - g.dep_count[c] + g.arr_total[c];
    }
    if (tid == nt - 1)
    {
        g.arr_base[nc] = sa[tid];
        T.cell_start[nc] = sn[tid];
        dyn->n_next = sn[tid];
    }
}

// Replay of the swap-remove walk of one source cell (src/misc.c:276-303)
// with A placeholder tokens for the atoms that arrived from lower-index
// cells.  Emits the departure rank of each leaving atom (and queues it in
// its destination's bucket), the final slot of each stayer, and the slot of
// each placeholder.
template <class L>
__global__ void k_bin_cells(__grid_constant__ const L loc)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    Dyn *dyn = g.dyn;
    if (!dyn->any_move) return;
    const int c = bx * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return;
    const Side S = g.side[dyn->cur];
    const int start = S.cell_start[c];
    const int n0 = S.cell_start[c + 1] - start;
    const int A = g.arr_lower[c];
    const int base = g.arr_base[c];
    if (g.dep_count[c] == 0)
    {
        for (int k = 0; k < A; k++) g.arr_slot[base + k] = n0 + k;
        return;
    }
    int len = n0 + A, i = 0, moved = -1, rank = 0;
    while (i < len)
    {
        const int tok = (moved >= 0) ? moved : i;
        const int a = start + tok;
        if (tok < n0 && g.bdest[a] != -2)
        {
            const int D = g.bdest[a];
            g.brank[a] = rank++;
            if (D >= 0)
            {
                const int pos = atomicAdd(&g.bucket_fill[D], 1);
                g.bucket[g.arr_base[D] + pos] = a;
            }
            len--;
            // the old last element (never overwritten: only the scan
            // position is) moves into slot i
            moved = (len != i) ? len : -1;
        }
        else
        {
            if (tok < n0) g.bslot[a] = i;
            else g.arr_slot[base + (tok - n0)] = i;
            i++;
            moved = -1;
        }
    }
}

// Order the arrivals of each destination cell and give them new indexes.
template <class L>
__global__ void k_bin_arrivals(__grid_constant__ const L loc)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    Dyn *dyn = g.dyn;
    if (!dyn->any_move) return;
    const int D = bx * blockDim.x + threadIdx.x;
    if (D >= g.ncell) return;
    const int total = g.arr_total[D];
    if (total == 0) return;
    const Side S = g.side[dyn->cur];
    const Side T = g.side[dyn->cur ^ 1];
    const int base = g.arr_base[D];
    int *b = g.bucket + base;
    auto key = [&](int a) -> unsigned long long {
        return ((unsigned long long)g.bpath[a] << 44) |
               ((unsigned long long)S.cell_of[a] << 20) |
               (unsigned long long)g.brank[a];
    };
    for (int k = 1; k < total; k++)
    {
        const int a = b[k];
        const unsigned long long ka = key(a);
        int j = k - 1;
        while (j >= 0 && key(b[j]) > ka) { b[j + 1] = b[j]; j--; }
        b[j + 1] = a;
    }
    const int A = g.arr_lower[D];
    const int nstay = S.cell_start[D + 1] - S.cell_start[D] - g.dep_count[D];
    const int ns = T.cell_start[D];
    for (int k = 0; k < total; k++)
    {
        const int a = b[k];
        g.bnewidx[a] = ns + (k < A ? g.arr_slot[base + k] : nstay + A + (k - A));
    }
}

template <class L>
__global__ void k_bin_scatter(__grid_constant__ const L loc)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    Dyn *dyn = g.dyn;
    if (!dyn->any_move) return;
    const int i = bx * blockDim.x + threadIdx.x;
    if (i >= dyn->n) return;
    const int d = g.bdest[i];
    if (d == -1) return;
    const Side S = g.side[dyn->cur];
    const Side T = g.side[dyn->cur ^ 1];
    const int c = S.cell_of[i];
    int idx, D;
    if (d == -2)
    {
        D = c;
        idx = T.cell_start[c] + (g.dep_count[c] == 0 ? (i - S.cell_start[c]) : g.bslot[i]);
    }
    else
    {
        D = d;
        idx = g.bnewidx[i];
    }
    if (idx < 0 || idx >= dyn->n_next)
    {
        // cannot happen for a consistent refresh; recorded instead of writing
        atomic_or_err(dyn, FMDG_ERRBIT_INTERNAL);
        return;
    }
    const int cap = g.cap;
    for (int k = 0; k < 3; k++)
    {
        T.x[k * cap + idx] = S.x[k * cap + i];
        T.v[k * cap + idx] = S.v[k * cap + i];
    }
    T.kind[idx] = S.kind[i];
    T.group[idx] = S.group[i];
    T.atomid[idx] = S.atomid[i];
    T.cell_of[idx] = D;
    if (g.skin_on) T.slot[idx] = S.slot[i];
}

// swaps sides after a refresh that moved atoms; advances the device copy of
// the simulation time by one step (src/integrators.c:203, :256)
template <class L>
__global__ void k_bin_flip(__grid_constant__ const L loc, int mode)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g) || threadIdx.x != 0) return;
    Dyn *dyn = g.dyn;
    dyn->time += (mode == FMDG_REFRESH_ONLY) ? 0.0 : g.st.dt;
    if (dyn->any_move)
    {
        dyn->cur ^= 1;
        dyn->n = dyn->n_next;
        dyn->any_move = 0;
    }
}

// per-cell binning counters of every system of a pack that refreshes its
// cells this step
__global__ void k_bin_clear(__grid_constant__ const LocPack loc)
{
    int bx, nb;
    const Geo &g = loc_geo(loc, bx, nb);
    if (loc_idle(loc, g)) return;
    if (!g.dyn->rebuild) return;
    const int c = bx * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return;
    g.dep_count[c] = 0;
    g.arr_lower[c] = 0;
    g.arr_total[c] = 0;
    g.bucket_fill[c] = 0;
}

} // namespace

// One refresh: optional integrator start step, then re-binning.  All
// launches go to the system's stream; graph-capturable (no host reads).
int fmdg_launch_refresh(fmdg_sys_t *s, int mode, double dt, int group, int thermostat)
{
    Geo &g = s->g;
    cudaStream_t st = s->stream;
    set_step_dt(s, dt);
    g.st.group = group;
    g.st.thermostat = thermostat;
    const LocOne L{g};
    // dep_count, arr_lower, arr_total, bucket_fill are contiguous
    FMDG_CK(cudaMemsetAsync(g.dep_count, 0, sizeof(int) * 4 * (size_t)g.ncell, st));
    k_bin_classify<<<fmdg_grid(g.cap, 256), 256, 0, st>>>(L, mode, 0);
    k_bin_scan<<<1, 1024, 0, st>>>(L);
    k_bin_cells<<<fmdg_grid(g.ncell, 128), 128, 0, st>>>(L);
    k_bin_arrivals<<<fmdg_grid(g.ncell, 128), 128, 0, st>>>(L);
    k_bin_scatter<<<fmdg_grid(g.cap, 256), 256, 0, st>>>(L);
    k_bin_flip<<<1, 32, 0, st>>>(L, mode);
    s->launches += 6;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

// Step start of every system of a pack: velocity-Verlet start step, slot
// tables and displacement test (fmdg_skin_launch_start), then the cell
// refresh of the systems that rebuild their skin list this step (between
// rebuilds an atom stays within skin/2 of its build position, less than a
// cell, and the packed kernels address atoms by slot, not by cell).
// Returns the kernels launched, or minus a status.
int fmdg_pack_launch_refresh(const fmdg_pack_launch &P)
{
    cudaStream_t st = P.stream;
    const int nab = P.la.bstart[P.nsys], ncb = P.lc.bstart[P.nsys];
    int n = fmdg_pack_launch_start(P);
    if (n < 0) return n;
    k_bin_clear<<<ncb, 128, 0, st>>>(P.lc);
    k_bin_classify<<<nab, 128, 0, st>>>(P.la, FMDG_REFRESH_ONLY, 1);
    k_bin_scan<<<P.nsys, 1024, 0, st>>>(P.ls);
    k_bin_cells<<<ncb, 128, 0, st>>>(P.lc);
    k_bin_arrivals<<<ncb, 128, 0, st>>>(P.lc);
    k_bin_scatter<<<nab, 128, 0, st>>>(P.la);
    k_bin_flip<<<P.nsys, 32, 0, st>>>(P.ls, FMDG_REFRESH_ONLY);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return -fmdg_fail("pack refresh", e);
    return n + 7;
}
