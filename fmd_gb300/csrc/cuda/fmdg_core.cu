// Device engine: system lifetime, uploads/downloads, step orchestration.
//
// A system owns one CUDA stream.  fmdg_vv_steps captures one
// velocity-Verlet step (refresh + forces + reductions, ~9 kernels) into a
// CUDA graph on first use and replays it once per step, so the host issues
// one graph launch per step and never waits inside the loop; it synchronises
// only when the caller reads results (thermo, errors, atoms).
#include <stdio.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <vector>
#include "fmdg_internal.cuh"
#include "fmdg_df.cuh"

static thread_local char g_errmsg[512] = "";

int fmdg_fail(const char *where, cudaError_t e)
{
    snprintf(g_errmsg, sizeof g_errmsg, "%s: %s", where, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? FMDG_E_NOMEM : FMDG_E_CUDA;
}

int fmdg_set_error(const char *msg)
{
    snprintf(g_errmsg, sizeof g_errmsg, "%s", msg);
    return FMDG_E_ARG;
}

extern "C" const char *fmdg_last_error(void) { return g_errmsg; }

extern "C" int fmdg_device_count(int *count)
{
    FMDG_CK(cudaGetDeviceCount(count));
    return FMDG_OK;
}

namespace {

// Device buffers are stream-ordered allocations on the system's stream from
// the device's default pool (kept cached), so creating and retiring
// systems never synchronises the device; the allocating call waits for its
// own stream only.
template <typename T>
int dalloc(fmdg_sys_t *s, T **p, size_t n)
{
    if (n == 0) n = 1;
    cudaError_t e = cudaMallocAsync((void **)p, n * sizeof(T), s->stream);
    if (e != cudaSuccess) return fmdg_fail("cudaMallocAsync", e);
    return FMDG_OK;
}

// Every transfer of a system goes through its own stream: its memory is
// allocated stream-ordered on that stream, and nothing else needs to wait.
// Host-to-device copies do not block on the device (a served job's set-up
// never waits behind the packed chunks queued on the GPU); device-to-host
// reads synchronise the system's stream.
int d2h_sync(fmdg_sys_t *s, void *dst, const void *src, size_t n)
{
    FMDG_CK(cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, s->stream));
    FMDG_CK(cudaStreamSynchronize(s->stream));
    return FMDG_OK;
}
#define FMDG_D2H(dst, src, n)                                            \
    do {                                                                 \
        const int r_ = d2h_sync(s, (dst), (src), (n));                   \
        if (r_) return r_;                                               \
    } while (0)

void dfree(fmdg_sys_t *s, void *p) { if (p) cudaFreeAsync(p, s->stream); }

void free_atoms(fmdg_sys_t *s)
{
    Geo &g = s->g;
    dfree(s, s->arena);
    s->arena = nullptr;
    for (int k = 0; k < 2; k++) memset(&g.side[k], 0, sizeof(Side));
    g.F = g.vaream = nullptr;
    g.xf4 = nullptr; g.nbr = nullptr; g.nbr_count = nullptr; g.fpf = nullptr;
    g.bdest = g.bpath = g.bslot = g.brank = g.bnewidx = nullptr;
    g.dep_count = g.arr_lower = g.arr_total = g.bucket_fill = g.arr_base = nullptr;
    g.bucket = g.arr_slot = nullptr;
    g.partials = nullptr;
    g.pos = g.cb = nullptr; g.xl = g.xb = nullptr; g.xd = nullptr; g.gslot = nullptr;
    g.fpb = nullptr; g.fpd = nullptr;
    g.cap = 0;
    s->atoms = false;
    if (s->graph_key_valid) { cudaGraphExecDestroy(s->graph); s->graph_key_valid = 0; }
}

// Lays the per-atom and per-cell buffers of a system out in one device
// allocation (256-byte aligned); a pass without a base measures it.
struct Carver
{
    char *base;
    size_t off;
    template <typename T>
    void take(T *&p, size_t n)
    {
        off = (off + 255) & ~(size_t)255;
        p = base ? (T *)(base + off) : nullptr;
        off += (n ? n : 1) * sizeof(T);
    }
};

// forget EAM tables that belong to another system
void drop_eam(fmdg_sys_t *s)
{
    Geo &g = s->g;
    g.eF = g.eFDD = g.erho = g.erhoDD = g.ephi = g.ephiDD = nullptr;
    g.pk_rho = g.pk_phi = g.pk_F = nullptr;
    g.pkf_rho = g.pkf_phi = g.pkf_F = g.pkf_pr = nullptr;
    g.pkd_rho = g.pkd_phi = nullptr;
    s->eam_borrowed = false;
}

void invalidate_graph(fmdg_sys_t *s)
{
    if (s->graph_key_valid) { cudaGraphExecDestroy(s->graph); s->graph_key_valid = 0; }
}

int read_dyn(fmdg_sys_t *s, Dyn *out)
{
    FMDG_CK(cudaMemcpyAsync(out, s->g.dyn, sizeof(Dyn), cudaMemcpyDeviceToHost, s->stream));
    FMDG_CK(cudaStreamSynchronize(s->stream));
    return FMDG_OK;
}

__global__ void k_add_velocity(Geo g, int group, double dx, double dy, double dz)
{
    const Dyn *dyn = g.dyn;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= dyn->n) return;
    const Side S = g.side[dyn->cur];
    if (group >= 0 && S.group[i] != group) return;
    S.v[i] += dx;
    S.v[g.cap + i] += dy;
    S.v[2 * g.cap + i] += dz;
}

__global__ void k_change_group(Geo g, int old_group, int new_group)
{
    const Dyn *dyn = g.dyn;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= dyn->n) return;
    const Side S = g.side[dyn->cur];
    if (old_group < 0 || S.group[i] == old_group) S.group[i] = new_group;
}

__global__ void k_flush(unsigned *buf, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        buf[i] = buf[i] * 1664525u + 1013904223u;
}

// d2f_rn (integer rounding) beside the conversion instruction
__global__ void k_d2f_check(const double *x, int n, float *ours, float *ref)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    ours[i] = d2f_rn(x[i]);
    ref[i] = __double2float_rn(x[i]);
}

// Independent FMA chains: the issue-rate ceiling of the CUDA cores for T.
template <typename T>
__global__ void k_fma_peak(T *out, int iters, T a, T b)
{
    T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++)
    {
        x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
        x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
    const T r = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (r == (T)12345.678) out[0] = r;
}

} // namespace

extern "C" int fmdg_check_d2f(fmdg_sys_t *s, const double *x, int n, float *ours, float *ref)
{
    if (n < 0) return fmdg_set_error("fmdg_check_d2f: negative count");
    if (n == 0) return FMDG_OK;
    double *dx = nullptr;
    float *d1 = nullptr, *d2 = nullptr;
    cudaError_t e = cudaMalloc(&dx, (size_t)n * 8);
    if (e == cudaSuccess) e = cudaMalloc(&d1, (size_t)n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&d2, (size_t)n * 4);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, (size_t)n * 8, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
    {
        k_d2f_check<<<fmdg_grid(n, 256), 256, 0, s->stream>>>(dx, n, d1, d2);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(ours, d1, (size_t)n * 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ref, d2, (size_t)n * 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(dx); cudaFree(d1); cudaFree(d2);
    return e == cudaSuccess ? FMDG_OK : fmdg_fail("fmdg_check_d2f", e);
}

extern "C" int fmdg_measure_fma_peak(fmdg_sys_t *s, int fp64, double *tflops)
{
    void *buf = nullptr;
    FMDG_CK(cudaMalloc(&buf, 64));
    int dev = 0, sms = 0;
    FMDG_CK(cudaGetDevice(&dev));
    FMDG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256;
    const int iters = fp64 ? 2048 : 16384;
    float best = 1e30f;
    for (int rep = 0; rep < 4; rep++)
    {
        FMDG_CK(cudaEventRecord(s->ev0, s->stream));
        if (fp64) k_fma_peak<double><<<blocks, threads, 0, s->stream>>>((double *)buf, iters, 0.999999, 1e-7);
        else k_fma_peak<float><<<blocks, threads, 0, s->stream>>>((float *)buf, iters, 0.999999f, 1e-7f);
        FMDG_CK(cudaEventRecord(s->ev1, s->stream));
        FMDG_CK(cudaEventSynchronize(s->ev1));
        float ms;
        FMDG_CK(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
        if (rep > 0 && ms < best) best = ms;
    }
    cudaFree(buf);
    const double flops = 2.0 * 8.0 * iters * (double)blocks * threads;
    *tflops = flops / (best * 1e-3) / 1e12;
    return FMDG_OK;
}

extern "C" int fmdg_create(fmdg_sys_t **out, int device)
{
    *out = nullptr;
    FMDG_CK(cudaSetDevice(device));
    static bool pool_kept[64];
    if (device >= 0 && device < 64 && !pool_kept[device])
    {
        // freed system buffers stay in this process's pool for the next system
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess)
        {
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        pool_kept[device] = true;
    }
    fmdg_sys_t *s = (fmdg_sys_t *)calloc(1, sizeof(fmdg_sys_t));
    if (!s) return FMDG_E_NOMEM;
    s->device = device;
    // a system's own stream has the device's highest priority: a served
    // job's set-up (first list, forces, thermo record) then takes SM slots
    // ahead of the packed chunks already queued instead of waiting behind
    // them (a lone fmd.h system has no other stream to compete with)
    int prio_least = 0, prio_greatest = 0;
    cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    cudaError_t e = cudaStreamCreateWithPriority(&s->stream, cudaStreamNonBlocking, prio_greatest);
    if (e != cudaSuccess) { free(s); return fmdg_fail("cudaStreamCreateWithPriority", e); }
    FMDG_CK(cudaEventCreate(&s->ev0));
    FMDG_CK(cudaEventCreate(&s->ev1));
    for (int k = 0; k < 6; k++) FMDG_CK(cudaEventCreate(&s->pev[k]));
    int rc = dalloc(s, &s->g.dyn, 1);
    if (rc) return rc;
    rc = dalloc(s, &s->g.thermo, 1);
    if (rc) return rc;
    FMDG_CK(cudaMemsetAsync(s->g.dyn, 0, sizeof(Dyn), s->stream));
    FMDG_CK(cudaMemsetAsync(s->g.thermo, 0, sizeof(fmdg_thermo_t), s->stream));
    s->ttm_turi = -1;
    s->fblk = 128;
    // Verlet skin of the neighbour list (A) of mixed-precision systems;
    // FMD_SKIN=0 keeps the exact per-step stencil list
    s->skin = 0.5;
    if (const char *e = getenv("FMD_SKIN")) s->skin = atof(e);
    s->g.xs = s->g.inv_xs = 1.0;
    *out = s;
    return FMDG_OK;
}

extern "C" void fmdg_destroy(fmdg_sys_t *s)
{
    if (!s) return;
    cudaSetDevice(s->device);
    cudaStreamSynchronize(s->stream);
    free_atoms(s);
    if (s->eam_borrowed) drop_eam(s);
    dfree(s, (void *)s->g.pairs); dfree(s, (void *)s->g.mass); dfree(s, (void *)s->g.eam_elem);
    dfree(s, (void *)s->g.pairf); dfree(s, (void *)s->g.paird);
    dfree(s, (void *)s->g.eF); dfree(s, (void *)s->g.eFDD); dfree(s, (void *)s->g.erho);
    dfree(s, (void *)s->g.erhoDD); dfree(s, (void *)s->g.ephi); dfree(s, (void *)s->g.ephiDD);
    dfree(s, (void *)s->g.pk_rho); dfree(s, (void *)s->g.pk_phi); dfree(s, (void *)s->g.pk_F);
    dfree(s, (void *)s->g.pkf_rho); dfree(s, (void *)s->g.pkf_phi); dfree(s, (void *)s->g.pkf_F);
    dfree(s, (void *)s->g.pkf_pr); dfree(s, (void *)s->g.pkd_rho); dfree(s, (void *)s->g.pkd_phi);
    for (int k = 0; k < s->nturi; k++)
    {
        DTuri &t = s->turi[k];
        dfree(s, t.acc); dfree(s, t.tacc); dfree(s, t.mass); dfree(s, t.vcm); dfree(s, t.Ti); dfree(s, t.num);
        dfree(s, t.Te); dfree(s, t.Te2); dfree(s, t.xi); dfree(s, t.Ke); dfree(s, t.Ce); dfree(s, t.Gc); dfree(s, t.srcz);
        dfree(s, t.Te_pre);
        dfree(s, (void *)t.p.T_C); dfree(s, (void *)t.p.Ct); dfree(s, (void *)t.p.C_DD);
        dfree(s, (void *)t.p.T_G); dfree(s, (void *)t.p.Gt); dfree(s, (void *)t.p.G_DD);
    }
    dfree(s, s->g.dyn); dfree(s, s->g.thermo);
    dfree(s, s->l2buf);
    cudaEventDestroy(s->ev0);
    cudaEventDestroy(s->ev1);
    for (int k = 0; k < 6; k++) cudaEventDestroy(s->pev[k]);
    cudaStreamDestroy(s->stream);
    free(s);
}

extern "C" int fmdg_set_box(fmdg_sys_t *s, const double l[3], const int pbc[3], const int nc[3], const double cellh[3])
{
    for (int d = 0; d < 3; d++)
        if (nc[d] < 1 || !(l[d] > 0.0) || !(cellh[d] > 0.0)) return fmdg_set_error("fmdg_set_box: bad geometry");
    if (s->atoms) free_atoms(s);
    for (int d = 0; d < 3; d++)
    {
        s->g.l[d] = l[d];
        s->g.pbc[d] = pbc[d] ? 1 : 0;
        s->g.nc[d] = nc[d];
        s->g.cellh[d] = cellh[d];
        s->g.inv_cellh[d] = 1.0 / cellh[d];
        s->g.l_f[d] = (float)l[d];
        s->g.inv_cellh_f[d] = (float)s->g.inv_cellh[d];
    }
    const long long ncell = (long long)nc[0] * nc[1] * nc[2];
    if (ncell > (1 << 24)) return fmdg_set_error("fmdg_set_box: more than 2^24 cells");
    s->g.ncell = (int)ncell;
    s->box_set = true;
    return FMDG_OK;
}

extern "C" int fmdg_set_kinds(fmdg_sys_t *s, int nkinds, const double *mass, const int *eam_elem)
{
    if (nkinds < 1 || nkinds > FMDG_MAXK) return fmdg_set_error("fmdg_set_kinds: 1..8 kinds supported");
    s->nkinds = nkinds;
    s->g.nkinds = nkinds;
    for (int k = 0; k < nkinds; k++)
    {
        s->h_mass[k] = mass[k];
        s->h_eam_elem[k] = eam_elem ? eam_elem[k] : -1;
    }
    if (!s->g.mass)
    {
        int rc = dalloc(s, (double **)&s->g.mass, FMDG_MAXK);
        if (rc) return rc;
        rc = dalloc(s, (int **)&s->g.eam_elem, FMDG_MAXK);
        if (rc) return rc;
        rc = dalloc(s, (fmdg_pair_t **)&s->g.pairs, FMDG_MAXK * FMDG_MAXK);
        if (rc) return rc;
        // the binary32 table, then the skin kernels' scaled copy (skin_params)
        rc = dalloc(s, (float4 **)&s->g.pairf, 2 * FMDG_MAXK * FMDG_MAXK);
        if (rc) return rc;
        rc = dalloc(s, (float2 **)&s->g.paird, 4 * FMDG_MAXK * FMDG_MAXK);
        if (rc) return rc;
    }
    FMDG_CK(cudaMemcpyAsync((void *)s->g.mass, s->h_mass, sizeof(double) * nkinds, cudaMemcpyHostToDevice, s->stream));
    FMDG_CK(cudaMemcpyAsync((void *)s->g.eam_elem, s->h_eam_elem, sizeof(int) * nkinds, cudaMemcpyHostToDevice, s->stream));
    invalidate_graph(s);
    return FMDG_OK;
}

extern "C" int fmdg_set_pairs(fmdg_sys_t *s, const fmdg_pair_t *table)
{
    if (s->nkinds < 1) return fmdg_set_error("fmdg_set_pairs: set kinds first");
    const int nk2 = s->nkinds * s->nkinds;
    s->cats = 0;
    for (int k = 0; k < nk2; k++)
    {
        s->h_pairs[k] = table[k];
        const int c = table[k].cat;
        if (c != FMDG_POT_LJ && c != FMDG_POT_MORSE && c != FMDG_POT_EAM)
            return fmdg_set_error("fmdg_set_pairs: every kind pair needs a potential");
        s->cats |= 1 << c;
    }
    FMDG_CK(cudaMemcpyAsync((void *)s->g.pairs, s->h_pairs, sizeof(fmdg_pair_t) * nk2, cudaMemcpyHostToDevice, s->stream));
    // binary32 and double-float copies of the parameters, formed here so
    // that kernel prologues do no binary64 or conversion work
    float4 pf[FMDG_MAXK * FMDG_MAXK];
    float2 pd[4 * FMDG_MAXK * FMDG_MAXK];
    for (int k = 0; k < nk2; k++)
    {
        const double *p = s->h_pairs[k].p;
        pf[k] = make_float4((float)p[0], (float)p[1], (float)p[2], (float)p[3]);
        for (int q = 0; q < 4; q++) pd[4 * k + q] = df_split(p[q]);
    }
    FMDG_CK(cudaMemcpyAsync((void *)s->g.pairf, pf, sizeof(float4) * nk2, cudaMemcpyHostToDevice, s->stream));
    FMDG_CK(cudaMemcpyAsync((void *)s->g.paird, pd, sizeof(float2) * 4 * nk2, cudaMemcpyHostToDevice, s->stream));
    s->g.has_eam = (s->cats >> FMDG_POT_EAM) & 1;
    invalidate_graph(s);
    return fmdg_skin_scale(s);
}

// The scaled frame of the skin-list binary32 coordinates (see Geo::xs):
// xs, the scaled cell widths, the scaled skin radii and the pair
// parameters in scaled units, each formed in binary64 and rounded once.
// Per category (the layout of fmdg_pair_t.p): LJ {eps4, sig^2 xs^2,
// rc^2 xs^2}, Morse {D0, alpha / xs, r0 xs, rc^2 xs^2}, EAM {rc^2 xs^2 in
// p[2]}.
int fmdg_skin_scale(fmdg_sys_t *s)
{
    Geo &g = s->g;
    if (!s->box_set) return FMDG_OK;
    const double xs = (g.prec == FMDG_PREC_MIXED) ? (double)(float)g.cellh[0] / g.cellh[0] : 1.0;
    g.xs = xs;
    g.inv_xs = 1.0 / xs;
    for (int d = 0; d < 3; d++) g.cellh_s[d] = (float)(g.cellh[d] * xs);
    if (s->rsk > 0.0)
    {
        g.rskin2 = (float)(s->rsk * xs * s->rsk * xs);
        g.half_skin2 = (float)(0.25 * s->skin * s->skin * xs * xs);
    }
    const int nk2 = s->nkinds * s->nkinds;
    if (nk2 > 0 && g.pairf)
    {
        float4 pf[FMDG_MAXK * FMDG_MAXK];
        for (int k = 0; k < nk2; k++)
        {
            const double *p = s->h_pairs[k].p;
            double q[4] = {p[0], p[1], p[2], p[3]};
            if (s->h_pairs[k].cat == FMDG_POT_LJ)
            {
                q[1] = p[1] * xs * xs;
                q[2] = p[2] * xs * xs;
            }
            else if (s->h_pairs[k].cat == FMDG_POT_MORSE)
            {
                q[1] = p[1] / xs;
                q[2] = p[2] * xs;
                q[3] = p[3] * xs * xs;
            }
            else
                q[2] = p[2] * xs * xs;
            pf[k] = make_float4((float)q[0], (float)q[1], (float)q[2], (float)q[3]);
        }
        FMDG_CK(cudaMemcpyAsync((void *)skin_params(g), pf, sizeof(float4) * nk2, cudaMemcpyHostToDevice, s->stream));
    }
    invalidate_graph(s);
    return FMDG_OK;
}

extern "C" int fmdg_set_eam(fmdg_sys_t *s, int nelem, int Nrho, double drho, int Nr2, double dr2,
                            const double *F, const double *F_DD, const double *rho, const double *rhoDD,
                            const double *phi, const double *phiDD)
{
    if (nelem < 1 || nelem > FMDG_MAXE || Nrho < 3 || Nr2 < 3) return fmdg_set_error("fmdg_set_eam: bad sizes");
    Geo &g = s->g;
    if (s->eam_borrowed) drop_eam(s);
    dfree(s, (void *)g.eF); dfree(s, (void *)g.eFDD); dfree(s, (void *)g.erho);
    dfree(s, (void *)g.erhoDD); dfree(s, (void *)g.ephi); dfree(s, (void *)g.ephiDD);
    const size_t nF = (size_t)nelem * Nrho, nR = (size_t)nelem * Nr2, nP = (size_t)nelem * nelem * Nr2;
    int rc;
    if ((rc = dalloc(s, (double **)&g.eF, nF)) || (rc = dalloc(s, (double **)&g.eFDD, nF)) ||
        (rc = dalloc(s, (double **)&g.erho, nR)) || (rc = dalloc(s, (double **)&g.erhoDD, nR)) ||
        (rc = dalloc(s, (double **)&g.ephi, nP)) || (rc = dalloc(s, (double **)&g.ephiDD, nP)))
        return rc;
    FMDG_CK(cudaMemcpyAsync((void *)g.eF, F, nF * 8, cudaMemcpyHostToDevice, s->stream));
    FMDG_CK(cudaMemcpyAsync((void *)g.eFDD, F_DD, nF * 8, cudaMemcpyHostToDevice, s->stream));
    FMDG_CK(cudaMemcpyAsync((void *)g.erho, rho, nR * 8, cudaMemcpyHostToDevice, s->stream));
    FMDG_CK(cudaMemcpyAsync((void *)g.erhoDD, rhoDD, nR * 8, cudaMemcpyHostToDevice, s->stream));
    FMDG_CK(cudaMemcpyAsync((void *)g.ephi, phi, nP * 8, cudaMemcpyHostToDevice, s->stream));
    FMDG_CK(cudaMemcpyAsync((void *)g.ephiDD, phiDD, nP * 8, cudaMemcpyHostToDevice, s->stream));
    g.nelem = nelem; g.Nrho = Nrho; g.Nr2 = Nr2; g.drho = drho; g.dr2 = dr2;
    g.inv_dr2 = 1.0 / dr2;
    g.inv_drho = 1.0 / drho;
    // Per-interval cubic coefficients of the natural spline (src/cspline.h:26-27)
    // in the local coordinate b = x/h - k in [0,1): with C = y''*h^2/6,
    //   y(b)   = k0 + k1 b + k2 b^2 + k3 b^3,
    //   k0 = y_k, k1 = y_k+1 - y_k - 2C_k - C_k+1, k2 = 3C_k, k3 = C_k+1 - C_k,
    //   dy/dx  = (k1 + 2 k2 b + 3 k3 b^2) / h,
    // algebraically the reference's a/b form (a = 1-b).  Computed in binary64;
    // the binary32 copy keeps k1 (the per-interval increment) to full relative
    // precision, which the two-sample difference y_k+1 - y_k would not.
    dfree(s, (void *)g.pk_rho); dfree(s, (void *)g.pk_phi); dfree(s, (void *)g.pk_F);
    dfree(s, (void *)g.pkf_rho); dfree(s, (void *)g.pkf_phi); dfree(s, (void *)g.pkf_F);
    dfree(s, (void *)g.pkf_pr); dfree(s, (void *)g.pkd_rho); dfree(s, (void *)g.pkd_phi);
    auto pack = [&](const double *y, const double *ydd, double h, int npts, int nfun, const double4_32a **d64,
                    const float4 **d32, const float4 **ddf) -> int {
        const size_t nint = (size_t)npts - 1;
        std::vector<double4_32a> h64(nint * nfun);
        std::vector<float4> h32(nint * nfun), hdf(ddf ? 2 * nint * nfun : 0);
        const double hh6 = h * h / 6.0;
        for (int f = 0; f < nfun; f++)
            for (size_t k = 0; k < nint; k++)
            {
                const double *yy = y + (size_t)f * npts, *dd = ydd + (size_t)f * npts;
                const double c0 = dd[k] * hh6, c1 = dd[k + 1] * hh6;
                const double k0 = yy[k], k1 = yy[k + 1] - yy[k] - 2.0 * c0 - c1, k2 = 3.0 * c0, k3 = c1 - c0;
                h64[f * nint + k] = make_double4_32a(k0, k1, k2, k3);
                h32[f * nint + k] = make_float4((float)k0, (float)k1, (float)k2, (float)k3);
                if (ddf)
                {
                    const float2 s0 = df_split(k0), s1 = df_split(k1), s2 = df_split(k2), s3 = df_split(k3);
                    hdf[2 * (f * nint + k)] = make_float4(s0.x, s1.x, s2.x, s3.x);
                    hdf[2 * (f * nint + k) + 1] = make_float4(s0.y, s1.y, s2.y, s3.y);
                }
            }
        int rc2;
        if ((rc2 = dalloc(s, (double4_32a **)d64, h64.size())) || (rc2 = dalloc(s, (float4 **)d32, h32.size()))) return rc2;
        FMDG_CK(cudaMemcpyAsync((void *)*d64, h64.data(), h64.size() * sizeof(double4_32a), cudaMemcpyHostToDevice, s->stream));
        FMDG_CK(cudaMemcpyAsync((void *)*d32, h32.data(), h32.size() * sizeof(float4), cudaMemcpyHostToDevice, s->stream));
        if (ddf)
        {
            if ((rc2 = dalloc(s, (float4 **)ddf, hdf.size()))) return rc2;
            FMDG_CK(cudaMemcpyAsync((void *)*ddf, hdf.data(), hdf.size() * sizeof(float4), cudaMemcpyHostToDevice, s->stream));
        }
        return FMDG_OK;
    };
    if ((rc = pack(rho, rhoDD, dr2, Nr2, nelem, &g.pk_rho, &g.pkf_rho, &g.pkd_rho))) return rc;
    if ((rc = pack(phi, phiDD, dr2, Nr2, nelem * nelem, &g.pk_phi, &g.pkf_phi, &g.pkd_phi))) return rc;
    if ((rc = pack(F, F_DD, drho, Nrho, nelem, &g.pk_F, &g.pkf_F, nullptr))) return rc;
    {
        // the one-element pair rows side by side for the lean force kernels
        const size_t nint = (size_t)Nr2 - 1;
        std::vector<float4> phi32(nint * nelem * nelem), rho32(nint * nelem), pr(2 * nint * nelem);
        FMDG_D2H(phi32.data(), g.pkf_phi, phi32.size() * sizeof(float4));
        FMDG_D2H(rho32.data(), g.pkf_rho, rho32.size() * sizeof(float4));
        for (int e = 0; e < nelem; e++)
            for (size_t k = 0; k < nint; k++)
            {
                pr[2 * (e * nint + k)] = phi32[((size_t)e * nelem + e) * nint + k];
                pr[2 * (e * nint + k) + 1] = rho32[(size_t)e * nint + k];
            }
        if ((rc = dalloc(s, (float4 **)&g.pkf_pr, pr.size()))) return rc;
        FMDG_CK(cudaMemcpyAsync((void *)g.pkf_pr, pr.data(), pr.size() * sizeof(float4), cudaMemcpyHostToDevice, s->stream));
    }
    // the 32-byte row tables are read with 256-bit loads (ld_row32)
    if (((uintptr_t)g.pkf_pr | (uintptr_t)g.pkd_rho | (uintptr_t)g.pkd_phi) % 32)
        return fmdg_set_error("fmdg_set_eam: row tables not 32-byte aligned");
    invalidate_graph(s);
    // other systems may read these tables on their own streams
    // (fmdg_share_eam): the copies complete before this call returns
    FMDG_CK(cudaStreamSynchronize(s->stream));
    return fmdg_skin_scale(s);
}

extern "C" int fmdg_set_precision(fmdg_sys_t *s, int mode)
{
    if (mode != FMDG_PREC_FP64 && mode != FMDG_PREC_MIXED) return fmdg_set_error("fmdg_set_precision: bad mode");
    s->g.prec = mode;
    invalidate_graph(s);
    return fmdg_skin_scale(s);
}

// Neighbour-list entries per atom: 1.3x the pairs an atom of the densest
// cell has within the list radius (largest cutoff + 0.01), at least 32.
int fmdg_list_capacity(const fmdg_sys_t *s, const int *cell_count, int ncell)
{
    const Geo &g = s->g;
    double rc2max = 0.0;
    for (int k = 0; k < s->nkinds * s->nkinds; k++)
    {
        const fmdg_pair_t &pp = s->h_pairs[k];
        const double r2 = pp.cat == FMDG_POT_MORSE ? pp.p[3] : pp.p[2];
        if (r2 > rc2max) rc2max = r2;
    }
    if (!(rc2max > 0.0))
    {
        const double hmin = fmin(g.cellh[0], fmin(g.cellh[1], g.cellh[2]));
        rc2max = hmin * hmin;
    }
    const double rlist = sqrt(rc2max) + (s->skin > 0.0 ? s->skin : 1e-2);
    if (s->list_capacity > 0) return s->list_capacity;
    return fmdg_capacity_estimate(cell_count, ncell, g.cellh[0] * g.cellh[1] * g.cellh[2], rlist);
}

// Neighbour-list entries per atom (before fmdg_upload); 0: the estimate.
extern "C" int fmdg_set_build_lanes(fmdg_sys_t *s, int lanes)
{
    if (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32)
        return fmdg_set_error("fmdg_set_build_lanes: 0, 1, 2, 4, 8, 16 or 32");
    s->build_lanes = lanes;
    return FMDG_OK;
}

extern "C" int fmdg_set_list_capacity(fmdg_sys_t *s, int entries)
{
    if (entries < 0 || entries > 1024 || (entries % 8) != 0)
        return fmdg_set_error("fmdg_set_list_capacity: 0 or a multiple of 8 up to 1024");
    s->list_capacity = entries;
    return FMDG_OK;
}

// Entries per atom a neighbour list of radius rlist holds: 1.3 x the count
// at the density of the fullest cell + 16, a multiple of 8 in [32, 1024].
// Atoms beyond it scan their stencil directly, so this is a performance and
// memory knob only (fmdg_set_list_capacity overrides it).
int fmdg_capacity_estimate(const int *cell_count, int ncell, double cell_volume, double rlist)
{
    int maxcell = 0;
    for (int c = 0; c < ncell; c++) maxcell = cell_count[c] > maxcell ? cell_count[c] : maxcell;
    const double dens = maxcell / cell_volume;
    const double est = 4.0 / 3.0 * 3.14159265358979 * rlist * rlist * rlist * dens;
    int maxnb = (int)(1.3 * est + 16);
    maxnb = (maxnb + 7) & ~7;
    if (maxnb < 32) maxnb = 32;
    if (maxnb > 1024) maxnb = 1024;
    return maxnb;
}

// device bytes of a system with n atoms, ncell cells and list capacity maxnb
size_t fmdg_bytes_estimate(int n, int ncell, int maxnb)
{
    const size_t cap = n > 0 ? n : 1;
    const size_t per_atom = 2 * (48 + 16) + 32 + 7 * 4 + 16 + 4 + 4 * (size_t)maxnb + 9 * 8 / 64 + 8 + 24 +
                            32;   // binary64 position rows (xdf)
    const size_t per_cell = 2 * 4 + 5 * 4 + 32;
    return cap * per_atom + (size_t)ncell * per_cell + 64 * 1024;
}

// packed launches: steps the system still takes
int fmdg_set_steps_left(fmdg_sys_t *s, int steps)
{
    FMDG_CK(cudaMemcpyAsync((char *)s->g.dyn + offsetof(Dyn, steps_left), &steps, sizeof steps, cudaMemcpyHostToDevice, s->stream));
    return FMDG_OK;
}

// Verlet skin of the neighbour list (before fmdg_upload), any precision.
extern "C" int fmdg_set_skin(fmdg_sys_t *s, double skin)
{
    if (!(skin >= 0.0)) return fmdg_set_error("fmdg_set_skin: negative skin");
    s->skin = skin;
    s->skin_set = true;
    return FMDG_OK;
}

// Use the EAM tables of another system on the same device without a copy;
// the owner must outlive every borrower.
extern "C" int fmdg_share_eam(fmdg_sys_t *s, const fmdg_sys_t *owner)
{
    if (!owner || !owner->g.pk_rho) return fmdg_set_error("fmdg_share_eam: the owner has no EAM tables");
    if (owner->device != s->device) return fmdg_set_error("fmdg_share_eam: different devices");
    Geo &g = s->g;
    if (!s->eam_borrowed)
    {
        dfree(s, (void *)g.eF); dfree(s, (void *)g.eFDD); dfree(s, (void *)g.erho);
        dfree(s, (void *)g.erhoDD); dfree(s, (void *)g.ephi); dfree(s, (void *)g.ephiDD);
        dfree(s, (void *)g.pk_rho); dfree(s, (void *)g.pk_phi); dfree(s, (void *)g.pk_F);
        dfree(s, (void *)g.pkf_rho); dfree(s, (void *)g.pkf_phi); dfree(s, (void *)g.pkf_F);
        dfree(s, (void *)g.pkf_pr); dfree(s, (void *)g.pkd_rho); dfree(s, (void *)g.pkd_phi);
    }
    const Geo &o = owner->g;
    g.eF = o.eF; g.eFDD = o.eFDD; g.erho = o.erho; g.erhoDD = o.erhoDD; g.ephi = o.ephi; g.ephiDD = o.ephiDD;
    g.pk_rho = o.pk_rho; g.pk_phi = o.pk_phi; g.pk_F = o.pk_F;
    g.pkf_rho = o.pkf_rho; g.pkf_phi = o.pkf_phi; g.pkf_F = o.pkf_F; g.pkf_pr = o.pkf_pr;
    g.pkd_rho = o.pkd_rho; g.pkd_phi = o.pkd_phi;
    g.nelem = o.nelem; g.Nrho = o.Nrho; g.Nr2 = o.Nr2; g.drho = o.drho; g.dr2 = o.dr2;
    g.inv_dr2 = o.inv_dr2; g.inv_drho = o.inv_drho;
    s->eam_borrowed = true;
    invalidate_graph(s);
    return fmdg_skin_scale(s);
}

extern "C" int fmdg_upload(fmdg_sys_t *s, int n, const int *cell_count, const double *x, const double *v,
                           const unsigned *kind, const int *group, const unsigned *atomid)
{
    if (!s->box_set) return fmdg_set_error("fmdg_upload: set the box first");
    if (n < 0) return fmdg_set_error("fmdg_upload: negative atom count");
    Geo &g = s->g;
    const int ncell = g.ncell;
    std::vector<int> start(ncell + 1), cell_of(n > 0 ? n : 1);
    long long acc = 0;
    for (int c = 0; c < ncell; c++)
    {
        start[c] = (int)acc;
        for (int k = 0; k < cell_count[c]; k++) cell_of[acc + k] = c;
        acc += cell_count[c];
    }
    start[ncell] = (int)acc;
    if (acc != n) return fmdg_set_error("fmdg_upload: cell counts do not add up to n");
    for (int i = 0; i < n; i++)
        if (kind[i] >= (unsigned)(s->nkinds > 0 ? s->nkinds : FMDG_MAXK))
            return fmdg_set_error("fmdg_upload: atom kind out of range");
    // the device time and step of an earlier upload carry over; a fresh
    // system's dynamic scalars are the zeros of fmdg_create (no device read,
    // so a served job's set-up does not wait for the GPU)
    Dyn d;
    if (s->uploaded) FMDG_D2H(&d, g.dyn, sizeof d);
    else memset(&d, 0, sizeof d);
    free_atoms(s);
    const int cap = n > 0 ? n : 1;
    g.cap = cap;
    int rc;
    // neighbour list: size from the densest cell (an atom with more
    // candidates falls back to a direct stencil scan)
    double rc2max = 0.0;
    for (int k = 0; k < s->nkinds * s->nkinds; k++)
    {
        const fmdg_pair_t &pp = s->h_pairs[k];
        const double r2 = pp.cat == FMDG_POT_MORSE ? pp.p[3] : pp.p[2];
        if (r2 > rc2max) rc2max = r2;
    }
    if (!(rc2max > 0.0))
    {
        const double hmin = fmin(g.cellh[0], fmin(g.cellh[1], g.cellh[2]));
        rc2max = hmin * hmin;
    }
    const double rlist = sqrt(rc2max) + 1e-2;
    g.rlist2 = (float)(rlist * rlist);
    const int maxnb = fmdg_list_capacity(s, cell_count, ncell);
    g.maxnb = maxnb;
    for (int d3 = 0; d3 < 3; d3++)
    {
        g.cellh_f[d3] = (float)g.cellh[d3];
    }
    // a skin list needs the list radius below half of every periodic box
    // length (one image inside it) and within two cells; otherwise the
    // exact stencil list is rebuilt every step
    // (default: mixed precision only -- in binary64 mode the double-float
    // pair arithmetic costs more on the longer list than the rebuilds save:
    // EAM 256k 3.0e8 vs 3.5e8 atom-steps/s; LJ and Morse gain 7-8%)
    g.skin_on = 0;
    if (s->skin > 0.0 && cap < (1 << 25) && (s->skin_set || g.prec == FMDG_PREC_MIXED))
    {
        const double rsk = sqrt(rc2max) + s->skin;
        bool ok = rsk <= 2.0 * fmin(g.cellh[0], fmin(g.cellh[1], g.cellh[2]));
        for (int d3 = 0; d3 < 3; d3++)
            if (g.pbc[d3] && !(g.l[d3] > 2.0 * rsk)) ok = false;
        g.skin_on = ok;
    }
    // partials for the smallest block size the tuner may pick (64)
    const int nb = fmdg_grid(cap, 64);
    auto layout = [&](Carver &c) {
        for (int k = 0; k < 2; k++)
        {
            Side &S = g.side[k];
            c.take(S.x, 3 * (size_t)cap); c.take(S.v, 3 * (size_t)cap);
            c.take(S.kind, cap); c.take(S.group, cap); c.take(S.atomid, cap);
            c.take(S.cell_of, cap); c.take(S.cell_start, (size_t)ncell + 1);
            if (g.skin_on) c.take(S.slot, cap);
        }
        c.take(g.F, 3 * (size_t)cap); c.take(g.vaream, cap);
        c.take(g.bdest, cap); c.take(g.bpath, cap); c.take(g.bslot, cap); c.take(g.brank, cap);
        c.take(g.bnewidx, cap); c.take(g.dep_count, 4 * (size_t)ncell); c.take(g.arr_base, (size_t)ncell + 1);
        c.take(g.bucket, cap); c.take(g.arr_slot, cap);
        c.take(g.fpf, cap); c.take(g.xf4, cap); c.take(g.nbr, (size_t)cap * maxnb); c.take(g.nbr_count, cap);
        c.take(g.xdf, 2 * (size_t)cap); c.take(g.fpdf, cap);
        c.take(g.partials, (size_t)nb * 9 + 8);
        c.take(g.corig, ncell);
        if (g.skin_on)
        {
            c.take(g.pos, cap); c.take(g.cb, cap); c.take(g.xl, cap); c.take(g.xb, cap);
            c.take(g.xd, cap); c.take(g.gslot, cap); c.take(g.fpb, cap); c.take(g.fpd, cap);
            c.take(g.xll, cap);
        }
    };
    Carver measure{nullptr, 0};
    layout(measure);
    if ((rc = dalloc(s, &s->arena, measure.off))) return rc;
    Carver carve{s->arena, 0};
    layout(carve);
    g.arr_lower = g.dep_count + ncell;
    g.arr_total = g.dep_count + 2 * ncell;
    g.bucket_fill = g.dep_count + 3 * ncell;
    cudaStream_t st = s->stream;
    std::vector<int> iota;
    if (g.skin_on)
    {
        iota.resize(cap);
        for (int k = 0; k < cap; k++) iota[k] = k;
        FMDG_CK(cudaMemcpyAsync(g.side[0].slot, iota.data(), (size_t)cap * 4, cudaMemcpyHostToDevice, st));
        FMDG_CK(cudaMemcpyAsync(g.pos, iota.data(), (size_t)cap * 4, cudaMemcpyHostToDevice, st));
        // build cells: valid cell indexes before the first build writes them
        FMDG_CK(cudaMemsetAsync(g.cb, 0, (size_t)cap * 4, st));
        const double rsk = sqrt(rc2max) + s->skin;
        s->rsk = rsk;
        g.srad = 1;
        for (int d3 = 0; d3 < 3; d3++)
            if (rsk > g.cellh[d3]) g.srad = 2;
    }
    if ((rc = fmdg_skin_scale(s))) return rc;
    // host SoA staging
    std::vector<double> hx(3 * (size_t)cap, 0.0), hv(3 * (size_t)cap, 0.0);
    for (int i = 0; i < n; i++)
        for (int d = 0; d < 3; d++)
        {
            hx[(size_t)d * cap + i] = x[3 * (size_t)i + d];
            hv[(size_t)d * cap + i] = v[3 * (size_t)i + d];
        }
    Side &S = g.side[0];
    FMDG_CK(cudaMemcpyAsync(S.x, hx.data(), hx.size() * 8, cudaMemcpyHostToDevice, st));
    FMDG_CK(cudaMemcpyAsync(S.v, hv.data(), hv.size() * 8, cudaMemcpyHostToDevice, st));
    if (n > 0)
    {
        FMDG_CK(cudaMemcpyAsync(S.kind, kind, (size_t)n * 4, cudaMemcpyHostToDevice, st));
        FMDG_CK(cudaMemcpyAsync(S.group, group, (size_t)n * 4, cudaMemcpyHostToDevice, st));
        FMDG_CK(cudaMemcpyAsync(S.atomid, atomid, (size_t)n * 4, cudaMemcpyHostToDevice, st));
        FMDG_CK(cudaMemcpyAsync(S.cell_of, cell_of.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st));
    }
    FMDG_CK(cudaMemcpyAsync(S.cell_start, start.data(), ((size_t)ncell + 1) * 4, cudaMemcpyHostToDevice, st));
    // frame origins of the cell-local binary32 coordinates: the cell centres
    // ((c + 1/2) * cellh per axis, binary64).  Centred frames keep the
    // coordinates within half a cell (plus the skin drift) of zero, so their
    // binary32 rounding is half that of corner-relative ones; pair geometry
    // only uses differences, so the choice of frame changes nothing else
    std::vector<double4_32a> corig(ncell);
    for (int c = 0; c < ncell; c++)
    {
        const int cx = c / (g.nc[1] * g.nc[2]), cy = (c / g.nc[2]) % g.nc[1], cz = c % g.nc[2];
        corig[c] = make_double4_32a((cx + 0.5) * g.cellh[0], (cy + 0.5) * g.cellh[1], (cz + 0.5) * g.cellh[2], 0.0);
    }
    FMDG_CK(cudaMemcpyAsync((void *)g.corig, corig.data(), (size_t)ncell * sizeof(double4_32a),
                            cudaMemcpyHostToDevice, st));
    FMDG_CK(cudaMemsetAsync(g.F, 0, 3 * (size_t)cap * 8, st));
    FMDG_CK(cudaMemsetAsync(g.vaream, 0, (size_t)cap * 8, st));
    const double keep_time = d.time, keep_dt = d.dt;
    memset(&d, 0, sizeof d);
    d.cur = 0;
    d.n = n;
    d.lambda = 1.0;
    d.rebuild = 1;
    d.time = keep_time;
    d.dt = keep_dt;
    FMDG_CK(cudaMemcpyAsync(g.dyn, &d, sizeof d, cudaMemcpyHostToDevice, st));
    // (copies from pageable host memory are staged before the calls return,
    // so the host buffers may go)
    s->atoms = true;
    s->uploaded = true;
    return FMDG_OK;
}

extern "C" int fmdg_natoms(fmdg_sys_t *s, int *n)
{
    if (!s->atoms) { *n = 0; return FMDG_OK; }
    Dyn d;
    int rc = read_dyn(s, &d);
    if (rc) return rc;
    *n = d.n;
    return FMDG_OK;
}

extern "C" int fmdg_download(fmdg_sys_t *s, int *cell_of, double *x, double *v, double *F, double *vaream,
                             unsigned *kind, int *group, unsigned *atomid)
{
    if (!s->atoms) return FMDG_E_STATE;
    Dyn d;
    int rc = read_dyn(s, &d);
    if (rc) return rc;
    const Geo &g = s->g;
    const Side &S = g.side[d.cur];
    const int n = d.n, cap = g.cap;
    std::vector<double> buf(3 * (size_t)cap);
    auto get3 = [&](const double *src, double *dst) -> int {
        FMDG_D2H(buf.data(), src, 3 * (size_t)cap * 8);
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) dst[3 * (size_t)i + k] = buf[(size_t)k * cap + i];
        return FMDG_OK;
    };
    if (x && (rc = get3(S.x, x))) return rc;
    if (v && (rc = get3(S.v, v))) return rc;
    if (F && (rc = get3(g.F, F))) return rc;
    if (n > 0)
    {
        if (vaream) FMDG_D2H(vaream, g.vaream, (size_t)n * 8);
        if (kind) FMDG_D2H(kind, S.kind, (size_t)n * 4);
        if (group) FMDG_D2H(group, S.group, (size_t)n * 4);
        if (atomid) FMDG_D2H(atomid, S.atomid, (size_t)n * 4);
        if (cell_of) FMDG_D2H(cell_of, S.cell_of, (size_t)n * 4);
    }
    return FMDG_OK;
}

extern "C" int fmdg_set_state(fmdg_sys_t *s, const double *x, const double *v)
{
    if (!s->atoms) return FMDG_E_STATE;
    Dyn d;
    int rc = read_dyn(s, &d);
    if (rc) return rc;
    const Side &S = s->g.side[d.cur];
    const int n = d.n, cap = s->g.cap;
    std::vector<double> buf(3 * (size_t)cap, 0.0);
    auto put3 = [&](const double *src, double *dst) -> int {
        FMDG_D2H(buf.data(), dst, 3 * (size_t)cap * 8);
        for (int i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) buf[(size_t)k * cap + i] = src[3 * (size_t)i + k];
        FMDG_CK(cudaMemcpyAsync(dst, buf.data(), 3 * (size_t)cap * 8, cudaMemcpyHostToDevice, s->stream));
        return FMDG_OK;
    };
    if (x && (rc = put3(x, S.x))) return rc;
    if (v && (rc = put3(v, S.v))) return rc;
    if (x)
    {
        // positions set from outside: the skin list is rebuilt first
        const int one = 1;
        FMDG_CK(cudaMemcpyAsync((char *)s->g.dyn + offsetof(Dyn, rebuild), &one, sizeof one, cudaMemcpyHostToDevice, s->stream));
    }
    return FMDG_OK;
}

extern "C" int fmdg_refresh(fmdg_sys_t *s)
{
    if (!s->atoms) return FMDG_E_STATE;
    return fmdg_launch_refresh(s, FMDG_REFRESH_ONLY, 0.0, -1, 0);
}

extern "C" int fmdg_compute_forces(fmdg_sys_t *s, int active_group)
{
    if (!s->atoms || !s->cats) return FMDG_E_STATE;
    return fmdg_launch_forces(s, active_group, 0, 0.0, 0, 1.0, 0.0);
}

extern "C" int fmdg_thermo(fmdg_sys_t *s, int active_group, fmdg_thermo_t *out)
{
    if (!s->atoms) return FMDG_E_STATE;
    int rc = fmdg_launch_thermo(s, active_group, 0, 0.0, 1.0, 0.0);
    if (rc) return rc;
    return out ? fmdg_get_thermo(s, out) : FMDG_OK;
}

static int vv_step_launches(fmdg_sys_t *s, double dt, int group, int thermostat, double tau, double T0)
{
    int rc = fmdg_launch_refresh(s, FMDG_REFRESH_VV, dt, group, thermostat);
    if (rc) return rc;
    rc = fmdg_launch_forces(s, group, 1, dt, thermostat, tau, T0);
    if (rc) return rc;
    // fields of every turi after the step (src/integrators.c:258-259)
    for (int k = 0; k < s->nturi; k++)
        if ((rc = fmdg_launch_turi(s, k, dt))) return rc;
    return FMDG_OK;
}

// symplectic Euler under TTM (src/integrators.c:129-179, 198-224)
static int se_step_launches(fmdg_sys_t *s, double dt, int group)
{
    int rc = fmdg_launch_refresh(s, FMDG_REFRESH_SE, dt, group, 0);
    if (rc) return rc;
    for (int k = 0; k < s->nturi; k++)
        if ((rc = fmdg_launch_turi(s, k, dt))) return rc;
    return fmdg_launch_forces(s, group, 0, dt, 0, 1.0, 0.0);
}

// Before the first step of a run the caller computes the forces of the
// current positions (fmdg_compute_forces) and, with a thermostat, sets the
// scale from the current temperature (fmdg_prepare_thermostat); each step
// then leaves the next step's scale on the device.
extern "C" int fmdg_prepare_thermostat(fmdg_sys_t *s, int group, double dt, double tau, double T0)
{
    if (!s->atoms) return FMDG_E_STATE;
    return fmdg_launch_thermo(s, group, 1, dt, tau, T0);
}

extern "C" int fmdg_vv_steps(fmdg_sys_t *s, int nsteps, double dt, int active_group,
                             int thermostat, double tau, double T0)
{
    if (!s->atoms || !s->cats) return FMDG_E_STATE;
    if (nsteps <= 0) return FMDG_OK;
    if (s->profiling)
    {
        // phases timed separately with events:
        // 0 refresh, 1 neighbour list, 2 density, 3 force (+ thermo record), 4 turi fields
        for (int k = 0; k < nsteps; k++)
        {
            FMDG_CK(cudaEventRecord(s->pev[0], s->stream));
            int rc = fmdg_launch_refresh(s, FMDG_REFRESH_VV, dt, active_group, thermostat);
            if (rc) return rc;
            FMDG_CK(cudaEventRecord(s->pev[1], s->stream));
            if ((rc = fmdg_launch_nlist(s))) return rc;
            FMDG_CK(cudaEventRecord(s->pev[2], s->stream));
            if ((rc = fmdg_launch_density(s, active_group))) return rc;
            FMDG_CK(cudaEventRecord(s->pev[3], s->stream));
            if ((rc = fmdg_launch_pair_forces(s, active_group, 1, dt, thermostat, tau, T0))) return rc;
            FMDG_CK(cudaEventRecord(s->pev[4], s->stream));
            for (int k = 0; k < s->nturi; k++)
                if ((rc = fmdg_launch_turi(s, k, dt))) return rc;
            FMDG_CK(cudaEventRecord(s->pev[5], s->stream));
            FMDG_CK(cudaEventSynchronize(s->pev[5]));
            for (int ph = 0; ph < 5; ph++)
            {
                float ms = 0.0f;
                FMDG_CK(cudaEventElapsedTime(&ms, s->pev[ph], s->pev[ph + 1]));
                s->prof_ms[ph] += ms;
                s->prof_n[ph] += 1;
            }
        }
        return FMDG_OK;
    }
    const bool same = s->graph_key_valid && s->graph_mode == 0 && s->graph_dt == dt &&
                      s->graph_group == active_group && s->graph_thermo == thermostat && s->graph_tau == tau &&
                      s->graph_T0 == T0;
    if (!same)
    {
        invalidate_graph(s);
        cudaGraph_t graph;
        FMDG_CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        const long long before = s->launches;
        int rc = vv_step_launches(s, dt, active_group, thermostat, tau, T0);
        cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
        if (rc) return rc;
        if (e != cudaSuccess) return fmdg_fail("cudaStreamEndCapture", e);
        s->launches = before;
        e = cudaGraphInstantiate(&s->graph, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fmdg_fail("cudaGraphInstantiate", e);
        s->graph_key_valid = 1;
        s->graph_dt = dt; s->graph_group = active_group; s->graph_thermo = thermostat;
        s->graph_tau = tau; s->graph_T0 = T0;
        s->graph_mode = 0;
        // kernels per captured step
        const bool eam = (s->cats & (1 << FMDG_POT_EAM)) != 0;
        // memset node + 6 refresh kernels + 2 list kernels + density + force
        s->graph_steps = 7 + 2 + (eam ? 1 : 0) + 1;
        for (int k = 0; k < s->nturi; k++) s->graph_steps += 5 + (s->turi[k].ttm ? 1 : 0);
    }
    for (int k = 0; k < nsteps; k++) FMDG_CK(cudaGraphLaunch(s->graph, s->stream));
    s->launches += (long long)nsteps * (s->graph_steps - 1);  // memset node is not a kernel
    return FMDG_OK;
}

extern "C" int fmdg_se_steps(fmdg_sys_t *s, int nsteps, double dt, int active_group)
{
    if (!s->atoms || !s->cats) return FMDG_E_STATE;
    if (nsteps <= 0) return FMDG_OK;
    if (s->profiling)
    {
        // phases timed separately with events: 0 kick-drift + refresh,
        // 4 turi field passes, 5 TTM solver, 3 neighbour list + density +
        // pair forces (+ friction term); the launches of se_step_launches
        // in the same order
        for (int k = 0; k < nsteps; k++)
        {
            FMDG_CK(cudaEventRecord(s->pev[0], s->stream));
            int rc = fmdg_launch_refresh(s, FMDG_REFRESH_SE, dt, active_group, 0);
            if (rc) return rc;
            FMDG_CK(cudaEventRecord(s->pev[1], s->stream));
            for (int q = 0; q < s->nturi; q++)
                if ((rc = fmdg_launch_turi_fields(s, q, dt))) return rc;
            FMDG_CK(cudaEventRecord(s->pev[2], s->stream));
            for (int q = 0; q < s->nturi; q++)
                if ((rc = fmdg_launch_ttm_solve(s, q, dt))) return rc;
            FMDG_CK(cudaEventRecord(s->pev[3], s->stream));
            if ((rc = fmdg_launch_forces(s, active_group, 0, dt, 0, 1.0, 0.0))) return rc;
            FMDG_CK(cudaEventRecord(s->pev[4], s->stream));
            FMDG_CK(cudaEventSynchronize(s->pev[4]));
            const int phase[4] = {0, 4, 5, 3};
            for (int q = 0; q < 4; q++)
            {
                float ms = 0.0f;
                FMDG_CK(cudaEventElapsedTime(&ms, s->pev[q], s->pev[q + 1]));
                s->prof_ms[phase[q]] += ms;
                s->prof_n[phase[q]] += 1;
            }
        }
        return FMDG_OK;
    }
    const bool same = s->graph_key_valid && s->graph_mode == 1 && s->graph_dt == dt && s->graph_group == active_group;
    if (!same)
    {
        invalidate_graph(s);
        cudaGraph_t graph;
        FMDG_CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        const long long before = s->launches;
        int rc = se_step_launches(s, dt, active_group);
        cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
        if (rc) return rc;
        if (e != cudaSuccess) return fmdg_fail("cudaStreamEndCapture", e);
        s->graph_steps = (int)(s->launches - before) + 1;
        s->launches = before;
        e = cudaGraphInstantiate(&s->graph, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fmdg_fail("cudaGraphInstantiate", e);
        s->graph_key_valid = 1;
        s->graph_mode = 1;
        s->graph_dt = dt;
        s->graph_group = active_group;
    }
    for (int k = 0; k < nsteps; k++) FMDG_CK(cudaGraphLaunch(s->graph, s->stream));
    s->launches += (long long)nsteps * (s->graph_steps - 1);
    return FMDG_OK;
}

extern "C" int fmdg_set_time(fmdg_sys_t *s, double time, double dt)
{
    Dyn d;
    int rc = read_dyn(s, &d);
    if (rc) return rc;
    d.time = time;
    d.dt = dt;
    FMDG_CK(cudaMemcpyAsync(s->g.dyn, &d, sizeof d, cudaMemcpyHostToDevice, s->stream));
    return FMDG_OK;
}

extern "C" int fmdg_turi_add(fmdg_sys_t *s, const int dims_local[3], const int g2l[3], const double tcellh[3],
                             double starttime, double stoptime, int *handle)
{
    if (s->nturi >= FMDG_MAXT) return fmdg_set_error("fmdg_turi_add: at most 4 turies per system");
    DTuri &t = s->turi[s->nturi];
    memset(&t, 0, sizeof t);
    long long nc = 1;
    for (int d = 0; d < 3; d++)
    {
        if (dims_local[d] < 1 || !(tcellh[d] > 0)) return fmdg_set_error("fmdg_turi_add: bad geometry");
        t.dims[d] = dims_local[d];
        t.g2l[d] = g2l[d];
        t.tcellh[d] = tcellh[d];
        t.inv_tcellh[d] = 1.0 / tcellh[d];
        nc *= dims_local[d];
    }
    if (nc > (1 << 22)) return fmdg_set_error("fmdg_turi_add: too many turi cells");
    t.ncells = (int)nc;
    t.tcell_volume = tcellh[0] * tcellh[1] * tcellh[2];
    t.starttime = starttime;
    t.stoptime = stoptime;
    int rc;
    if ((rc = dalloc(s, &t.acc, 5 * nc)) || (rc = dalloc(s, &t.tacc, nc)) || (rc = dalloc(s, &t.mass, nc)) ||
        (rc = dalloc(s, &t.vcm, 3 * nc)) || (rc = dalloc(s, &t.Ti, nc)) || (rc = dalloc(s, &t.num, nc)))
        return rc;
    FMDG_CK(cudaMemsetAsync(t.num, 0, nc * sizeof(unsigned), s->stream));
    FMDG_CK(cudaMemsetAsync(t.mass, 0, nc * sizeof(double), s->stream));
    FMDG_CK(cudaMemsetAsync(t.vcm, 0, 3 * nc * sizeof(double), s->stream));
    FMDG_CK(cudaMemsetAsync(t.Ti, 0, nc * sizeof(double), s->stream));
    *handle = s->nturi++;
    invalidate_graph(s);
    return FMDG_OK;
}

extern "C" int fmdg_ttm_setup(fmdg_sys_t *s, int turi, int itc_lo, int itc_hi, const fmdg_ttm_params_t *p)
{
    if (turi < 0 || turi >= s->nturi) return fmdg_set_error("fmdg_ttm_setup: bad turi");
    DTuri &t = s->turi[turi];
    if (t.dims[0] != 1 || t.dims[1] != 1) return fmdg_set_error("fmdg_ttm_setup: 1-D grids along z only");
    if (p->type != 1 && p->type != 2) return fmdg_set_error("fmdg_ttm_setup: type 1 or 2");
    if (p->ratio < 1) return fmdg_set_error("fmdg_ttm_setup: timestep ratio must be positive");
    if (itc_lo < 1 || itc_hi > t.dims[2] - 1 || itc_lo >= itc_hi) return fmdg_set_error("fmdg_ttm_setup: range");
    const int nz = t.dims[2];
    int rc;
    if (!t.Te)
    {
        if ((rc = dalloc(s, &t.Te, nz)) || (rc = dalloc(s, &t.Te2, nz)) || (rc = dalloc(s, &t.xi, nz)) ||
            (rc = dalloc(s, &t.Ke, nz)) || (rc = dalloc(s, &t.Ce, nz)) || (rc = dalloc(s, &t.Gc, nz)) ||
            (rc = dalloc(s, &t.srcz, nz)) || (rc = dalloc(s, &t.Te_pre, nz)))
            return rc;
        std::vector<double> m1(nz, -1.0), z0(nz, 0.0);
        FMDG_CK(cudaMemcpyAsync(t.Te, m1.data(), nz * 8, cudaMemcpyHostToDevice, s->stream));
        FMDG_CK(cudaMemcpyAsync(t.Te2, m1.data(), nz * 8, cudaMemcpyHostToDevice, s->stream));
        FMDG_CK(cudaMemcpyAsync(t.Te_pre, m1.data(), nz * 8, cudaMemcpyHostToDevice, s->stream));
        FMDG_CK(cudaMemcpyAsync(t.xi, z0.data(), nz * 8, cudaMemcpyHostToDevice, s->stream));
        FMDG_CK(cudaMemcpyAsync(t.Ke, z0.data(), nz * 8, cudaMemcpyHostToDevice, s->stream));
        FMDG_CK(cudaMemcpyAsync(t.Ce, z0.data(), nz * 8, cudaMemcpyHostToDevice, s->stream));
        FMDG_CK(cudaMemcpyAsync(t.Gc, z0.data(), nz * 8, cudaMemcpyHostToDevice, s->stream));
    }
    dfree(s, (void *)t.p.T_C); dfree(s, (void *)t.p.Ct); dfree(s, (void *)t.p.C_DD);
    dfree(s, (void *)t.p.T_G); dfree(s, (void *)t.p.Gt); dfree(s, (void *)t.p.G_DD);
    TtmParams q;
    memset(&q, 0, sizeof q);
    q.type = p->type; q.ratio = p->ratio; q.min_atoms = p->min_atoms; q.nC = p->nC; q.nG = p->nG;
    q.C_gamma = p->C_gamma; q.K = p->K; q.G = p->G; q.dz2 = p->dz2; q.frontsurf = p->frontsurf;
    q.laser_t0 = p->laser_t0; q.laser_tdiff = p->laser_tdiff; q.laser_m_2sig2_inv = p->laser_m_2sig2_inv;
    q.laser_m_absdepth_inv = p->laser_m_absdepth_inv; q.laser_factor = p->laser_factor;
    q.Kzh_v2 = p->Kzh_v2; q.Kzh_A = p->Kzh_A; q.Kzh_B = p->Kzh_B;
    if (p->type == 2)
    {
        if (p->nC < 2 || p->nG < 2 || !p->T_C || !p->Ct || !p->C_DD || !p->T_G || !p->Gt || !p->G_DD)
            return fmdg_set_error("fmdg_ttm_setup: type 2 needs C(Te) and G(Te) tables");
        auto up = [&](const double *h, int n, const double **d) -> int {
            int r = dalloc(s, (double **)d, n);
            if (r) return r;
            FMDG_CK(cudaMemcpyAsync((void *)*d, h, (size_t)n * 8, cudaMemcpyHostToDevice, s->stream));
            return FMDG_OK;
        };
        if ((rc = up(p->T_C, p->nC, &q.T_C)) || (rc = up(p->Ct, p->nC, &q.Ct)) || (rc = up(p->C_DD, p->nC, &q.C_DD)) ||
            (rc = up(p->T_G, p->nG, &q.T_G)) || (rc = up(p->Gt, p->nG, &q.Gt)) || (rc = up(p->G_DD, p->nG, &q.G_DD)))
            return rc;
    }
    t.p = q;
    t.ttm = 1;
    t.itc_lo = itc_lo;
    t.itc_hi = itc_hi;
    s->ttm_turi = turi;
    Geo &g = s->g;
    g.ttm_on = 1;
    g.ttm_g2l_z = t.g2l[2];
    g.ttm_nz = nz;
    g.ttm_tcellh_z = t.tcellh[2];
    g.ttm_inv_tcellh_z = t.inv_tcellh[2];
    g.ttm_start = t.starttime;
    g.ttm_stop = t.stoptime;
    g.ttm_xi = t.xi;
    g.ttm_vcm = t.vcm;
    invalidate_graph(s);
    return FMDG_OK;
}

extern "C" int fmdg_ttm_set_te(fmdg_sys_t *s, int turi, const double *Te)
{
    if (turi < 0 || turi >= s->nturi || !s->turi[turi].Te) return fmdg_set_error("fmdg_ttm_set_te: no TTM");
    DTuri &t = s->turi[turi];
    FMDG_CK(cudaMemcpyAsync(t.Te, Te, (size_t)t.dims[2] * 8, cudaMemcpyHostToDevice, s->stream));
    return FMDG_OK;
}

extern "C" int fmdg_turi_download(fmdg_sys_t *s, int turi, unsigned *num, double *mass, double *vcm, double *Ti,
                                  double *Te, double *xi)
{
    if (turi < 0 || turi >= s->nturi) return fmdg_set_error("fmdg_turi_download: bad turi");
    FMDG_CK(cudaStreamSynchronize(s->stream));
    DTuri &t = s->turi[turi];
    const size_t nc = t.ncells;
    if (num) FMDG_D2H(num, t.num, nc * 4);
    if (mass) FMDG_D2H(mass, t.mass, nc * 8);
    if (vcm) FMDG_D2H(vcm, t.vcm, 3 * nc * 8);
    if (Ti) FMDG_D2H(Ti, t.Ti, nc * 8);
    if (t.Te)
    {
        if (Te) FMDG_D2H(Te, t.Te, (size_t)t.dims[2] * 8);
        if (xi) FMDG_D2H(xi, t.xi, (size_t)t.dims[2] * 8);
    }
    return FMDG_OK;
}

extern "C" int fmdg_ttm_download_te(fmdg_sys_t *s, int turi, int presolve, double *Te)
{
    if (turi < 0 || turi >= s->nturi || !s->turi[turi].Te) return fmdg_set_error("fmdg_ttm_download_te: no TTM");
    FMDG_CK(cudaStreamSynchronize(s->stream));
    DTuri &t = s->turi[turi];
    FMDG_D2H(Te, presolve ? t.Te_pre : t.Te, (size_t)t.dims[2] * 8);
    return FMDG_OK;
}

extern "C" int fmdg_turi_update(fmdg_sys_t *s, double dt, unsigned mask)
{
    if (!s->atoms) return FMDG_E_STATE;
    for (int k = 0; k < s->nturi; k++)
    {
        if (!(mask & (1u << k))) continue;
        int rc = fmdg_launch_turi(s, k, dt);
        if (rc) return rc;
    }
    return FMDG_OK;
}

extern "C" int fmdg_host_alloc(void **p, size_t bytes)
{
    FMDG_CK(cudaHostAlloc(p, bytes ? bytes : 1, cudaHostAllocDefault));
    return FMDG_OK;
}

extern "C" int fmdg_host_free(void *p)
{
    FMDG_CK(cudaFreeHost(p));
    return FMDG_OK;
}

// Host-buffer entry point: positions/velocities in, nsteps velocity-Verlet
// steps, positions/velocities/atom ids (new order) and the thermo record out.
// Host arrays are structure-of-arrays, 3 rows of n (the current atom count);
// pinned buffers (fmdg_host_alloc) make the copies asynchronous.
extern "C" int fmdg_run_host(fmdg_sys_t *s, int nsteps, double dt, int group, const double *x_in,
                             const double *v_in, double *x_out, double *v_out, unsigned *id_out,
                             fmdg_thermo_t *th_out)
{
    if (!s->atoms || !s->cats) return FMDG_E_STATE;
    Dyn d;
    int rc = read_dyn(s, &d);
    if (rc) return rc;
    const size_t cap = s->g.cap, n = d.n;
    if (n > 0)
    {
        const Side &S = s->g.side[d.cur];
        if (x_in) FMDG_CK(cudaMemcpy2DAsync(S.x, cap * 8, x_in, n * 8, n * 8, 3, cudaMemcpyHostToDevice, s->stream));
        if (v_in) FMDG_CK(cudaMemcpy2DAsync(S.v, cap * 8, v_in, n * 8, n * 8, 3, cudaMemcpyHostToDevice, s->stream));
    }
    if ((rc = fmdg_vv_steps(s, nsteps, dt, group, 0, 1.0, 0.0))) return rc;
    if ((rc = read_dyn(s, &d))) return rc;
    const size_t m = d.n;
    if (m > 0)
    {
        const Side &T = s->g.side[d.cur];
        if (x_out) FMDG_CK(cudaMemcpy2DAsync(x_out, m * 8, T.x, cap * 8, m * 8, 3, cudaMemcpyDeviceToHost, s->stream));
        if (v_out) FMDG_CK(cudaMemcpy2DAsync(v_out, m * 8, T.v, cap * 8, m * 8, 3, cudaMemcpyDeviceToHost, s->stream));
        if (id_out) FMDG_CK(cudaMemcpyAsync(id_out, T.atomid, m * 4, cudaMemcpyDeviceToHost, s->stream));
    }
    if (th_out) FMDG_CK(cudaMemcpyAsync(th_out, s->g.thermo, sizeof(fmdg_thermo_t), cudaMemcpyDeviceToHost, s->stream));
    FMDG_CK(cudaStreamSynchronize(s->stream));
    return FMDG_OK;
}

extern "C" int fmdg_get_thermo(fmdg_sys_t *s, fmdg_thermo_t *out)
{
    FMDG_CK(cudaMemcpyAsync(out, s->g.thermo, sizeof(fmdg_thermo_t), cudaMemcpyDeviceToHost, s->stream));
    FMDG_CK(cudaStreamSynchronize(s->stream));
    return FMDG_OK;
}

extern "C" int fmdg_get_errors(fmdg_sys_t *s, unsigned *bits, int clear)
{
    Dyn d;
    int rc = read_dyn(s, &d);
    if (rc) return rc;
    *bits = d.err;
    if (clear && d.err)
    {
        unsigned z = 0;
        FMDG_CK(cudaMemcpyAsync((char *)s->g.dyn + offsetof(Dyn, err), &z, sizeof z, cudaMemcpyHostToDevice, s->stream));
    }
    return FMDG_OK;
}

extern "C" int fmdg_add_velocity(fmdg_sys_t *s, int group, const double dv[3])
{
    if (!s->atoms) return FMDG_E_STATE;
    k_add_velocity<<<fmdg_grid(s->g.cap, 256), 256, 0, s->stream>>>(s->g, group, dv[0], dv[1], dv[2]);
    s->launches++;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

extern "C" int fmdg_change_group(fmdg_sys_t *s, int old_group, int new_group)
{
    if (!s->atoms) return FMDG_E_STATE;
    k_change_group<<<fmdg_grid(s->g.cap, 256), 256, 0, s->stream>>>(s->g, old_group, new_group);
    s->launches++;
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}

extern "C" int fmdg_sync(fmdg_sys_t *s)
{
    FMDG_CK(cudaStreamSynchronize(s->stream));
    return FMDG_OK;
}

extern "C" int fmdg_timer_start(fmdg_sys_t *s)
{
    FMDG_CK(cudaEventRecord(s->ev0, s->stream));
    return FMDG_OK;
}

extern "C" int fmdg_timer_stop(fmdg_sys_t *s, float *ms)
{
    FMDG_CK(cudaEventRecord(s->ev1, s->stream));
    FMDG_CK(cudaEventSynchronize(s->ev1));
    FMDG_CK(cudaEventElapsedTime(ms, s->ev0, s->ev1));
    return FMDG_OK;
}

extern "C" int fmdg_set_profiling(fmdg_sys_t *s, int on)
{
    s->profiling = on != 0;
    memset(s->prof_ms, 0, sizeof s->prof_ms);
    memset(s->prof_n, 0, sizeof s->prof_n);
    return FMDG_OK;
}

extern "C" int fmdg_get_profile(fmdg_sys_t *s, const char *name, float *ms, int *launches)
{
    static const char *names[6] = {"bin", "nlist", "density", "force", "turi", "ttm"};
    for (int k = 0; k < 6; k++)
        if (strcmp(name, names[k]) == 0)
        {
            *ms = s->prof_ms[k];
            *launches = s->prof_n[k];
            return FMDG_OK;
        }
    return fmdg_set_error("fmdg_get_profile: unknown phase");
}

extern "C" int fmdg_launch_count(fmdg_sys_t *s, long long *count)
{
    *count = s->launches;
    return FMDG_OK;
}

extern "C" int fmdg_flush_l2(fmdg_sys_t *s)
{
    if (!s->l2buf)
    {
        s->l2bytes = (size_t)256 << 20;
        int rc = dalloc(s, (char **)&s->l2buf, s->l2bytes);
        if (rc) return rc;
        FMDG_CK(cudaMemsetAsync(s->l2buf, 0, s->l2bytes, s->stream));
    }
    k_flush<<<1216, 256, 0, s->stream>>>((unsigned *)s->l2buf, s->l2bytes / 4);
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}
