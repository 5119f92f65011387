// Pair forces without any allocation by the library.
//
// Some callers cannot let a library call cudaMalloc: code that records the
// call into a CUDA graph (allocation is not a capturable stream operation),
// hosts that own all device memory through their own pool or arena, and
// serving loops where the implicit device synchronisation of cudaMalloc
// would stall work queued by other streams.  fmdg_pair_forces_noalloc gives
// them the binary64 LJ / Morse force evaluation of fmdg_compute_forces with
// every input and output supplied by the caller.  The only scratch it needs,
// the per-block energy partials of the deterministic two-level reduction,
// lives in a fixed file-scope device array (FMDG_NOALLOC_MAX_BLOCKS blocks
// of 128 atoms, i.e. at most FMDG_NOALLOC_MAX_ATOMS atoms per call; 512 KiB
// held by every GPU that loads the library until the process exits).
//
// Host code cannot use the array's name as a device address, so the first
// call on each device (with that device current) looks the address up with
// cudaGetSymbolAddress and keeps it; that first call should be made before
// any stream capture begins.  All calls share the one array and each call
// overwrites it completely, so calls that overlap on the GPU (different
// streams, no ordering between them) race and must be serialised by the
// caller.
//
// The first look-up is made under a lock, so first calls from several host
// threads are safe.  A cudaDeviceReset of a device invalidates the address
// kept for it: this entry point must not be called on that device again in
// the same process.  Atom kinds must lie in [0, nkinds): an atom whose kind,
// or a neighbour's kind, lies outside gets NaN forces (and the energy is
// NaN), the pair table is never read out of range.
#include <mutex>
#include <stdio.h>
#include <string.h>
#include "fmdg_internal.cuh"

#define FMDG_NOALLOC_MAX_BLOCKS 8192
#define FMDG_NOALLOC_MAX_ATOMS (FMDG_NOALLOC_MAX_BLOCKS * 128)
#define FMDG_NOALLOC_MAX_KINDS 4
#define FMDG_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) double g_noalloc_partials[FMDG_NOALLOC_MAX_BLOCKS];

namespace {

struct NoallocArgs   // passed by value: no device copy of the parameters
{
    int n, nkinds;
    int nc[3], pbc[3];
    double l[3];
    fmdg_pair_t pairs[FMDG_NOALLOC_MAX_KINDS * FMDG_NOALLOC_MAX_KINDS];
};

__device__ __forceinline__ int wrap_axis(const NoallocArgs &a, int d, int h, int o, double *s)
{
    int j = h + o;
    *s = 0.0;
    if (j < 0) { if (!a.pbc[d]) return -1; j += a.nc[d]; *s = -a.l[d]; }
    else if (j >= a.nc[d]) { if (!a.pbc[d]) return -1; j -= a.nc[d]; *s = a.l[d]; }
    return j;
}

// binary64 gather over the 27-cell stencil (same pair arithmetic as the
// binary64 path of fmdg_force.cu: src/lj.h:26-58, src/morse.h:26-58)
__global__ void __launch_bounds__(128) k_pair_noalloc(NoallocArgs a, const double *__restrict__ x,
                                                       const unsigned *__restrict__ kind,
                                                       const int *__restrict__ cell_start,
                                                       const int *__restrict__ cell_of, double *__restrict__ F,
                                                       double *partials)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = a.n;
    double pe = 0.0;
    if (i < n)
    {
        const int c = cell_of[i];
        const int cx = c / (a.nc[1] * a.nc[2]), cy = (c / a.nc[2]) % a.nc[1], cz = c % a.nc[2];
        const double xi[3] = {x[i], x[n + i], x[2 * (size_t)n + i]};
        const unsigned ki = kind[i];
        bool bad = ki >= (unsigned)a.nkinds;
        double f[3] = {0.0, 0.0, 0.0};
        for (int code = 0; code < 27; code++)
        {
            double s[3];
            const int jx = wrap_axis(a, 0, cx, code / 9 - 1, &s[0]);
            const int jy = wrap_axis(a, 1, cy, (code / 3) % 3 - 1, &s[1]);
            const int jz = wrap_axis(a, 2, cz, code % 3 - 1, &s[2]);
            if (jx < 0 || jy < 0 || jz < 0) continue;
            const int nb = jz + a.nc[2] * (jy + a.nc[1] * jx);
            for (int j = cell_start[nb]; j < cell_start[nb + 1]; j++)
            {
                if (code == 13 && j == i) continue;
                const unsigned kj = kind[j];
                if (bad || kj >= (unsigned)a.nkinds)
                {
                    bad = true;     // kinds outside the pair table: no table read
                    continue;
                }
                const fmdg_pair_t &pp = a.pairs[ki * a.nkinds + kj];
                double rv[3];
                for (int d = 0; d < 3; d++)
                {
                    double x2 = x[(size_t)d * n + j];
                    if (s[d] != 0.0) x2 = __dadd_rn(x2, s[d]);
                    rv[d] = __dsub_rn(xi[d], x2);
                }
                const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(rv[0], rv[0]), __dmul_rn(rv[1], rv[1])),
                                            __dmul_rn(rv[2], rv[2]));
                if (pp.cat == FMDG_POT_LJ)
                {
                    if (!(r2 < pp.p[2])) continue;
                    const double inv_r2 = 1.0 / r2;
                    const double inv_rs2 = pp.p[1] * inv_r2;
                    const double inv_rs6 = inv_rs2 * inv_rs2 * inv_rs2;
                    const double inv_rs12 = inv_rs6 * inv_rs6;
                    const double factor = 12.0 * pp.p[0] * inv_r2 * (inv_rs12 - 0.5 * inv_rs6);
                    for (int d = 0; d < 3; d++) f[d] += rv[d] * factor;
                    pe += 0.5 * (pp.p[0] * (inv_rs12 - inv_rs6));
                }
                else
                {
                    if (!(r2 < pp.p[3])) continue;
                    const double r = sqrt(r2);
                    const double inv_r = 1.0 / r;
                    const double e1 = exp(-pp.p[1] * (r - pp.p[2]));
                    const double e2 = e1 * e1;
                    const double factor = 2.0 * pp.p[1] * pp.p[0] * inv_r * (e2 - e1);
                    for (int d = 0; d < 3; d++) f[d] += factor * rv[d];
                    pe += 0.5 * (pp.p[0] * (e2 - 2.0 * e1));
                }
            }
        }
        if (bad)
        {
            for (int d = 0; d < 3; d++) f[d] = __longlong_as_double(0x7ff8000000000000ll);
            pe = f[0];
        }
        for (int d = 0; d < 3; d++) F[(size_t)d * n + i] = f[d];
    }
    // deterministic block sum -> this block's slot of the static partials
    __shared__ double red[4];
    for (int off = 16; off > 0; off >>= 1) pe += __shfl_down_sync(0xffffffffu, pe, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = pe;
    __syncthreads();
    if (threadIdx.x == 0) partials[blockIdx.x] = red[0] + red[1] + red[2] + red[3];
}

__global__ void k_pair_noalloc_final(const double *partials, int nblocks, double *pe_out)
{
    __shared__ double red[256];
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partials[b];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1)
    {
        if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) *pe_out = red[0];
}

double *g_partials_addr[FMDG_NOALLOC_MAX_DEVICES];
std::mutex g_partials_lock;   // guards the first look-up on each device

} // namespace

extern "C" int fmdg_pair_forces_noalloc(int n, const int nc[3], const int pbc[3], const double l[3], int nkinds,
                                        const fmdg_pair_t *pairs, const double *x, const unsigned *kind,
                                        const int *cell_start, const int *cell_of, double *F, double *pe,
                                        void *stream)
{
    if (n < 0 || n > FMDG_NOALLOC_MAX_ATOMS)
    {
        char msg[160];
        snprintf(msg, sizeof msg, "fmdg_pair_forces_noalloc: %d atoms exceed the fixed scratch limit of %d",
                 n, FMDG_NOALLOC_MAX_ATOMS);
        return fmdg_set_error(msg);
    }
    if (nkinds < 1 || nkinds > FMDG_NOALLOC_MAX_KINDS)
        return fmdg_set_error("fmdg_pair_forces_noalloc: 1..4 atom kinds");
    NoallocArgs a;
    memset(&a, 0, sizeof a);
    a.n = n;
    a.nkinds = nkinds;
    for (int d = 0; d < 3; d++)
    {
        if (nc[d] < 1) return fmdg_set_error("fmdg_pair_forces_noalloc: bad cell grid");
        a.nc[d] = nc[d];
        a.pbc[d] = pbc[d] ? 1 : 0;
        a.l[d] = l[d];
    }
    for (int k = 0; k < nkinds * nkinds; k++)
    {
        if (pairs[k].cat != FMDG_POT_LJ && pairs[k].cat != FMDG_POT_MORSE)
            return fmdg_set_error("fmdg_pair_forces_noalloc: LJ and Morse pairs only");
        a.pairs[k] = pairs[k];
    }
    int dev = 0;
    FMDG_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= FMDG_NOALLOC_MAX_DEVICES) return fmdg_set_error("fmdg_pair_forces_noalloc: device id");
    double *partials = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_partials_lock);
        if (g_partials_addr[dev] == nullptr)
        {
            void *p = nullptr;
            FMDG_CK(cudaGetSymbolAddress(&p, g_noalloc_partials));
            g_partials_addr[dev] = (double *)p;
        }
        partials = g_partials_addr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    const int nb = n > 0 ? (n + 127) / 128 : 1;
    k_pair_noalloc<<<nb, 128, 0, st>>>(a, x, kind, cell_start, cell_of, F, partials);
    k_pair_noalloc_final<<<1, 256, 0, st>>>(partials, nb, pe);
    FMDG_CK(cudaGetLastError());
    return FMDG_OK;
}
