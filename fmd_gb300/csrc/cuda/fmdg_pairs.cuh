// Device helpers shared by the pair kernels of the single-system path
// (fmdg_force.cu) and of the packed skin-list path (fmdg_skin.cu): pair
// table in shared memory, stencil codes, spline evaluation, deterministic
// block reductions and the thermo record.
#pragma once

#include "fmdg_internal.cuh"
#include "fmdg_df.cuh"

namespace {

enum { CAT_LJ = 1, CAT_EAM = 2, CAT_MORSE = 3, CAT_HYBRID = 4 };

// Shared per-block potential data.  DF (binary64 mode) adds the
// double-float parameters and offset remainders; ONE (kernels for systems
// of one kind) holds the single pair.  The binary32 kernels carry
// one-element placeholders so that they keep a small shared footprint: the
// rest of the SM's 256 KB of L1/shared stays L1 cache for the list and
// position gathers.
template <bool DF, bool ONE = false>
struct SmemPotT
{
    static constexpr int NP = ONE ? 1 : FMDG_MAXK * FMDG_MAXK;
    static constexpr int NPD = DF ? NP : 1;
    fmdg_pair_t pairs[NP];
    float pf[NP][4];
    float2 pd[NPD][4];  // double-float parameters (binary64 mode)
    double mass[FMDG_MAXK];
    double hk[FMDG_MAXK];   // half kick dt * 0.5 / m of each kind (one division per kind)
    int elem[FMDG_MAXK];
    // per-step kernels only (ONE: the skin kernels' one-kind layout has its own offsets)
    float4 off[ONE ? 1 : 27];    // image offset of stencil code c: (ox, oy, oz) * cellh (binary32)
    float4 offl[ONE ? 1 : 27];   // the remainders (ox, oy, oz) * (cellh - binary32 cellh): off + offl = the binary64 offset
};

// one 32-byte table row (two float4) in a single 256-bit load; p must be
// 32-byte aligned (the row tables are whole allocations, checked when they
// are built)
__device__ __forceinline__ void ld_row32(const float4 *p, float4 &a, float4 &b)
{
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

// small integer v (|v| < 2^22) as binary32 without a conversion
// instruction (conversions issue at the binary64 rate on GB300)
__device__ __forceinline__ float small_int_f(int v) { return __int_as_float(0x4B400000 + v) - 12582912.f; }

// Block prologue: pair parameters, per-kind constants and the 27 stencil
// offsets into shared memory.  DF: also the double-float parameters and
// offset remainders (binary64 mode).  Everything was formed on the host
// (no binary64 or conversion work here).
template <bool DF, bool ONE>
__device__ __forceinline__ void load_pot(const Geo &g, SmemPotT<DF, ONE> &sp, const float4 *pf = nullptr)
{
    // pf: the binary32 parameter table (default g.pairf; the skin kernels
    // pass skin_params(g), their scaled frame)
    if (!pf) pf = g.pairf;
    const int nk2 = ONE ? 1 : g.nkinds * g.nkinds;
    for (int k = threadIdx.x; k < nk2; k += blockDim.x)
    {
        sp.pairs[k] = g.pairs[k];
        const float4 f = pf[k];
        sp.pf[k][0] = f.x; sp.pf[k][1] = f.y; sp.pf[k][2] = f.z; sp.pf[k][3] = f.w;
        if (DF)
            for (int q = 0; q < 4; q++) sp.pd[k][q] = g.paird[4 * k + q];
    }
    for (int k = threadIdx.x; k < g.nkinds; k += blockDim.x)
    {
        sp.mass[k] = g.mass[k];
        sp.hk[k] = g.st.hk[k];
        sp.elem[k] = g.eam_elem[k];
    }
    // remainders cellh - binary32 cellh (3 binary64 operations per block)
    const float lx = (float)(g.cellh[0] - (double)g.cellh_f[0]), ly = (float)(g.cellh[1] - (double)g.cellh_f[1]),
                lz = (float)(g.cellh[2] - (double)g.cellh_f[2]);
    for (int c = threadIdx.x; c < (ONE ? 0 : 27); c += blockDim.x)
    {
        const float ox = small_int_f(c / 9 - 1), oy = small_int_f((c / 3) % 3 - 1), oz = small_int_f(c % 3 - 1);
        sp.off[c] = make_float4(ox * g.cellh_f[0], oy * g.cellh_f[1], oz * g.cellh_f[2], 0.f);
        sp.offl[c] = make_float4(ox * lx, oy * ly, oz * lz, 0.f);
    }
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

// binary64 pair geometry: rv = x_i - (x_j + image shift), r2 summed without
// fused multiply-adds as the reference does (src/forces.h:25-34)
struct Geom64 { double rv[3]; double r2; };

// double-float pair geometry (binary64 mode) from cell-local
// coordinates hi + lo (a row of xdf): rv = x_i - x_j - offset * cellh, the
// image shift of a periodic neighbour being offset * cellh in the cell
// frame; r^2 from exact squares of the hi parts.  Agrees with the
// reference's binary64 geometry to about 1e-14 relative.
struct GeomDF { dfl rv[3]; dfl r2; };

__device__ __forceinline__ GeomDF geom_df(float4 ih4, float4 il4, float4 jh4, float4 jl4, float4 oh4, float4 ol4)
{
    const float ih[3] = {ih4.x, ih4.y, ih4.z}, il[3] = {il4.x, il4.y, il4.z};
    const float jh[3] = {jh4.x, jh4.y, jh4.z}, jl[3] = {jl4.x, jl4.y, jl4.z};
    const float oha[3] = {oh4.x, oh4.y, oh4.z}, ola[3] = {ol4.x, ol4.y, ol4.z};
    GeomDF p;
    for (int d = 0; d < 3; d++)
    {
        const float oh = oha[d], ol = ola[d];
        const dfl a = two_sum(ih[d], -jh[d]);
        const dfl b = two_sum(a.hi, -oh);
        const float lo = __fadd_rn(__fadd_rn(__fsub_rn(__fsub_rn(il[d], jl[d]), ol), a.lo), b.lo);
        p.rv[d] = fast_two_sum(b.hi, lo);
    }
    const dfl s0 = two_prod(p.rv[0].hi, p.rv[0].hi), s1 = two_prod(p.rv[1].hi, p.rv[1].hi);
    const dfl s2 = two_prod(p.rv[2].hi, p.rv[2].hi);
    const dfl t = two_sum(s0.hi, s1.hi);
    const dfl u = two_sum(t.hi, s2.hi);
    float cross = __fmul_rn(p.rv[0].hi, p.rv[0].lo);
    cross = __fmaf_rn(p.rv[1].hi, p.rv[1].lo, cross);
    cross = __fmaf_rn(p.rv[2].hi, p.rv[2].lo, cross);
    const float lo = __fadd_rn(__fadd_rn(__fadd_rn(s0.lo, s1.lo), __fadd_rn(s2.lo, t.lo)),
                               __fadd_rn(u.lo, __fmul_rn(2.f, cross)));
    p.r2 = fast_two_sum(u.hi, lo);
    return p;
}

// interval k = min(floor(q), kmax) and fraction b = q - k of a double-float
// table coordinate 0 <= q < 2^22, without conversion instructions (they
// issue at the binary64 rate on GB300): adding 2^23 rounding towards minus
// infinity leaves floor(q.hi) in the significand
__device__ __forceinline__ int df_table_index(dfl q, float kmax, dfl &b)
{
    float kf = __fadd_rd(q.hi, 8388608.f) - 8388608.f;
    if (kf == q.hi && q.lo < 0.f) kf -= 1.f;
    kf = fminf(kf, kmax);
    b = fast_two_sum(__fsub_rn(q.hi, kf), q.lo);
    return __float_as_int(kf + 8388608.f) - 0x4B000000;
}

// a binary64 pair geometry as double-float (exact splits)
__device__ __forceinline__ GeomDF geom_df_of64(const Geom64 &q)
{
    GeomDF p;
    for (int d = 0; d < 3; d++) p.rv[d] = df_of(df_split(q.rv[d]));
    p.r2 = df_of(df_split(q.r2));
    return p;
}

// Binary64-mode pair arithmetic in double-float, in the reference's formulas
// -- LJ src/lj.h:35-56, Morse src/morse.h:35-56, EAM src/eam.h:186-226 --
// for a pair of category cat: f_i += fa * rv, energy share eh.  fpj() gives
// F'(rho_j) as a double-float; it is called for EAM pairs only.
template <typename FPJ, bool DF, bool ONE>
__device__ __forceinline__ void df_pair(const Geo &g, const SmemPotT<DF, ONE> &sp, int pidx, const fmdg_pair_t &pp, int cat,
                                        const GeomDF &p, dfl fpi, dfl inv_h, float kmax, int nint, size_t ne,
                                        FPJ &&fpj, dfl &fa, dfl &eh)
{
    if (cat == FMDG_POT_LJ)
    {
        const dfl eps4 = df_of(sp.pd[pidx][0]), sig2 = df_of(sp.pd[pidx][1]);
        const dfl inv_r2 = df_rcp(p.r2);
        const dfl s2 = df_mul(sig2, inv_r2);
        const dfl s6 = df_mul(df_mul(s2, s2), s2);
        const dfl s12 = df_mul(s6, s6);
        fa = df_mul(df_mul(df_mul_f(eps4, 12.f), inv_r2), df_sub(s12, df_scale2(s6, 0.5f)));
        eh = df_scale2(df_mul(eps4, df_sub(s12, s6)), 0.5f);
    }
    else if (cat == FMDG_POT_MORSE)
    {
        const dfl D0 = df_of(sp.pd[pidx][0]), al = df_of(sp.pd[pidx][1]);
        const dfl r0 = df_of(sp.pd[pidx][2]);
        const dfl r = df_sqrt(p.r2);
        const dfl inv_r = df_rcp(r);
        const dfl e1 = df_exp(df_mul(df_neg(al), df_sub(r, r0)));
        const dfl e2 = df_mul(e1, e1);
        fa = df_mul(df_mul(df_scale2(df_mul(al, D0), 2.f), inv_r), df_sub(e2, e1));
        eh = df_scale2(df_mul(D0, df_sub(e2, df_scale2(e1, 2.f))), 0.5f);
    }
    else
    {
        dfl b;
        const int ir2 = df_table_index(df_mul(p.r2, inv_h), kmax, b);
        const int ei = pp.iloc, ej = pp.jloc;
        float4 ph0, ph1, ri0, ri1;
        ld_row32(g.pkd_phi + 2 * (((size_t)ei * ne + ej) * nint + ir2), ph0, ph1);
        ld_row32(g.pkd_rho + 2 * ((size_t)ei * nint + ir2), ri0, ri1);
        const dfl phi_d = df_spl_der(ph0, ph1, b, inv_h);
        const dfl rho_ip = df_spl_der(ri0, ri1, b, inv_h);
        dfl rho_jp = rho_ip;
        if (ei != ej)
        {
            float4 rj0, rj1;
            ld_row32(g.pkd_rho + 2 * ((size_t)ej * nint + ir2), rj0, rj1);
            rho_jp = df_spl_der(rj0, rj1, b, inv_h);
        }
        const dfl fj = fpj();
        fa = df_neg(df_scale2(df_add(df_add(df_mul(fpi, rho_jp), df_mul(fj, rho_ip)), phi_d), 2.f));
        eh = df_scale2(df_spl_val(ph0, ph1, b), 0.5f);
    }
}

// EAM density term f_elem(j)(r^2) of an EAM pair (src/eam.h:278-300)
__device__ __forceinline__ dfl df_rho(const Geo &g, const fmdg_pair_t &pp, const GeomDF &p, dfl inv_h, float kmax,
                                      int nint)
{
    dfl b;
    const int ir2 = df_table_index(df_mul(p.r2, inv_h), kmax, b);
    float4 r0, r1;
    ld_row32(g.pkd_rho + 2 * ((size_t)pp.jloc * nint + ir2), r0, r1);
    return df_spl_val(r0, r1, b);
}

// Sum over the 32 lanes of a warp of v[0..NV), NV <= 8, by a transposing
// butterfly: each exchange halves the values a lane carries (v padded to 8),
// 4 + 2 + 1 + 1 + 1 additions per lane instead of 5 NV.  Value k ends in
// every lane whose bits 4, 3, 2 spell k (bit 4 the most significant);
// returns the value of this lane's index.  Fixed order: deterministic.
template <int NV>
__device__ __forceinline__ double warp_sum_transposed(const double (&v)[NV], int lane)
{
    static_assert(NV >= 1 && NV <= 8, "at most 8 values");
    double a[8];
    for (int k = 0; k < 8; k++) a[k] = (k < NV) ? v[k] : 0.0;
    const bool up4 = (lane & 16) != 0;
    double b[4];
    for (int q = 0; q < 4; q++)
    {
        const double keep = up4 ? a[q + 4] : a[q], give = up4 ? a[q] : a[q + 4];
        b[q] = keep + __shfl_xor_sync(0xffffffffu, give, 16);
    }
    const bool up3 = (lane & 8) != 0;
    double c[2];
    for (int q = 0; q < 2; q++)
    {
        const double keep = up3 ? b[q + 2] : b[q], give = up3 ? b[q] : b[q + 2];
        c[q] = keep + __shfl_xor_sync(0xffffffffu, give, 8);
    }
    const bool up2 = (lane & 4) != 0;
    const double keep = up2 ? c[1] : c[0], give = up2 ? c[0] : c[1];
    double d = keep + __shfl_xor_sync(0xffffffffu, give, 4);
    d += __shfl_xor_sync(0xffffffffu, d, 2);
    d += __shfl_xor_sync(0xffffffffu, d, 1);
    return d;
}

// Deterministic block reduction of NV doubles; thread 0 writes out[0..NV).
template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double *out)
{
    __shared__ double red[32][NV];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (NV >= 3)
    {
        const double s = warp_sum_transposed<NV>(v, lane);
        const int k = ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1);
        if ((lane & 3) == 0 && k < NV) red[w][k] = s;
    }
    else
    {
        for (int k = 0; k < NV; k++)
            for (int off = 16; off > 0; off >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
        if (lane == 0)
            for (int k = 0; k < NV; k++) red[w][k] = v[k];
    }
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

// binary32 partial sums of at most 8 terms (one tick per list entry
// visited, so the lanes of a warp flush together), accumulated into the
// unevaluated sum hi + lo of two binary32 numbers by Knuth's TwoSum: the
// running sum carries about 48 significant bits, as good as a binary64
// accumulation of the same partials for these sums, with no binary64
// instruction in the pair loop (binary64 issues at 1/64 of the binary32
// rate on GB300).  total() = hi + lo in binary64.
template <int NV>
struct Acc32
{
    float part[NV];
    float hi[NV], lo[NV];
    int n;
    __device__ __forceinline__ Acc32() : n(0)
    {
        for (int k = 0; k < NV; k++) { part[k] = 0.f; hi[k] = 0.f; lo[k] = 0.f; }
    }
    __device__ __forceinline__ void tick()
    {
        if (++n == 8) flush();
    }
    // k entries visited at once (rounds of four: the same flush points as
    // k single ticks)
    __device__ __forceinline__ void entries(int k)
    {
        n += k;
        if (n >= 8) flush();
    }
    __device__ __forceinline__ void flush()
    {
        for (int k = 0; k < NV; k++)
        {
            const float s = __fadd_rn(hi[k], part[k]);
            const float bp = __fsub_rn(s, hi[k]);
            const float err = __fadd_rn(__fsub_rn(hi[k], __fsub_rn(s, bp)), __fsub_rn(part[k], bp));
            lo[k] = __fadd_rn(lo[k], err);
            hi[k] = s;
            part[k] = 0.f;
        }
        n = 0;
    }
    __device__ __forceinline__ double total(int k) const { return (double)hi[k] + (double)lo[k]; }
};

// Second level: sums the per-block partials in a fixed order, writes the
// thermo record (src/integrators.c:78-92) and, when a Berendsen thermostat
// is active, the velocity scale of the next start step
// (src/integrators.c:44-50): lambda = sqrt(1 + dt/tau * (T0/T - 1)).
// Partial rows per block: 0 pair energy, 1 m v^2, 2-4 m v, 5 count,
// 6 pair virial, 8 embedding energy.  keep_pe: the energy and virial of the
// last force evaluation stay (thermo-only reductions).
// Run by one whole block of at most 256 threads.
__device__ __forceinline__ void final_reduce(const Geo &g, int nblocks, int keep_pe, int with_emb, int thermostat,
                             double dt, double tau, double T0)
{
    __shared__ double red[8][8];
    const int t = threadIdx.x;
    double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int b = t; b < nblocks; b += blockDim.x)
    {
        for (int k = 0; k < 6; k++) s[k] += __ldcg(&g.partials[(size_t)k * nblocks + b]);
        if (with_emb) s[6] += __ldcg(&g.partials[(size_t)nblocks * 8 + b]);
        if (!keep_pe) s[7] += __ldcg(&g.partials[(size_t)nblocks * 6 + b]);
    }
    for (int k = 0; k < 8; k++)
        for (int off = 16; off > 0; off >>= 1) s[k] += __shfl_down_sync(0xffffffffu, s[k], off);
    if ((t & 31) == 0)
        for (int k = 0; k < 8; k++) red[t >> 5][k] = s[k];
    __syncthreads();
    if (t == 0)
    {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++)
            for (int k = 0; k < 8; k++) red[0][k] += red[w][k];
        fmdg_thermo_t *th = g.thermo;
        const double mv2 = red[0][1];
        const double N = red[0][5];
        th->kinetic = 0.5 * mv2;
        th->temperature = mv2 / (3.0 * N * K_BOLTZMANN_D);
        th->momentum[0] = red[0][2];
        th->momentum[1] = red[0][3];
        th->momentum[2] = red[0][4];
        th->count = N;
        if (!keep_pe)
        {
            th->potential = red[0][0] + red[0][6];
            th->virial = red[0][7];
        }
        if (thermostat)
            g.dyn->lambda = sqrt(1 + dt / tau * (T0 / th->temperature - 1));
    }
}

// ---- pair terms: force factor f (F_i += f * rv, rv = x_i - x_j) and half
// the pair energy (each atom of the pair takes half)
// LJ (src/lj.h:35-56): p = {4 eps, sigma^2, rc^2}
__device__ __forceinline__ void lj_pair(double r2, const fmdg_pair_t &pp, double &f, double &e)
{
    const double inv_r2 = 1.0 / r2;
    const double inv_rs2 = pp.p[1] * inv_r2;
    const double inv_rs6 = inv_rs2 * inv_rs2 * inv_rs2;
    const double inv_rs12 = inv_rs6 * inv_rs6;
    f = 12.0 * pp.p[0] * inv_r2 * (inv_rs12 - 0.5 * inv_rs6);
    e = 0.5 * (pp.p[0] * (inv_rs12 - inv_rs6));
}
__device__ __forceinline__ void lj_pair(float r2, float eps4, float sig2, float &f, float &e)
{
    const float inv_r2 = __fdividef(1.f, r2);
    const float inv_rs2 = sig2 * inv_r2;
    const float inv_rs6 = inv_rs2 * inv_rs2 * inv_rs2;
    const float inv_rs12 = inv_rs6 * inv_rs6;
    f = 12.f * eps4 * inv_r2 * (inv_rs12 - 0.5f * inv_rs6);
    e = 0.5f * (eps4 * (inv_rs12 - inv_rs6));
}
// Hardware approximations (PTX ex2.approx / rsqrt.approx / rcp.approx,
// flush-to-zero; relative error about 2^-22) for the binary32 pair
// arithmetic of the lean kernels; a mixed-precision pair never produces a
// subnormal argument or result in them.
__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_approx(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Morse (src/morse.h:35-56): p = {D0, alpha, r0, rc^2}
__device__ __forceinline__ void morse_pair(double r2, const fmdg_pair_t &pp, double &f, double &e)
{
    const double r = sqrt(r2);
    const double inv_r = 1.0 / r;
    const double e1 = exp(-pp.p[1] * (r - pp.p[2]));
    const double e2 = e1 * e1;
    f = 2.0 * pp.p[1] * pp.p[0] * inv_r * (e2 - e1);
    e = 0.5 * (pp.p[0] * (e2 - 2.0 * e1));
}
// (binary32: exp(-alpha (r - r0)) as 2^((r0 - r) alpha log2(e)))
__device__ __forceinline__ void morse_pair(float r2, float D0, float al, float r0, float &f, float &e)
{
    const float inv_r = rsqrtf(r2);
    const float r = r2 * inv_r;
    const float e1 = exp2f((r0 - r) * (al * 1.44269504f));
    const float e2 = e1 * e1;
    f = 2.f * al * D0 * inv_r * (e2 - e1);
    e = 0.5f * (D0 * (e2 - 2.f * e1));
}

} // namespace
