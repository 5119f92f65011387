// Double-binary32 ("double-float") arithmetic for the binary64 kernels.
//
// GB300 issues binary64 at 1/64 of the binary32 rate, so the binary64 pair
// loops are bound by the binary64 pipe.  A value carried as the unevaluated
// sum hi + lo of two binary32 numbers (|lo| <= ulp(hi)/2) has about 48
// significant bits; the operations below keep that precision (errors of a
// few units of 2^-48 relative) with binary32 instructions only.  The
// binary64 modes use them where the result needs binary64 accuracy (pair
// geometry, spline evaluation, sums) and the reference's binary64 rounding
// is not itself part of the result: every cutoff decision near the cutoff
// is still taken in binary64, as the reference forms it.
//
// Published methods: Knuth's TwoSum (The Art of Computer Programming,
// vol. 2, 4.2.2, theorem B), Dekker's FastTwoSum and the exact product
// (Dekker 1971, "A floating-point technique for extending the available
// precision", with the product's error term from a fused multiply-add),
// and the double-word addition and multiplication built from them as in
// Hida, Li and Bailey, "Algorithms for quad-double precision floating
// point arithmetic" (ARITH 2001), sections 3-4 (the "sloppy" addition).
// Explicit _rn intrinsics keep the compiler from contracting or
// reassociating the error terms.
#pragma once

#include <cuda_runtime.h>

struct dfl
{
    float hi, lo;
};

// s + e == a + b exactly (Knuth)
__device__ __forceinline__ dfl two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// s + e == a + b exactly when |a| >= |b| (Dekker)
__device__ __forceinline__ dfl fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// p + e == a * b exactly (fused multiply-add error term)
__device__ __forceinline__ dfl two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.hi, -a.lo}; }

// a + b; error about 2^-46 (|a| + |b|)
__device__ __forceinline__ dfl df_add(dfl a, dfl b)
{
    const dfl s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}

__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }

// a * b; error about 2^-46 |a b|
__device__ __forceinline__ dfl df_mul(dfl a, dfl b)
{
    const dfl p = two_prod(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.lo, p.lo);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p.hi, e);
}

// a * b with b a binary32 number
__device__ __forceinline__ dfl df_mul_f(dfl a, float b)
{
    const dfl p = two_prod(a.hi, b);
    return fast_two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}

// a * 2^k: exact
__device__ __forceinline__ dfl df_scale2(dfl a, float pow2) { return {a.hi * pow2, a.lo * pow2}; }

// a * b + c
__device__ __forceinline__ dfl df_fma(dfl a, dfl b, dfl c) { return df_add(df_mul(a, b), c); }

__device__ __forceinline__ double df_to_double(dfl a) { return (double)a.hi + (double)a.lo; }

// Hardware approximations (PTX rcp.approx / rsqrt.approx, relative error
// about 2^-22) as Newton starting points; conversion and rounding
// instructions are avoided in the pair loops (they issue at the binary64
// rate on GB300).
__device__ __forceinline__ float rcp_start(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_start(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// 1 / a: binary32 reciprocal y0, then one Newton step y0 + y0 (1 - a y0)
// evaluated in double-float (the residual doubles the precision)
__device__ __forceinline__ dfl df_rcp(dfl a)
{
    const float y0 = rcp_start(a.hi);
    const dfl e = df_sub({1.f, 0.f}, df_mul_f(a, y0));
    return df_add({y0, 0.f}, df_mul_f(e, y0));
}

// sqrt(a), a > 0: binary32 root r0 = a * rsqrt(a), then one Newton step
// r0 + (a - r0^2) / (2 r0) with the residual in double-float
__device__ __forceinline__ dfl df_sqrt(dfl a)
{
    const float y0 = rsqrt_start(a.hi);
    const float r0 = __fmul_rn(a.hi, y0);
    const dfl res = df_sub(a, two_prod(r0, r0));
    return df_add({r0, 0.f}, df_mul_f(res, __fmul_rn(0.5f, y0)));
}

// 2^(j/32), j = 0..31, as double-float (hi, lo): each rounded from a
// 200-bit value (relative error below 2^-49)
static __device__ const float2 df_exp2_tab[32] = {
    {0x1.p+0f, 0.f}, {0x1.059b0ep+0f, -0x1.9d4f52p-25f}, {0x1.0b5586p+0f, 0x1.9f3122p-25f}, {0x1.11301ep+0f, -0x1.fdb496p-25f},
    {0x1.172b84p+0f, -0x1.c15742p-27f}, {0x1.1d4874p+0f, -0x1.d2e8cap-25f}, {0x1.2387a6p+0f, 0x1.ceac48p-25f}, {0x1.29e9e0p+0f, -0x1.5c0424p-25f},
    {0x1.306fe0p+0f, 0x1.4636e2p-25f}, {0x1.371a74p+0f, -0x1.18aac6p-25f}, {0x1.3dea64p+0f, 0x1.824684p-25f}, {0x1.44e086p+0f, 0x1.8624b4p-30f},
    {0x1.4bfdaep+0f, -0x1.593abcp-25f}, {0x1.5342b6p+0f, -0x1.2c5610p-25f}, {0x1.5ab07ep+0f, -0x1.5bd5ecp-27f}, {0x1.6247ecp+0f, -0x1.f8b550p-25f},
    {0x1.6a09e6p+0f, 0x1.9fcef4p-26f}, {0x1.71f75ep+0f, 0x1.1d8beep-25f}, {0x1.7a1148p+0f, -0x1.829fd0p-25f}, {0x1.82589ap+0f, -0x1.accc7cp-26f},
    {0x1.8ace54p+0f, 0x1.15506ep-27f}, {0x1.93737cp+0f, -0x1.e64744p-25f}, {0x1.9c4918p+0f, 0x1.51f848p-27f}, {0x1.a5503cp+0f, -0x1.b83b54p-25f},
    {0x1.ae89fap+0f, -0x1.a94b14p-26f}, {0x1.b7f770p+0f, -0x1.a09438p-25f}, {0x1.c199bep+0f, -0x1.3d56b2p-27f}, {0x1.cb720ep+0f, -0x1.8837ccp-27f},
    {0x1.d5818ep+0f, -0x1.822dbcp-27f}, {0x1.dfc974p+0f, -0x1.908c94p-25f}, {0x1.ea4afap+0f, 0x1.52486cp-27f}, {0x1.f50766p+0f, -0x1.246eb0p-26f}};

// exp(x) for |x| < 80, table-driven (Tang's method, ACM TOMS 15(2), 1989,
// in double-float): x = (32 m + j) ln2/32 + r with |r| <= ln2/64, so
// exp(x) = 2^m 2^(j/32) exp(r); exp(r) by its Taylor series to degree 6
// (truncation below 4e-18), the terms from r^4 on summed in binary32 (they
// enter multiplied by r^3 < 1.3e-6); 2^m assembled from exponent bits.
// Relative error about 1e-13 for |x| <= 30, dominated by the rounding of x
// itself.
__device__ __forceinline__ dfl df_exp(dfl x)
{
    const dfl ln2_32 = {0x1.62e43p-6f, -0x1.05c61p-34f};
    const dfl c3 = {0x1.555556p-3f, -0x1.555556p-28f};   // 1/6
    // n = x 32/ln2 rounded to an integer (|n| < 2^12) by the 1.5 * 2^23
    // addition: no conversion instruction
    const float big = 12582912.f;
    const float nb = __fadd_rn(__fmul_rn(x.hi, 46.16624f), big);
    const float n = __fsub_rn(nb, big);
    const int ni = __float_as_int(nb) - 0x4B400000;
    const dfl r = df_sub(x, df_mul_f(ln2_32, n));
    const float rh = r.hi;
    const float t = __fmul_rn(rh, __fmaf_rn(rh, __fmaf_rn(rh, 1.f / 720.f, 1.f / 120.f), 1.f / 24.f));
    dfl p = df_add(c3, {t, 0.f});
    p = df_add({0.5f, 0.f}, df_mul(r, p));
    p = df_add({1.f, 0.f}, df_mul(r, p));
    p = df_add({1.f, 0.f}, df_mul(r, p));
    const float2 tj = df_exp2_tab[ni & 31];
    p = df_mul(p, {tj.x, tj.y});
    const float s = __int_as_float(((ni >> 5) + 127) << 23);
    return {__fmul_rn(p.hi, s), __fmul_rn(p.lo, s)};
}

// nearest double-float of a binary64 number (hi = x rounded to binary32,
// lo = the rounded remainder)
__host__ __device__ __forceinline__ float2 df_split(double x)
{
    const float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}

__device__ __forceinline__ dfl df_of(float2 v) { return {v.x, v.y}; }

// Natural cubic spline in the interval fraction b (the coefficient form of
// the binary64 tables: y = k0 + k1 b + k2 b^2 + k3 b^3), rows stored as two
// float4 (hi parts, lo parts)
__device__ __forceinline__ dfl df_spl_val(float4 h, float4 l, dfl b)
{
    dfl t = df_fma({h.w, l.w}, b, {h.z, l.z});
    t = df_fma(t, b, {h.y, l.y});
    return df_fma(t, b, {h.x, l.x});
}

// dy/dx = (k1 + 2 k2 b + 3 k3 b^2) * inv_h
__device__ __forceinline__ dfl df_spl_der(float4 h, float4 l, dfl b, dfl inv_h)
{
    dfl t = df_fma(df_mul_f({h.w, l.w}, 3.f), b, df_scale2({h.z, l.z}, 2.f));
    t = df_fma(t, b, {h.y, l.y});
    return df_mul(t, inv_h);
}
