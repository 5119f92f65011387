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

// exp(x) for |x| < 80 (the double-double method of Hida, Li and Bailey):
// x = n ln2 + t with |t| <= ln2/2, exp(t) = (exp(t / 32))^32, the inner
// exponential by its Taylor series to degree 8 (|t / 32| < 0.011, truncation
// below 1e-23), five squarings, then the exact scaling by 2^n.  Relative
// error about 32 x 2^-47.
__device__ __forceinline__ dfl df_exp(dfl x)
{
    // ln2 and 1/k! (k = 2..8) as double-float constants
    const dfl ln2 = {6.931471825e-01f, -1.904654212e-09f};
    const dfl c[9] = {{1.f, 0.f}, {1.f, 0.f}, {0.5f, 0.f},
                      {1.666666716e-01f, -4.967053879e-09f}, {4.166666791e-02f, -1.241763470e-09f},
                      {8.333333768e-03f, -4.346172033e-10f}, {1.388888923e-03f, -3.363109444e-11f},
                      {1.984127011e-04f, -2.725596875e-12f}, {2.480158764e-05f, -3.406996094e-13f}};
    // n = x log2(e) rounded to an integer (|n| < 126) by the 1.5 * 2^23
    // addition; 2^n assembled from its exponent bits
    const float big = 12582912.f;
    const float nb = __fadd_rn(__fmul_rn(x.hi, 1.442695041f), big);
    const float n = __fsub_rn(nb, big);
    const dfl t = df_scale2(df_sub(x, df_mul_f(ln2, n)), 0.03125f);
    dfl p = c[8];
    for (int k = 7; k >= 0; k--) p = df_fma(p, t, c[k]);
    for (int k = 0; k < 5; k++) p = df_mul(p, p);
    const float s = __int_as_float((__float_as_int(nb) - 0x4B400000 + 127) << 23);
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
