// se2p_ff.cuh -- float-float ("double-single") arithmetic for the FP64 form.
//
// GB300 issues FP32 fused multiply-adds at about 73 times its FP64 rate
// (117 vs 1.6 per clock per SM measured), so a double-precision result is
// cheaper to build from pairs of floats than from FP64 instructions.  A
// value is hi + lo with two floats, |lo| <= ulp(hi): about 48 significant
// bits, a unit roundoff near 2^-48 = 3.6e-15.  The building blocks are the
// error-free transformations of Dekker (1971) and Knuth (TAOCP vol. 2,
// 4.2.2): TwoSum, Fast2Sum and the FMA form of TwoProduct.
//
// Conversions between double and float run at the FP64 rate on GB300, so the
// double -> (hi, lo) split is done with integer operations on the bit pattern.
// The split is exact for hi and rounds lo once: hi + lo = d (1 + delta),
// |delta| <= 2^-48, for 2^-74 <= |d| < 2^128.  Below 2^-74 lo is flushed (the
// relative error grows to 2^-24 there; every caller works with magnitudes
// relative to much larger values), zero maps to (0, 0), and inf / NaN take the
// slow conversion.
#pragma once
#include <cuda_runtime.h>

namespace se2p {

__device__ __forceinline__ float2 ff_split(double d)
{
    const int hw = __double2hiint(d);
    const unsigned lw = (unsigned)__double2loint(d);
    const int e = (hw >> 20) & 0x7ff;
    const unsigned sign = (unsigned)hw & 0x80000000u;
    if (e <= 896) return make_float2(0.f, 0.f);      // |d| < 2^-126 (and zero)
    if (e >= 1151) {                                  // |d| >= 2^128, inf, NaN
        return make_float2(__double2float_rn(d), 0.f);
    }
    const unsigned hb = sign | ((unsigned)(e - 896) << 23) | (((unsigned)hw & 0xfffffu) << 3) |
                        (lw >> 29);
    const float hi = __uint_as_float(hb);
    // lo = low 29 mantissa bits * 2^(e - 1075), with the sign of d
    const int se = e - 948;                           // float exponent field of 2^(e-1075)
    const float scale = __uint_as_float((unsigned)max(se, 0) << 23);
    const float lo = __uint_as_float(__float_as_uint(__uint2float_rn(lw & 0x1fffffffu) * scale) ^
                                     sign);
    return make_float2(hi, lo);
}

__device__ __forceinline__ double ff_to_double(float2 a)
{
    return (double)a.x + (double)a.y;
}

// s + e = a + b exactly (Knuth's TwoSum, no magnitude condition).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// s + e = a + b exactly when |a| >= |b| or a == 0 (Dekker's Fast2Sum).
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e)
{
    s = a + b;
    e = b - (s - a);
}

// Normalises an unevaluated sum (hi + lo with |lo| possibly > ulp(hi)).
__device__ __forceinline__ float2 ff_norm(float hi, float lo)
{
    float s, e;
    two_sum(hi, lo, s, e);
    return make_float2(s, e);
}

__device__ __forceinline__ float2 ff_add(float2 a, float2 b)
{
    float s, e;
    two_sum(a.x, b.x, s, e);
    e += a.y + b.y;
    float h, l;
    fast_two_sum(s, e, h, l);
    return make_float2(h, l);
}

__device__ __forceinline__ float2 ff_mul(float2 a, float2 b)
{
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    float h, l;
    fast_two_sum(p, e, h, l);
    return make_float2(h, l);
}

// a1 b1 + a2 b2 (+ a3 b3): the products' exact heads summed by TwoSum, their
// FMA-formed errors and the TwoSum errors added in the tail, normalised once.
__device__ __forceinline__ float2 ff_dot2(float2 a1, float2 b1, float2 a2, float2 b2)
{
    const float p1 = a1.x * b1.x;
    float e1 = fmaf(a1.x, b1.x, -p1);
    e1 = fmaf(a1.x, b1.y, e1);
    e1 = fmaf(a1.y, b1.x, e1);
    const float p2 = a2.x * b2.x;
    float e2 = fmaf(a2.x, b2.x, -p2);
    e2 = fmaf(a2.x, b2.y, e2);
    e2 = fmaf(a2.y, b2.x, e2);
    float s, t;
    two_sum(p1, p2, s, t);
    t += e1 + e2;
    float h, l;
    fast_two_sum(s, t, h, l);
    return make_float2(h, l);
}

__device__ __forceinline__ float2 ff_dot3(float2 a1, float2 b1, float2 a2, float2 b2, float2 a3,
                                          float2 b3)
{
    const float p1 = a1.x * b1.x;
    float e1 = fmaf(a1.x, b1.x, -p1);
    e1 = fmaf(a1.x, b1.y, e1);
    e1 = fmaf(a1.y, b1.x, e1);
    const float p2 = a2.x * b2.x;
    float e2 = fmaf(a2.x, b2.x, -p2);
    e2 = fmaf(a2.x, b2.y, e2);
    e2 = fmaf(a2.y, b2.x, e2);
    const float p3 = a3.x * b3.x;
    float e3 = fmaf(a3.x, b3.x, -p3);
    e3 = fmaf(a3.x, b3.y, e3);
    e3 = fmaf(a3.y, b3.x, e3);
    float s, t, u, v;
    two_sum(p1, p2, s, t);
    two_sum(s, p3, u, v);
    t += v + (e1 + e2 + e3);
    float h, l;
    fast_two_sum(u, t, h, l);
    return make_float2(h, l);
}

// Dot-product accumulator: (s, c) += a * b with a, b float-float.  The
// product's exact head and the TwoSum error go to the float c; s stays the
// running float sum (Ogita-Rump-Oishi Dot2 with float-float operands).
__device__ __forceinline__ void ff_dot_acc(float2 a, float2 b, float &s, float &c)
{
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    float t, err;
    two_sum(s, p, t, err);
    s = t;
    c += err + e;
}

__device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ float2 ff_sub(float2 a, float2 b) { return ff_add(a, ff_neg(b)); }

// Exact scaling by a float power of two.
__device__ __forceinline__ float2 ff_scale(float2 a, float p2) { return make_float2(a.x * p2, a.y * p2); }

__device__ __forceinline__ float2 ff_sqr(float2 a)
{
    const float p = a.x * a.x;
    float e = fmaf(a.x, a.x, -p);
    e = fmaf(2.0f * a.x, a.y, e);
    float h, l;
    fast_two_sum(p, e, h, l);
    return make_float2(h, l);
}

// a * b with b a float.
__device__ __forceinline__ float2 ff_mul_f(float2 a, float b)
{
    const float p = a.x * b;
    float e = fmaf(a.x, b, -p);
    e = fmaf(a.y, b, e);
    float h, l;
    fast_two_sum(p, e, h, l);
    return make_float2(h, l);
}

// a + b with b a float.
__device__ __forceinline__ float2 ff_add_f(float2 a, float b)
{
    float s, e;
    two_sum(a.x, b, s, e);
    e += a.y;
    float h, l;
    fast_two_sum(s, e, h, l);
    return make_float2(h, l);
}

// 1/a: the correctly rounded float reciprocal of the head, then one Newton
// step r + r (1 - a r) with the residual formed by FMAs (relative error
// about 2^-47).
__device__ __forceinline__ float2 ff_rcp(float2 a)
{
    const float r = __frcp_rn(a.x);
    float e = fmaf(-a.x, r, 1.0f);
    e = fmaf(-a.y, r, e);
    float h, l;
    fast_two_sum(r, r * e, h, l);
    return make_float2(h, l);
}

// exp(-x) for 1 <= x <= 80 in float-float, Tang's table-driven method
// (P. T. P. Tang, ACM TOMS 15(2), 1989) with 64 table entries:
// x = (n/64) ln 2 + r, |r| <= ln2/128 (+ rounding), exp(-x) =
// 2^-(n>>6) * 2^-((n&63)/64) * exp(-r).  ln2/64 is split in three floats
// (C1 with 11 significant bits, so n*C1 is exact for n < 2^13).  exp(-r) =
// 1 - r + r^2/2 - r^3 (1/6 - r/24 + r^2/120): the first three terms in
// float-float, the rest in FP32 (|r^3/6| < 3e-8, so its FP32 rounding is
// below 2e-15).  tab[j] = 2^(-j/64) as float-float.
__device__ __forceinline__ float2 ff_exp_neg(float2 x, const float2 *tab)
{
    const float C1 = 0x1.63p-7f, C2 = -0x1.bd0106p-19f, C3 = 0x1.cf79acp-46f;
    const float kd = rintf(x.x * 0x1.715476p+6f);
    const int n = (int)kd;
    const float t1 = fmaf(-kd, C1, x.x);             // exact
    const float p2 = kd * C2;
    const float e2 = fmaf(kd, C2, -p2);
    float s, e;
    two_sum(t1, -p2, s, e);
    e += (x.y - e2) - kd * C3;
    float rh, rl;
    two_sum(s, e, rh, rl);
    const float q = fmaf(fmaf(rh, 1.0f / 120.0f, -1.0f / 24.0f), rh, 1.0f / 6.0f);
    const float t3 = rh * rh * rh * q;
    const float p = rh * rh;
    float pe = fmaf(rh, rh, -p);
    pe = fmaf(2.0f * rh, rl, pe);
    float s1, e1, s2, e2b;
    two_sum(1.0f, -rh, s1, e1);
    two_sum(s1, 0.5f * p, s2, e2b);
    const float lo = (e1 + e2b) + ((0.5f * pe - rl) - t3);
    float h, l;
    fast_two_sum(s2, lo, h, l);
    const float2 m = ff_mul(make_float2(h, l), tab[n & 63]);
    return ff_scale(m, __int_as_float((127 - (n >> 6)) << 23));
}

}  // namespace se2p
