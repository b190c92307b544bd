// Double-float ("two-float") arithmetic: a value is an unevaluated sum
// hi + lo of two FP32 numbers, ~48-bit significand.  Used by the mixed path
// to run FP64-accuracy arithmetic on GB300's FP32 pipe (~64x its FP64 rate).
//
// Building blocks are the error-free transformations: TwoSum (Knuth),
// FastTwoSum (Dekker), TwoProd via fmaf; products and sums follow Dekker
// (1971) and Hida, Li & Bailey (2001).  sin/cos: Cody-Waite reduction of an
// FP64 argument by pi/2 (pi/2 held as two doubles), then the Taylor series of
// sin and cos on [-pi/4, pi/4] evaluated by Horner in double-float; the
// coefficients are (-1)^k / n! (exact rationals rounded to double, split).
#pragma once
#include <cuda_runtime.h>

namespace ia {

struct dfl {
    float hi, lo;
};

__device__ __forceinline__ dfl df_make(float h, float l) { return dfl{h, l}; }

__device__ __forceinline__ dfl df_from_double(double x)
{
    float h = __double2float_rn(x);
    return dfl{h, __double2float_rn(x - (double)h)};
}

__device__ __forceinline__ double df_to_double(dfl a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ dfl fast_two_sum(float a, float b)
{
    float s = a + b;
    return dfl{s, b - (s - a)};
}

__device__ __forceinline__ dfl two_sum(float a, float b)
{
    float s = a + b;
    float v = s - a;
    return dfl{s, (a - (s - v)) + (b - v)};
}

__device__ __forceinline__ dfl df_add(dfl a, dfl b)
{
    dfl s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ dfl df_neg(dfl a) { return dfl{-a.hi, -a.lo}; }
__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }

__device__ __forceinline__ dfl df_mul(dfl a, dfl b)
{
    float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}

// acc += a * b with the low word left unnormalised (renormalise with df_norm)
__device__ __forceinline__ void df_mac(dfl &acc, dfl a, dfl b)
{
    float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    dfl s = two_sum(acc.hi, p);
    acc.hi = s.hi;
    acc.lo += s.lo + e;
}

__device__ __forceinline__ dfl df_norm(dfl a) { return fast_two_sum(a.hi, a.lo); }

// 1/sqrt(x) for x > 0: FP32 estimate, one Newton step in double-float
// (y' = y + y (1 - x y^2) / 2)
__device__ __forceinline__ dfl df_rsqrt(dfl x)
{
    float y0 = rsqrtf(x.hi);
    dfl y{y0, 0.0f};
    dfl r = df_mul(x, df_mul(y, y));                 // x y^2
    dfl c = df_add(dfl{1.0f, 0.0f}, df_neg(r));       // 1 - x y^2
    return df_add(y, df_mul(y, dfl{0.5f * c.hi, 0.5f * c.lo}));
}

// Taylor coefficients (-1)^k/(2k+1)! and (-1)^k/(2k)! as double-float pairs
struct DfTrigCoef {
    float sh[9], sl[9];   // sin: k = 0..8  (t^1 .. t^17)
    float ch[10], cl[10]; // cos: k = 0..9  (t^0 .. t^18)
};

__host__ inline DfTrigCoef df_trig_coefficients()
{
    DfTrigCoef c;
    double f = 1.0;   // n!
    for (int n = 0; n <= 18; ++n) {
        if (n > 0) f *= n;
        double v = ((n / 2) % 2 ? -1.0 : 1.0) / f;
        float h = (float)v, l = (float)(v - (double)h);
        if (n % 2) { c.sh[n / 2] = h; c.sl[n / 2] = l; }
        else { c.ch[n / 2] = h; c.cl[n / 2] = l; }
    }
    return c;
}

// sin and cos of an FP64 argument |theta| < 2^20, results in double-float
__device__ __forceinline__ void df_sincos(double theta, const DfTrigCoef &C, dfl &s, dfl &c)
{
    const double PIO2_HI = 1.5707963267948966, PIO2_LO = 6.123233995736766e-17;
    const double n = rint(theta * 0.6366197723675814);
    double t = fma(-n, PIO2_HI, theta);
    t = fma(-n, PIO2_LO, t);
    const dfl x = df_from_double(t);
    const dfl x2 = df_mul(x, x);
    dfl ps{C.sh[8], C.sl[8]};
#pragma unroll
    for (int k = 7; k >= 0; --k) ps = df_add(df_mul(ps, x2), dfl{C.sh[k], C.sl[k]});
    ps = df_mul(ps, x);
    dfl pc{C.ch[9], C.cl[9]};
#pragma unroll
    for (int k = 8; k >= 0; --k) pc = df_add(df_mul(pc, x2), dfl{C.ch[k], C.cl[k]});
    const int q = ((int)n) & 3;
    if (q == 0) { s = ps; c = pc; }
    else if (q == 1) { s = pc; c = df_neg(ps); }
    else if (q == 2) { s = df_neg(ps); c = df_neg(pc); }
    else { s = df_neg(pc); c = ps; }
}

}  // namespace ia
