// Double-float ("two-float") arithmetic: a value is an unevaluated sum
// hi + lo of two FP32 numbers, ~48-bit significand.  Used by the mixed path
// to run FP64-accuracy arithmetic on GB300's FP32 pipe (~64x its FP64 rate).
//
// Building blocks are the error-free transformations: TwoSum (Knuth),
// FastTwoSum (Dekker), TwoProd via fmaf; products and sums follow Dekker
// (1971) and Hida, Li & Bailey (2001).  sin/cos: df_sincos_tab (below) for
// double-float arguments, table plus short series, FP32 operations only; and
// df_sincos for FP64 arguments, Cody-Waite reduction by pi/2 (pi/2 held as two
// doubles) then the Taylor series on [-pi/4, pi/4] by Horner in double-float
// with coefficients (-1)^k / n! (exact rationals rounded to double, split).
#pragma once
#include <cuda_runtime.h>
#include <math.h>

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

// ---- table-driven sin/cos of a double-float argument (no FP64 operations)
//
// theta = N pi/128 + u with N = rint(theta 128/pi) and |u| <= ~pi/256;
// sin/cos(N pi/128) come from a 256-entry table (N mod 256) held in shared
// memory as (sin hi, sin lo, cos hi, cos lo), computed once per mesh on the
// host in extended precision and copied in by each CTA; sin u and
// cos u by their Taylor series to u^7 and u^8 (terms below 1e-17 dropped);
// then the angle-sum formulas.  pi/128 is carried as p0 + p1 + p2 + p3 with
// p0..p2 of 12 significant bits, so N p_i is exact for |N| < 4096 and the
// reduction is exact up to the last part (Cody & Waite 1980).  Larger
// arguments take the FP64-reduced series above.
struct DfTrigRed {
    float p[4];            // pi/128 split
    float s3h, s3l;        // -1/6
    float c2h, c2l;        // 1/24
};

__host__ inline float df_round_bits(double x, int bits)
{
    if (x == 0.0) return 0.0f;
    int e;
    frexp(x, &e);                                   // x = m 2^e, 0.5 <= |m| < 1
    const double scale = ldexp(1.0, bits - e);
    return (float)(nearbyint(x * scale) / scale);
}

__host__ inline DfTrigRed df_trig_reduction_constants()
{
    // pi/2 as a double-double (hi exact to 53 bits, lo the next 53), / 64
    const double hi = 1.5707963267948966 / 64.0, lo = 6.123233995736766e-17 / 64.0;
    DfTrigRed r;
    const float p0 = df_round_bits(hi, 12);
    const double r1 = hi - (double)p0;
    const float p1 = df_round_bits(r1, 12);
    const double r2 = r1 - (double)p1;
    const float p2 = df_round_bits(r2, 12);
    const double r3 = (r2 - (double)p2) + lo;
    r.p[0] = p0;
    r.p[1] = p1;
    r.p[2] = p2;
    r.p[3] = (float)r3;
    const double s3 = -1.0 / 6.0, c2 = 1.0 / 24.0;
    r.s3h = (float)s3;
    r.s3l = (float)(s3 - (double)r.s3h);
    r.c2h = (float)c2;
    r.c2l = (float)(c2 - (double)r.c2h);
    return r;
}

__device__ __forceinline__ dfl df_add_f(dfl a, float b)
{
    dfl s = two_sum(a.hi, b);
    s.lo += a.lo;
    return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ void df_sincos_tab(dfl theta, const float4 *__restrict__ tab, const DfTrigRed &P,
                                              const DfTrigCoef &C, dfl &s, dfl &c)
{
    const float N = rintf(theta.hi * 40.74366543152521f);     // 128 / pi
    if (!(fabsf(N) < 4096.0f)) {                               // outside the exact reduction range
        df_sincos(df_to_double(theta), C, s, c);
        return;
    }
    // u = theta - N (p0 + p1 + p2 + p3); theta.hi - N p0 is exact
    dfl u = two_sum(fmaf(-N, P.p[0], theta.hi), theta.lo);
    u = df_add_f(u, -N * P.p[1]);
    u = df_add_f(u, -N * P.p[2]);
    u = df_add_f(u, -N * P.p[3]);
    const dfl u2 = df_mul(u, u);
    // sin u = u + u u2 (-1/6 + u2/120 - u2^2/5040)
    const float ts = u2.hi * fmaf(u2.hi, -1.0f / 5040.0f, 1.0f / 120.0f);
    const dfl su = df_add(u, df_mul(u, df_mul(u2, df_add_f(dfl{P.s3h, P.s3l}, ts))));
    // cos u = 1 + u2 (-1/2 + u2 (1/24 - u2/720 + u2^2/40320))
    const float tc = u2.hi * fmaf(u2.hi, 1.0f / 40320.0f, -1.0f / 720.0f);
    const dfl cu = df_add_f(df_mul(u2, df_add_f(df_mul(u2, df_add_f(dfl{P.c2h, P.c2l}, tc)), -0.5f)), 1.0f);
    const float4 t = tab[((int)N) & 255];
    const dfl sj{t.x, t.y}, cj{t.z, t.w};
    s = df_add(df_mul(sj, cu), df_mul(cj, su));
    c = df_sub(df_mul(cj, cu), df_mul(sj, su));
}

}  // namespace ia
