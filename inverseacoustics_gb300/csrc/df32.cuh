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
// theta = N pi/512 + u with N = rint(theta 512/pi) and |u| <= ~pi/1024;
// sin/cos(N pi/512) come from a 1024-entry table (N mod 1024) held in shared
// memory as (sin hi, sin lo, cos hi, cos lo), computed once per mesh on the
// host in extended precision and copied in by each CTA.  With |u| <= 3.1e-3
// the series need little double-float work: sin u = u + u^3 (-1/6 + u^2/120)
// with the correction (< 5e-9) in FP32 plus its first-order term in u's low
// word, and cos u = 1 - u^2/2 + u^4/24 with u^2 in double-float and u^4/24
// (< 4e-12) in FP32; dropped terms are below 2e-18 and the FP32 parts add
// ~1e-15 absolute, the level of a double-float result near 1.  Then the
// angle-sum formulas.  pi/512 is carried as p0 + ... + p4 with p0..p3 of 10
// significant bits, so N p_i is exact for |N| < 2^14 (theta < 100) and the
// reduction is exact up to the last part (Cody & Waite 1980).  Larger
// arguments take the FP64-reduced series above.
constexpr int DF_TRIG_TABLE = 1024;

struct DfTrigRed {
    float p[5];            // pi/512 split
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
    // pi/2 as a double-double (hi exact to 53 bits, lo the next 53), / 256
    const double hi = 1.5707963267948966 / 256.0, lo = 6.123233995736766e-17 / 256.0;
    DfTrigRed r;
    double rest = hi;
    for (int i = 0; i < 4; ++i) {
        r.p[i] = df_round_bits(rest, 10);
        rest -= (double)r.p[i];
    }
    r.p[4] = (float)(rest + lo);
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
    const float N = rintf(theta.hi * 162.97466172610082f);    // 512 / pi
    if (!(fabsf(N) < 16384.0f)) {                              // outside the exact reduction range
        df_sincos(df_to_double(theta), C, s, c);
        return;
    }
    // u = theta - N (p0 + ... + p4); theta.hi - N p0 is exact
    dfl u = two_sum(fmaf(-N, P.p[0], theta.hi), theta.lo);
    u = df_add_f(u, -N * P.p[1]);
    u = df_add_f(u, -N * P.p[2]);
    u = df_add_f(u, -N * P.p[3]);
    u = df_add_f(u, -N * P.p[4]);
    const float uh = u.hi, u2h = uh * uh;
    // sin u = u + u^3 (-1/6 + u^2/120); d(-u^3/6)/du = -u^2/2 carries u.lo
    const float ds = fmaf(uh * u2h, fmaf(u2h, 1.0f / 120.0f, -1.0f / 6.0f), -0.5f * u2h * u.lo);
    const dfl su = df_add_f(u, ds);
    // cos u = 1 - u^2/2 + u^4/24
    const dfl u2 = df_mul(u, u);
    const dfl w = df_add_f(dfl{-0.5f * u2.hi, -0.5f * u2.lo}, u2h * u2h * (1.0f / 24.0f));
    const dfl cu = df_add_f(w, 1.0f);
    const float4 t = tab[((int)N) & (DF_TRIG_TABLE - 1)];
    const dfl sj{t.x, t.y}, cj{t.z, t.w};
    s = df_add(df_mul(sj, cu), df_mul(cj, su));
    c = df_sub(df_mul(cj, cu), df_mul(sj, su));
}

}  // namespace ia
