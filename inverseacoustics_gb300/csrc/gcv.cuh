// GCV lambda selection, FP64, shared by the regularisation kernels.
//
//   grid:       gcv_points values, descending -- regtools' geometric grid from
//               s_1 down to max(s_p, 16 eps s_1) (gcvG.m:28-30) or a fixed
//               log-spaced [lo, hi]
//   standard:   G = (sum f^2 |beta|^2 + delta0) / ((m-p) + sum f)^2,
//               f = lambda^2/(s^2+lambda^2); lambda* = zero of dG/dlog(lambda)
//               on the bracket around the grid minimum, 64 bisection steps
//   reference:  gcvG.m as written -- grid filter lambda/(s+lambda) (:38),
//               objective filter lambda^2/(s+lambda^2) (:47), Brent's bounded
//               minimiser with fminbnd's tolerances (:51)
// All sums over the p singular values are warp reductions in a fixed order.
#pragma once
#include "ia_common.cuh"

namespace ia {

constexpr int GCV_BISECT_ITERS = 64;

struct GcvData {
    const double *s;
    const double *b2;
    int p;
    double delta0, dof;
};

__device__ __forceinline__ double gcv_value(const GcvData &d, double lam, int mode, bool grid_filter, int lane)
{
    double num = 0.0, den = 0.0;
    const double l2 = lam * lam;
    for (int j = lane; j < d.p; j += 32) {
        double sj = d.s[j], f;
        if (mode == IA_GCV_REFERENCE) f = grid_filter ? lam / (sj + lam) : l2 / (sj + l2);
        else f = l2 / (sj * sj + l2);
        num = fma(f * f, d.b2[j], num);
        den += f;
    }
    num = warp_sum(num) + d.delta0;
    den = warp_sum(den) + d.dof;
    return num / (den * den);
}

// sign carrier of dG/dt, t = log lambda: N' D - 2 N D'
__device__ __forceinline__ double gcv_slope(const GcvData &d, double t, int lane)
{
    const double lam = exp(t), l2 = lam * lam;
    double num = 0.0, den = 0.0, dnum = 0.0, dden = 0.0;
    for (int j = lane; j < d.p; j += 32) {
        double sj = d.s[j];
        double f = l2 / (sj * sj + l2);
        double g = f * (1.0 - f);
        num = fma(f * f, d.b2[j], num);
        den += f;
        dnum = fma(f * g, d.b2[j], dnum);
        dden += g;
    }
    num = warp_sum(num) + d.delta0;
    den = warp_sum(den) + d.dof;
    dnum = 4.0 * warp_sum(dnum);
    dden = 2.0 * warp_sum(dden);
    return dnum * den - 2.0 * num * dden;
}

__device__ __forceinline__ double gcv_bisect(const GcvData &d, double lo, double hi, int lane)
{
    if (lo == hi) return lo;
    double a = log(lo), b = log(hi);
    if (gcv_slope(d, a, lane) >= 0.0) return lo;
    if (gcv_slope(d, b, lane) <= 0.0) return hi;
    for (int it = 0; it < GCV_BISECT_ITERS; ++it) {
        double mid = 0.5 * (a + b);
        if (gcv_slope(d, mid, lane) < 0.0) a = mid;
        else b = mid;
    }
    return exp(0.5 * (a + b));
}

// Brent's bounded minimiser, fminbnd tolerances tol1 = sqrt(eps)|x| + tolx/3,
// tolx = 1e-4; every lane runs the same control flow.
__device__ __forceinline__ double fminbnd_dev(const GcvData &d, double ax, double bx, int lane)
{
    const double seps = 1.4901161193847656e-08, tolx = 1e-4;
    const double cg = 0.5 * (3.0 - sqrt(5.0));
    double a = ax, b = bx;
    double v = a + cg * (b - a), w = v, xf = v, dd = 0.0, e = 0.0;
    double fx = gcv_value(d, xf, IA_GCV_REFERENCE, false, lane);
    double fv = fx, fw = fx;
    double xm = 0.5 * (a + b);
    double tol1 = seps * fabs(xf) + tolx / 3.0, tol2 = 2.0 * tol1;
    for (int it = 0; it < 500 && fabs(xf - xm) > (tol2 - 0.5 * (b - a)); ++it) {
        bool golden = true;
        if (fabs(e) > tol1) {
            golden = false;
            double r = (xf - w) * (fx - fv);
            double q = (xf - v) * (fx - fw);
            double p = (xf - v) * q - (xf - w) * r;
            q = 2.0 * (q - r);
            if (q > 0.0) p = -p;
            q = fabs(q);
            r = e;
            e = dd;
            if (fabs(p) < fabs(0.5 * q * r) && p > q * (a - xf) && p < q * (b - xf)) {
                dd = p / q;
                double x = xf + dd;
                if ((x - a) < tol2 || (b - x) < tol2) dd = (xm - xf) >= 0.0 ? tol1 : -tol1;
            } else {
                golden = true;
            }
        }
        if (golden) {
            e = (xf >= xm) ? (a - xf) : (b - xf);
            dd = cg * e;
        }
        double x = xf + (dd >= 0.0 ? 1.0 : -1.0) * fmax(fabs(dd), tol1);
        double fu = gcv_value(d, x, IA_GCV_REFERENCE, false, lane);
        if (fu <= fx) {
            if (x >= xf) a = xf;
            else b = xf;
            v = w; fv = fw;
            w = xf; fw = fx;
            xf = x; fx = fu;
        } else {
            if (x < xf) a = x;
            else b = x;
            if (fu <= fw || w == xf) {
                v = w; fv = fw;
                w = x; fw = fu;
            } else if (fu <= fv || v == xf || v == w) {
                v = x; fv = fu;
            }
        }
        xm = 0.5 * (a + b);
        tol1 = seps * fabs(xf) + tolx / 3.0;
        tol2 = 2.0 * tol1;
    }
    return xf;
}

__device__ __forceinline__ double gcv_grid_point(bool fixed, double lhi, double llo, double ratio, double rpm, int np,
                                                 int t)
{
    return fixed ? exp(lhi + ((double)t / (np - 1)) * (llo - lhi)) : pow(ratio, (double)(np - 1 - t)) * rpm;
}

// Whole-CTA lambda selection.  s (descending), b2 = |beta|^2 in shared
// memory; gval: shared scratch of cfg.gcv_points doubles.  Returns lambda
// (the same value in every thread).
static __device__ double select_lambda(const double *s, const double *b2, int p, double delta0, double dof,
                                       const ia_config &cfg, double *gval)
{
    __shared__ double s_lam;
    __shared__ int s_jmin;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    GcvData d{s, b2, p, delta0, dof};
    const int np = cfg.gcv_points;
    const double s1 = s[0];
    if (!(s1 > 0.0)) return 0.0;
    const bool fixed = (cfg.gcv_lo > 0.0 && cfg.gcv_hi > 0.0);
    double rpm = 0.0, ratio = 0.0, lhi = 0.0, llo = 0.0;
    if (fixed) {
        lhi = log(cfg.gcv_hi);
        llo = log(cfg.gcv_lo);
    } else {
        rpm = fmax(s[p - 1], s1 * 16.0 * 2.220446049250313e-16);
        ratio = pow(s1 / rpm, 1.0 / (np - 1));
    }
    for (int t = wid; t < np; t += nw) {
        double lt = gcv_grid_point(fixed, lhi, llo, ratio, rpm, np, t);
        double g = gcv_value(d, lt, cfg.gcv_mode, true, lane);
        if (lane == 0) gval[t] = g;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int jm = 0;
        double gm = gval[0];
        for (int t = 1; t < np; ++t)
            if (gval[t] < gm) { gm = gval[t]; jm = t; }
        s_jmin = jm;
    }
    __syncthreads();
    if (wid == 0) {
        int jm = s_jmin;
        int jl = jm + 1 < np ? jm + 1 : np - 1, jh = jm - 1 > 0 ? jm - 1 : 0;
        double lo = gcv_grid_point(fixed, lhi, llo, ratio, rpm, np, jl);
        double hi = gcv_grid_point(fixed, lhi, llo, ratio, rpm, np, jh);
        double res = (cfg.gcv_mode == IA_GCV_REFERENCE) ? fminbnd_dev(d, lo, hi, lane) : gcv_bisect(d, lo, hi, lane);
        if (lane == 0) s_lam = res;
    }
    __syncthreads();
    return s_lam;
}

// filter factor times beta for the chosen method
__device__ __forceinline__ double filter_phi(int method, int j, double sj, double lam, int tsvd_k)
{
    if (method == IA_METHOD_TSVD) return (j < tsvd_k) ? 1.0 / sj : 0.0;
    const double l2 = lam * lam;
    return (sj > 0.0 || l2 > 0.0) ? sj / (sj * sj + l2) : 0.0;
}

}  // namespace ia
