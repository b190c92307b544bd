// GCV lambda selection, FP64, shared by the regularisation kernels.
//
//   grid:       gcv_points values, descending -- regtools' geometric grid from
//               s_1 down to max(s_p, 16 eps s_1) (gcvG.m:28-30) or a fixed
//               log-spaced [lo, hi]
//   standard:   G = (sum f^2 |beta|^2 + delta0) / ((m-p) + sum f)^2,
//               f = lambda^2/(s^2+lambda^2); lambda* = zero of dG/dlog(lambda)
//               on the bracket around the grid minimum, by the Illinois
//               method, to a bracket below 1e-12 in log(lambda)
//   reference:  gcvG.m as written -- grid filter lambda/(s+lambda) (:38),
//               objective filter lambda^2/(s+lambda^2) (:47), Brent's bounded
//               minimiser with fminbnd's tolerances (:51)
// All sums over the p singular values are warp reductions in a fixed order.
#pragma once
#include "ia_common.cuh"

namespace ia {

// iteration cap of the root finder on the slope of G (it stops on width first)
constexpr int GCV_ROOT_MAX_ITERS = 64;

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

// The root of the slope in t = log lambda on the grid bracket, by the Illinois
// variant of regula falsi (Dowell & Jarratt 1971): secant steps that keep the
// bracket, the retained end's value halved when the same end moves twice, so
// both ends converge superlinearly.  Stops when the bracket is below 1e-12 in
// t (lambda to ~1e-12 relative) or the slope is exactly 0; a midpoint step
// replaces a secant point that falls outside the open bracket.  Each slope
// evaluation is ~200 FP64 warp instructions on GB300's slow FP64 pipe, so this
// takes ~10 evaluations where bisection to the same width took 40.
__device__ __forceinline__ double gcv_root(const GcvData &d, double lo, double hi, int lane)
{
    if (lo == hi) return lo;
    double a = log(lo), b = log(hi);
    double fa = gcv_slope(d, a, lane), fb;
    if (fa >= 0.0) return lo;
    fb = gcv_slope(d, b, lane);
    if (fb <= 0.0) return hi;
    int side = 0;
    for (int it = 0; it < GCV_ROOT_MAX_ITERS && b - a > 1e-12; ++it) {
        double c = b - fb * (b - a) / (fb - fa);
        if (!(c > a && c < b)) c = 0.5 * (a + b);
        const double fc = gcv_slope(d, c, lane);
        if (fc == 0.0) return exp(c);
        if (fc < 0.0) {
            a = c;
            fa = fc;
            if (side < 0) fb *= 0.5;
            side = -1;
        } else {
            b = c;
            fb = fc;
            if (side > 0) fa *= 0.5;
            side = 1;
        }
    }
    return exp(0.5 * (a + b));
}

// Brent's bounded minimiser of obj(x) (a warp-uniform value), fminbnd
// tolerances tol1 = sqrt(eps)|x| + tolx/3, tolx = 1e-4; every lane runs the
// same control flow.
template <class Obj>
__device__ __forceinline__ double brent_min(const Obj &obj, double ax, double bx)
{
    const double seps = 1.4901161193847656e-08, tolx = 1e-4;
    const double cg = 0.5 * (3.0 - sqrt(5.0));
    double a = ax, b = bx;
    double v = a + cg * (b - a), w = v, xf = v, dd = 0.0, e = 0.0;
    double fx = obj(xf);
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
        double fu = obj(x);
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

__device__ __forceinline__ double fminbnd_dev(const GcvData &d, double ax, double bx, int lane)
{
    return brent_min([&](double x) { return gcv_value(d, x, IA_GCV_REFERENCE, false, lane); }, ax, bx);
}

// Filter factor f(lambda) and, for the L-curve, its use as written in
// lcfunG.m: Tikhonov s^2/(s^2+l^2), damped SVD s/(s+l) (dsvdG.m).
__device__ __forceinline__ double filt(double s, double lam, bool damped)
{
    return damped ? s / (s + lam) : (s * s) / (s * s + lam * lam);
}

// Negative curvature of the L-curve (log rho, log eta) at lambda, restating
// lcfunG.m:12-49: xi = beta/s (0 where s = 0), rho^2 = sum (1-f)^2 |beta|^2
// (+ the least-squares residual rho_ls2), eta^2 = sum f^2 |xi|^2, and the
// derivative sums phi, psi, dphi, dpsi with f1 = -2 f (1-f)/l,
// f2 = -f1 (3 - 4f)/l (lcfunG.m uses these for both filters).
__device__ __forceinline__ double lcurve_value(const double *s, const double *b2, int p, double rho_ls2, double lam,
                                               bool damped, int lane)
{
    double eta2 = 0, rho2 = 0, phi = 0, psi = 0, dphi = 0, dpsi = 0;
    for (int j = lane; j < p; j += 32) {
        const double sj = s[j], bb = b2[j];
        const double xx = sj > 0.0 ? bb / (sj * sj) : 0.0;
        const double f = filt(sj, lam, damped), cf = 1.0 - f;
        const double f1 = -2.0 * f * cf / lam, f2 = -f1 * (3.0 - 4.0 * f) / lam;
        eta2 = fma(f * f, xx, eta2);
        rho2 = fma(cf * cf, bb, rho2);
        phi = fma(f * f1, xx, phi);
        psi = fma(cf * f1, bb, psi);
        dphi = fma(f1 * f1 + f * f2, xx, dphi);
        dpsi = fma(-f1 * f1 + cf * f2, bb, dpsi);
    }
    const double eta = sqrt(warp_sum(eta2)), rho = sqrt(warp_sum(rho2) + rho_ls2);
    phi = warp_sum(phi);
    psi = warp_sum(psi);
    dphi = warp_sum(dphi);
    dpsi = warp_sum(dpsi);
    const double deta = phi / eta, drho = -psi / rho;
    const double ddeta = dphi / eta - deta * (deta / eta), ddrho = -dpsi / rho - drho * (drho / rho);
    const double dle = deta / eta, dlr = drho / rho;
    const double ddle = ddeta / eta - dle * dle, ddlr = ddrho / rho - dlr * dlr;
    return -(dlr * ddle - ddlr * dle) / pow(dlr * dlr + dle * dle, 1.5);
}

// Quasi-optimality function Q(lambda) = || (1-f) f xi || (quasioptG.m:31-37)
__device__ __forceinline__ double quasiopt_value(const double *s, const double *b2, int p, double lam, bool damped,
                                                 int lane)
{
    double q = 0.0;
    for (int j = lane; j < p; j += 32) {
        const double sj = s[j];
        const double xx = sj > 0.0 ? b2[j] / (sj * sj) : 0.0;
        const double f = filt(sj, lam, damped), g = (1.0 - f) * f;
        q = fma(g * g, xx, q);
    }
    return sqrt(warp_sum(q));
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
    // grid values first, one pow per thread (a warp-uniform pow per grid point
    // would run on all 32 lanes of the slow FP64 pipe); each slot then holds
    // its G value, written by the one warp that read its lambda
    for (int t = threadIdx.x; t < np; t += blockDim.x) gval[t] = gcv_grid_point(fixed, lhi, llo, ratio, rpm, np, t);
    __syncthreads();
    for (int t = wid; t < np; t += nw) {
        const double lt = gval[t];
        const double g = gcv_value(d, lt, cfg.gcv_mode, true, lane);
        __syncwarp();
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
        double res = (cfg.gcv_mode == IA_GCV_REFERENCE) ? fminbnd_dev(d, lo, hi, lane) : gcv_root(d, lo, hi, lane);
        if (lane == 0) s_lam = res;
    }
    __syncthreads();
    return s_lam;
}

// Grid minimum, then Brent (fminbnd tolerances) on the bracket of the grid
// points either side of it -- the scheme of l_curveG.m:42-53 and
// quasioptG.m:24-41 -- over a descending geometric grid of np values from s1
// down to rpm.  obj is warp-cooperative.  Returns lambda in every thread.
template <class Obj>
static __device__ double grid_brent(const Obj &obj, double s1, double rpm, int np, double *gval)
{
    __shared__ double s_lam;
    __shared__ int s_jmin;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const double ratio = pow(s1 / rpm, 1.0 / (np - 1));
    for (int t = threadIdx.x; t < np; t += blockDim.x) gval[t] = pow(ratio, (double)(np - 1 - t)) * rpm;
    __syncthreads();
    for (int t = wid; t < np; t += nw) {
        const double g = obj(gval[t]);
        __syncwarp();
        if (lane == 0) gval[t] = g;
    }
    __syncthreads();
    if (threadIdx.x == 0) {   // first minimum; NaN never wins (MATLAB min)
        int jm = 0;
        double gm = gval[0];
        for (int t = 1; t < np; ++t)
            if (gval[t] < gm || !(gm == gm)) { gm = gval[t]; jm = t; }
        s_jmin = jm;
    }
    __syncthreads();
    if (wid == 0) {
        const int jm = s_jmin;
        const int jl = jm + 1 < np ? jm + 1 : np - 1, jh = jm - 1 > 0 ? jm - 1 : 0;
        const double lo = pow(ratio, (double)(np - 1 - jl)) * rpm, hi = pow(ratio, (double)(np - 1 - jh)) * rpm;
        const double res = brent_min(obj, lo, hi);
        if (lane == 0) s_lam = res;
    }
    __syncthreads();
    return s_lam;
}

// lambda for cfg.method: GCV (select_lambda), L-curve corner (l_curveG.m;
// grid down to max(s_p, 16 eps s_1), least-squares residual delta0 when
// m > p), quasi-optimality (quasioptG.m; grid down to s_p), a fixed value, or
// 0 for TSVD.
static __device__ double choose_lambda(const double *s, const double *b2, int p, double delta0, double dof,
                                       const ia_config &cfg, double *gval)
{
    const int mth = cfg.method;
    if (mth == IA_METHOD_TIKHONOV_GCV) return select_lambda(s, b2, p, delta0, dof, cfg, gval);
    if (mth == IA_METHOD_TIKHONOV_FIXED || mth == IA_METHOD_DSVD_FIXED) return cfg.lambda_fixed;
    if (mth == IA_METHOD_TSVD) return 0.0;
    const double s1 = s[0];
    if (!(s1 > 0.0)) return 0.0;
    const bool damped = mth == IA_METHOD_DSVD_LCURVE || mth == IA_METHOD_DSVD_QUASIOPT;
    const int lane = threadIdx.x & 31;
    const double floor = s1 * 16.0 * 2.220446049250313e-16;
    if (mth == IA_METHOD_TIKHONOV_LCURVE || mth == IA_METHOD_DSVD_LCURVE) {
        auto obj = [&](double lam) { return lcurve_value(s, b2, p, delta0, lam, damped, lane); };
        return grid_brent(obj, s1, fmax(s[p - 1], floor), cfg.gcv_points, gval);
    }
    auto obj = [&](double lam) { return quasiopt_value(s, b2, p, lam, damped, lane); };
    return grid_brent(obj, s1, s[p - 1] > 0.0 ? s[p - 1] : floor, cfg.gcv_points, gval);
}

// host-side validation of the regularisation settings for p singular values
inline int check_method(const ia_config &cfg, int p)
{
    if (cfg.method < IA_METHOD_TIKHONOV_GCV || cfg.method > IA_METHOD_DSVD_QUASIOPT) return IA_ERR_ARG;
    if (cfg.method == IA_METHOD_TSVD && (cfg.tsvd_k < 1 || cfg.tsvd_k > p)) return IA_ERR_ARG;
    const bool grid = cfg.method == IA_METHOD_TIKHONOV_GCV || cfg.method == IA_METHOD_TIKHONOV_LCURVE ||
                      cfg.method == IA_METHOD_TIKHONOV_QUASIOPT || cfg.method == IA_METHOD_DSVD_LCURVE ||
                      cfg.method == IA_METHOD_DSVD_QUASIOPT;
    if (grid && cfg.gcv_points < 2) return IA_ERR_ARG;
    if ((cfg.method == IA_METHOD_TIKHONOV_FIXED || cfg.method == IA_METHOD_DSVD_FIXED) && !(cfg.lambda_fixed >= 0.0))
        return IA_ERR_ARG;
    return IA_OK;
}

// filter factor over s (x = V diag(phi) beta) for the chosen method
__device__ __forceinline__ double filter_phi(int method, int j, double sj, double lam, int tsvd_k)
{
    if (method == IA_METHOD_TSVD) return (j < tsvd_k) ? 1.0 / sj : 0.0;
    if (method == IA_METHOD_DSVD_FIXED || method == IA_METHOD_DSVD_LCURVE || method == IA_METHOD_DSVD_QUASIOPT)
        return (sj + lam) > 0.0 ? 1.0 / (sj + lam) : 0.0;       // damped SVD, dsvdG.m:26
    const double l2 = lam * lam;
    return (sj > 0.0 || l2 > 0.0) ? sj / (sj * sj + l2) : 0.0;
}

}  // namespace ia
