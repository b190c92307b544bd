// Fused filter-factor / GCV / back-projection kernel, FP64.
//
// One CTA per (frequency, right-hand side):
//   beta = U^H b                                    (tsvd.cuh:151, gcvG.m:25)
//   delta0 = ||b||^2 - ||beta||^2 if m > p          (gcvG.m:26, :32-35)
//   lambda: GCV grid of gcv_points values           (gcvG.m:28-42)
//           standard  -- zero of dG/dlog(lambda) on the bracket around the
//                        grid minimum, 64 bisection steps in log(lambda)
//           reference -- gcvG.m's own filters (:38, :47) and Brent's bounded
//                        minimiser with fminbnd's tolerances (:51)
//   x = V (phi .* beta): Tikhonov phi = s/(s^2+lambda^2) (tikhonovG.m:30) or
//                        TSVD phi = 1/s on the first k  (tsvdG.m:21-23, betak
//                        tsvd.cuh:1-8)
// Sums over the p singular values are warp-shuffle reductions in a fixed
// order; the result does not depend on launch order.
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

constexpr int REG_THREADS = 256;
constexpr int GCV_BISECT_ITERS = 64;

struct GcvData {
    const double *s;
    const double *b2;
    int p;
    double delta0, dof;
};

// standard Tikhonov GCV: G = (sum f^2 b2 + delta0) / (dof + sum f)^2
__device__ double gcv_value(const GcvData &d, double lam, int mode, bool grid_filter, int lane)
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

// sign carrier of dG/dt (t = log lambda): N' D - 2 N D'
__device__ double gcv_slope(const GcvData &d, double t, int lane)
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

__device__ double gcv_bisect(const GcvData &d, double lo, double hi, int lane)
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

// Brent's bounded minimiser (golden section + parabolic interpolation), with
// MATLAB fminbnd's tolerances tol1 = sqrt(eps)|x| + tolx/3, tolx = 1e-4.
// Every lane of the warp runs the same control flow.
__device__ double fminbnd_dev(const GcvData &d, double ax, double bx, int lane)
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

__global__ void __launch_bounds__(REG_THREADS) regularize_kernel(int m, int n, int p, const double2 *U,
                                                                   const double *S, const double2 *V, int nrhs,
                                                                   const double2 *B, ia_config cfg, double2 *X,
                                                                   double *LAM)
{
    extern __shared__ double sm[];
    double *s = sm;                 // p
    double *b2 = s + p;             // p
    double2 *z = reinterpret_cast<double2 *>(b2 + p);   // p  (beta, then phi*beta)
    double *gval = reinterpret_cast<double *>(z + p);   // gcv_points
    __shared__ double red[REG_THREADS / 32];
    __shared__ double s_lam;
    __shared__ int s_jmin;

    const int f = blockIdx.x, r = blockIdx.y;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    U += (size_t)f * m * p;
    V += (size_t)f * n * p;
    S += (size_t)f * p;
    const double2 *b = B + ((size_t)f * nrhs + r) * m;
    double2 *x = X + ((size_t)f * nrhs + r) * n;

    for (int j = threadIdx.x; j < p; j += blockDim.x) s[j] = S[j];
    // beta_j = U_j^H b  (warp per column)
    for (int j = wid; j < p; j += nw) {
        double2 acc = make_double2(0.0, 0.0);
        for (int i = lane; i < m; i += 32) zcfma(acc, U[i + (size_t)j * m], b[i]);
        acc = warp_sum2(acc);
        if (lane == 0) {
            z[j] = acc;
            b2[j] = zabs2(acc);
        }
    }
    // ||b||^2
    double nb = 0.0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) nb += zabs2(b[i]);
    nb = warp_sum(nb);
    if (lane == 0) red[wid] = nb;
    __syncthreads();

    double lam = 0.0;
    const int method = cfg.method;
    if (method == IA_METHOD_TIKHONOV_GCV) {
        if (threadIdx.x == 0) {
            double tb = 0.0, tbeta = 0.0;
            for (int w = 0; w < nw; ++w) tb += red[w];
            for (int j = 0; j < p; ++j) tbeta += b2[j];
            double d0 = tb - tbeta;
            red[0] = (m > p && d0 > 0.0) ? d0 : 0.0;
        }
        __syncthreads();
        GcvData d{s, b2, p, red[0], (double)(m - p)};
        const int np = cfg.gcv_points;
        const double s1 = s[0];
        if (!(s1 > 0.0)) {
            lam = 0.0;
        } else {
            // grid, descending
            double rpm = 0.0, ratio = 0.0, lhi = 0.0, llo = 0.0;
            const bool fixed = (cfg.gcv_lo > 0.0 && cfg.gcv_hi > 0.0);
            if (fixed) {
                lhi = log(cfg.gcv_hi);
                llo = log(cfg.gcv_lo);
            } else {
                rpm = fmax(s[p - 1], s1 * 16.0 * 2.220446049250313e-16);
                ratio = pow(s1 / rpm, 1.0 / (np - 1));
            }
            for (int t = wid; t < np; t += nw) {
                double lt = fixed ? exp(lhi + ((double)t / (np - 1)) * (llo - lhi)) : pow(ratio, (double)(np - 1 - t)) * rpm;
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
                double lo = fixed ? exp(lhi + ((double)jl / (np - 1)) * (llo - lhi)) : pow(ratio, (double)(np - 1 - jl)) * rpm;
                double hi = fixed ? exp(lhi + ((double)jh / (np - 1)) * (llo - lhi)) : pow(ratio, (double)(np - 1 - jh)) * rpm;
                double res = (cfg.gcv_mode == IA_GCV_REFERENCE) ? fminbnd_dev(d, lo, hi, lane) : gcv_bisect(d, lo, hi, lane);
                if (lane == 0) s_lam = res;
            }
            __syncthreads();
            lam = s_lam;
        }
    } else if (method == IA_METHOD_TIKHONOV_FIXED) {
        lam = cfg.lambda_fixed;
    }
    // phi * beta
    const double l2 = lam * lam;
    for (int j = threadIdx.x; j < p; j += blockDim.x) {
        double phi;
        if (method == IA_METHOD_TSVD) phi = (j < cfg.tsvd_k) ? 1.0 / s[j] : 0.0;
        else phi = (s[j] > 0.0 || l2 > 0.0) ? s[j] / (s[j] * s[j] + l2) : 0.0;
        z[j] = zscale(z[j], phi);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double2 acc = make_double2(0.0, 0.0);
        for (int j = 0; j < p; ++j) zfma(acc, V[i + (size_t)j * n], z[j]);
        x[i] = acc;
    }
    if (LAM && threadIdx.x == 0) LAM[(size_t)f * nrhs + r] = (method == IA_METHOD_TSVD) ? 0.0 : lam;
}

int regularize_batched(ia_context *ctx, int m, int n, int p, int batch, const double2 *U, const double *s,
                       const double2 *V, int nrhs, const double2 *b, const ia_config *cfg, double2 *x,
                       double *lambda)
{
    if (cfg->method == IA_METHOD_TSVD && (cfg->tsvd_k < 1 || cfg->tsvd_k > p)) return IA_ERR_ARG;
    if (cfg->method == IA_METHOD_TIKHONOV_GCV && cfg->gcv_points < 2) return IA_ERR_ARG;
    size_t smem = sizeof(double) * (size_t)p * 2 + sizeof(double2) * (size_t)p + sizeof(double) * (size_t)cfg->gcv_points;
    if (smem > 200 * 1024) return IA_ERR_TOO_LARGE;
    if (smem > 48 * 1024) IA_CUDA_TRY(cudaFuncSetAttribute(regularize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 g(batch, nrhs);
    regularize_kernel<<<g, REG_THREADS, smem, ctx->stream>>>(m, n, p, U, s, V, nrhs, b, *cfg, x, lambda);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

}  // namespace ia
