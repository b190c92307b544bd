// ADMM for L1 / L2 / Lp regularised complex least squares, batched over
// frequencies and right-hand sides: the reference's MATLAB/ADMMG.m:1-90.
//
//   min_c ||A c - b||^2 + lambda R(x)   s.t. c = x
//   c <- (2 A^H A + rho I)^-1 (2 A^H b + rho x - u)      (ADMMG.m:15,39,64)
//   x <- shrink(c + u / rho)                              (:17-18, :41, :66-76)
//   u <- u + gamma rho (c - x)                            (:20, :43, :78)
// with L1 soft thresholding at lambda / rho, the L2 step (rho c + u) /
// (2 lambda_0 + rho), and Lp generalised soft thresholding (threshold tpgst,
// N fixed-point steps) at lambda_p = 2 lambda / rho.  L1 and Lp run the
// continuation lambda = 5 lambda_0 * 0.75^j while lambda > lambda_0 / 10; the
// first iteration with ||c - c_old||, ||c - x||, ||u - u_old|| all <= epsilon
// ends the run (:21-28).
//
// GB300 layout.  The c-update's inverse is formed once per frequency: for
// m <= l (primal) P = (2 A^H A + rho I)^-1 (m x m) and c = P r; for m > l (dual,
// Woodbury) K2 = 2 (rho I + 2 A A^H)^-1 (l x l) and c = (r - A^H K2 A r) / rho.
// One persistent CTA -- or, for the dual form, a thread-block cluster of cs CTAs
// splitting the m columns, with the l-vector A r and the three norms summed
// across the cluster through distributed shared memory -- runs every
// iteration of one (frequency, right-hand side); c, x, u, r stay in shared
// memory and A, A^T, K2 are read from L2.  cs depends on (l, m) only, so a
// problem's result does not depend on the rest of the batch.
#include <cooperative_groups.h>
#include "ia_common.cuh"
#include "ia_internal.h"

namespace cg = cooperative_groups;

namespace ia {

constexpr int ADMM_THREADS = 256;
constexpr int ADMM_WARPS = ADMM_THREADS / 32;

struct AdmmArgs {
    int l, m, nrhs, norm, nm, gst;
    double rho, gamma, eps, p;
    const double2 *A;     // F x (l x m)     dual
    const double2 *AT;    // F x (m x l)     dual
    const double2 *K;     // dual: F x (l x l) K2; primal: F x (m x m) P
    const double2 *aa22;  // F x (m x nrhs)  2 A^H b
    const double *lam0;   // F x nrhs
    const double2 *x0;    // F x (m x nrhs)
    double2 *c;           // F x (m x nrhs)
    int *iters;           // F x nrhs, or null
    int *info;            // F
};

__device__ __forceinline__ double admm_gst_tau(double lam_p, double p)
{
    const double t = 2.0 * lam_p * (1.0 - p);
    return pow(t, 1.0 / (2.0 - p)) + lam_p * p * pow(t, (p - 1.0) / (2.0 - p));
}

// shared-memory floats per CTA: c, x, u, r (mloc each), y partials (2 l),
// y, z (l each), norm partials (2 x 4 doubles + warps x 3 doubles)
static size_t admm_smem_bytes(int l, int mloc, bool dual)
{
    size_t v = 4 * (size_t)mloc + (dual ? 4 * (size_t)l : 0);
    return v * sizeof(double2) + (8 + 3 * ADMM_WARPS + 8) * sizeof(double);
}

template <bool DUAL>
__global__ void __launch_bounds__(ADMM_THREADS) admm_kernel(AdmmArgs a, int cs)
{
    extern __shared__ double2 sm[];
    const int rank = DUAL && cs > 1 ? (int)cg::this_cluster().block_rank() : 0;
    const int pid = blockIdx.x / cs;
    const int f = pid / a.nrhs, rr = pid - f * a.nrhs;
    const int l = a.l, m = a.m;
    const int mloc = (m + cs - 1) / cs, j0 = rank * mloc;
    const int nloc = max(0, min(m, j0 + mloc) - j0);
    double2 *c = sm, *x = c + mloc, *u = x + mloc, *r = u + mloc;
    double2 *ypart = r + mloc;        // 2 x l
    double2 *y = ypart + 2 * l;       // l
    double2 *z = y + l;               // l
    double *red = reinterpret_cast<double *>(DUAL ? z + l : r + mloc);   // 2 x 4
    double *wred = red + 8;                                               // warps x 3
    int *flag = reinterpret_cast<int *>(wred + 3 * ADMM_WARPS);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

    const double2 *A = a.A + (size_t)f * l * m;
    const double2 *AT = a.AT + (size_t)f * l * m;
    const double2 *K = a.K + (size_t)f * (DUAL ? (size_t)l * l : (size_t)m * m);
    const double2 *aa22 = a.aa22 + ((size_t)f * a.nrhs + rr) * m + j0;
    const double2 *x0 = a.x0 + ((size_t)f * a.nrhs + rr) * m + j0;
    const double lam0 = a.lam0[(size_t)f * a.nrhs + rr];
    const double rho = a.rho, inv_rho = 1.0 / rho, gr = a.gamma * a.rho, p = a.p;

    for (int j = tid; j < nloc; j += ADMM_THREADS) {
        const double2 xv = x0[j];
        c[j] = make_double2(0.0, 0.0);
        x[j] = xv;
        u[j] = a.norm == 3 ? xv : make_double2(0.0, 0.0);
    }
    int its = 0, buf = 0;
    bool conv = false;
    const double lam_e = lam0 / 10.0;
    double lam = a.norm == 2 ? lam0 : lam0 * 5.0;
    const double dlr = 2.0 * lam0 + rho;
    while (a.norm == 2 || lam > lam_e) {
        const double lr = lam / rho;
        const double lam_p = 2.0 * lam / rho;
        const double tau = a.norm == 3 ? admm_gst_tau(lam_p, p) : 0.0;
        for (int k = 0; k < a.nm; ++k) {
            __syncthreads();
            for (int j = tid; j < nloc; j += ADMM_THREADS) {
                const double2 xv = x[j], uv = u[j], bv = aa22[j];
                r[j] = make_double2(fma(rho, xv.x, bv.x) - uv.x, fma(rho, xv.y, bv.y) - uv.y);
            }
            __syncthreads();
            if (DUAL) {
                // y (this CTA's part) = A(:, loc) r_loc
                for (int i = wid; i < l; i += ADMM_WARPS) {
                    const double2 *row = AT + (size_t)i * m + j0;
                    double2 acc = make_double2(0.0, 0.0);
                    for (int j = lane; j < nloc; j += 32) zfma(acc, row[j], r[j]);
                    acc = warp_sum2(acc);
                    if (lane == 0) ypart[buf * l + i] = acc;
                }
                if (cs > 1) cg::this_cluster().sync();
                else __syncthreads();
                for (int i = tid; i < l; i += ADMM_THREADS) {
                    double2 s = make_double2(0.0, 0.0);
                    for (int q = 0; q < cs; ++q) {
                        const double2 *yp = cs > 1 ? cg::this_cluster().map_shared_rank(ypart, q) : ypart;
                        s = zadd(s, yp[buf * l + i]);
                    }
                    y[i] = s;
                }
                __syncthreads();
                // z = K2 y (K2 Hermitian: z_i = sum_k conj(K2[k, i]) y_k)
                for (int i = wid; i < l; i += ADMM_WARPS) {
                    const double2 *col = K + (size_t)i * l;
                    double2 acc = make_double2(0.0, 0.0);
                    for (int q = lane; q < l; q += 32) zcfma(acc, col[q], y[q]);
                    acc = warp_sum2(acc);
                    if (lane == 0) z[i] = acc;
                }
                __syncthreads();
            }
            // c_j, then the shrink and dual updates of entry j (lane 0)
            double dc = 0.0, dcx = 0.0, du = 0.0;
            for (int j = wid; j < nloc; j += ADMM_WARPS) {
                double2 acc = make_double2(0.0, 0.0);
                if (DUAL) {
                    const double2 *col = A + (size_t)(j0 + j) * l;
                    for (int i = lane; i < l; i += 32) zcfma(acc, col[i], z[i]);
                } else {
                    const double2 *col = K + (size_t)j * m;     // P Hermitian
                    for (int q = lane; q < m; q += 32) zcfma(acc, col[q], r[q]);
                }
                acc = warp_sum2(acc);
                if (lane == 0) {
                    double2 cn;
                    if (DUAL) cn = make_double2((r[j].x - acc.x) * inv_rho, (r[j].y - acc.y) * inv_rho);
                    else cn = acc;
                    const double2 co = c[j], uo = u[j];
                    dc += zabs2(zsub(cn, co));
                    double2 xn;
                    if (a.norm == 2) {
                        xn = make_double2(fma(rho, cn.x, uo.x) / dlr, fma(rho, cn.y, uo.y) / dlr);
                    } else {
                        const double2 yv = make_double2(fma(uo.x, inv_rho, cn.x), fma(uo.y, inv_rho, cn.y));
                        const double ay = hypot(yv.x, yv.y);
                        if (a.norm == 1) {
                            const double sc = ay > lr ? (ay - lr) / ay : 0.0;
                            xn = zscale(yv, sc);
                        } else if (!(ay <= tau)) {
                            double s = ay;
                            for (int d = 0; d < a.gst; ++d) s = ay - lam_p * p * pow(s, p - 1.0);
                            xn = ay > 0.0 ? zscale(yv, s / ay) : make_double2(0.0, 0.0);
                        } else {
                            xn = make_double2(0.0, 0.0);
                        }
                    }
                    const double2 dx = zsub(cn, xn);
                    dcx += zabs2(dx);
                    const double2 un = make_double2(fma(gr, dx.x, uo.x), fma(gr, dx.y, uo.y));
                    du += zabs2(zsub(un, uo));
                    c[j] = cn;
                    x[j] = xn;
                    u[j] = un;
                }
            }
            if (lane == 0) {
                wred[3 * wid] = dc;
                wred[3 * wid + 1] = dcx;
                wred[3 * wid + 2] = du;
            }
            __syncthreads();
            if (tid == 0) {
                double s0 = 0.0, s1 = 0.0, s2 = 0.0;
                for (int w = 0; w < ADMM_WARPS; ++w) {
                    s0 += wred[3 * w];
                    s1 += wred[3 * w + 1];
                    s2 += wred[3 * w + 2];
                }
                red[4 * buf] = s0;
                red[4 * buf + 1] = s1;
                red[4 * buf + 2] = s2;
            }
            if (DUAL && cs > 1) cg::this_cluster().sync();
            else __syncthreads();
            if (tid == 0) {
                double s0 = 0.0, s1 = 0.0, s2 = 0.0;
                for (int q = 0; q < (DUAL ? cs : 1); ++q) {
                    const double *rp = DUAL && cs > 1 ? cg::this_cluster().map_shared_rank(red, q) : red;
                    s0 += rp[4 * buf];
                    s1 += rp[4 * buf + 1];
                    s2 += rp[4 * buf + 2];
                }
                *flag = sqrt(s0) <= a.eps && sqrt(s1) <= a.eps && sqrt(s2) <= a.eps;
            }
            __syncthreads();
            conv = *flag != 0;
            ++its;
            buf ^= 1;
            if (conv) break;
        }
        if (conv || a.norm == 2) break;
        lam = fmax(0.75 * lam, lam_e);
    }
    __syncthreads();
    double2 *cout = a.c + ((size_t)f * a.nrhs + rr) * m + j0;
    for (int j = tid; j < nloc; j += ADMM_THREADS) cout[j] = c[j];
    if (tid == 0 && rank == 0) {
        if (a.iters) a.iters[(size_t)f * a.nrhs + rr] = its;
        if (!conv && a.info) atomicOr(&a.info[f], IA_INFO_NOCONV);
    }
    // no CTA leaves while others may still read its shared memory
    if (DUAL && cs > 1) cg::this_cluster().sync();
}

// M += s I (n x n per batch entry)
__global__ void admm_diag_kernel(int n, double2 *M, long long sM, double s, double2 *Id, long long sI, double id)
{
    const int f = blockIdx.y;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 *d = M + f * sM + (size_t)i * n + i;
        d->x += s;
        if (Id) {
            double2 *col = Id + f * sI + (size_t)i * n;
            for (int q = 0; q < n; ++q) col[q] = make_double2(q == i ? id : 0.0, 0.0);
        }
    }
}

// y = (R^H)^-1 b: R upper triangular (the first l rows of an m x l QR, leading
// dimension m); warp per (frequency, right-hand side)
__global__ void admm_fwd_kernel(int m, int l, int nrhs, const double2 *Y, const double2 *B, double2 *Yout, int F)
{
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (w >= F * nrhs) return;
    const int f = w / nrhs, rr = w - f * nrhs;
    const double2 *R = Y + (size_t)f * m * l;
    const double2 *b = B + ((size_t)f * nrhs + rr) * l;
    double2 *y = Yout + ((size_t)f * nrhs + rr) * l;
    for (int i = 0; i < l; ++i) {
        const double2 *col = R + (size_t)i * m;
        double2 acc = make_double2(0.0, 0.0);
        for (int k = lane; k < i; k += 32) zcfma(acc, col[k], y[k]);
        acc = warp_sum2(acc);
        if (lane == 0) y[i] = zdiv(zsub(b[i], acc), zconj(col[i]));
        __syncwarp();
    }
}

static int admm_cluster_size(int l, int m)
{
    if (m <= l) return 1;
    int cs = 1;
    while (cs < 8 && (m + 2 * cs - 1) / (2 * cs) >= 128) cs *= 2;
    while (cs < 8 && admm_smem_bytes(l, (m + cs - 1) / cs, true) > 200 * 1024) cs *= 2;
    return cs;
}

size_t admm_ws_bytes(int l, int m, int F, int nrhs)
{
    const size_t L = l, M = m, FF = F, R = nrhs;
    const size_t kd = m <= l ? M * M : L * L;
    return 2 * ws_round(16 * L * M * FF) + 2 * ws_round(16 * kd * FF) + 2 * ws_round(16 * M * R * FF) +
           ws_round(16 * (L > M ? L : M) * R * FF) + ws_round(16 * (L < M ? L : M) * FF) +
           ws_round(4 * (L < M ? L : M) * FF) + 4096;
}

int admm_batched(ia_context *ctx, int l, int m, int F, const double2 *H, int nrhs, const double2 *P,
                 const double *lam0, const ia_admm_config *acfg, const double2 *x0_in, double2 *c, int *iters,
                 int *info, WsCursor &cur)
{
    const bool dual = m > l;
    const long long lm = (long long)l * m, n2 = dual ? (long long)l * l : (long long)m * m;
    const int n = dual ? l : m;
    double2 *AT = cur.take<double2>(lm * F);
    double2 *Kf = cur.take<double2>(n2 * F), *Ki = cur.take<double2>(n2 * F);
    double2 *aa22 = cur.take<double2>((size_t)m * nrhs * F);
    double2 *x0 = cur.take<double2>((size_t)m * nrhs * F);
    double2 *Aq = cur.take<double2>(lm * F);
    double2 *Bq = cur.take<double2>((size_t)(l > m ? l : m) * nrhs * F);
    double2 *tau = cur.take<double2>((size_t)(l < m ? l : m) * F);
    int *ipiv = cur.take<int>((size_t)n * F);
    const double2 zero = make_double2(0.0, 0.0), two = make_double2(2.0, 0.0);
    int st;
    // 2 A^H b
    if ((st = zgemm_batched(ctx, OP_C, OP_N, m, nrhs, l, two, H, l, lm, P, l, (long long)l * nrhs, zero, aa22, m,
                            (long long)m * nrhs, F)))
        return st;
    // the c-update inverse: dual K2 = 2 (rho I + 2 A A^H)^-1, primal P = (2 A^H A + rho I)^-1
    if (dual) st = zgemm_batched(ctx, OP_N, OP_C, l, l, m, two, H, l, lm, H, l, lm, zero, Kf, l, n2, F);
    else st = zgemm_batched(ctx, OP_C, OP_N, m, m, l, two, H, l, lm, H, l, lm, zero, Kf, m, n2, F);
    if (st) return st;
    admm_diag_kernel<<<dim3((n + 127) / 128, F), 128, 0, ctx->stream>>>(n, Kf, n2, acfg->rho, Ki, n2,
                                                                          dual ? 2.0 : 1.0);
    IA_LAUNCH_CHECK(ctx);
    if ((st = zgetrf_batched(ctx, n, Kf, n, n2, ipiv, info, F))) return st;
    if ((st = zgetrs_batched(ctx, n, n, Kf, n, n2, ipiv, Ki, n, n2, F))) return st;
    if (dual && (st = ztranspose_batched(ctx, l, m, H, l, lm, AT, m, lm, false, F))) return st;
    // x0 = A \ b: least squares (m <= l) or minimum norm (m > l) through Householder QR
    if (x0_in) {
        if ((st = zcopy2d_batched(ctx, m, nrhs * F, x0_in, m, 0, x0, m, 0, false, 1))) return st;
    } else if (!dual) {
        if ((st = zcopy2d_batched(ctx, l, m * F, H, l, 0, Aq, l, 0, false, 1))) return st;
        if ((st = zcopy2d_batched(ctx, l, nrhs * F, P, l, 0, Bq, l, 0, false, 1))) return st;
        if ((st = zgeqrs_batched(ctx, l, m, Aq, l, lm, nrhs, Bq, l, (long long)l * nrhs, F))) return st;
        if ((st = zbacksolve_upper_batched(ctx, m, nrhs, Aq, l, lm, Bq, l, (long long)l * nrhs, F))) return st;
        if ((st = zcopy2d_batched(ctx, m, nrhs, Bq, l, (long long)l * nrhs, x0, m, (long long)m * nrhs, false, F)))
            return st;
    } else {
        // A^H = Q R (m x l): A x = b with x = Q [y; 0], R^H y = b
        if ((st = ztranspose_batched(ctx, l, m, H, l, lm, Aq, m, lm, true, F))) return st;
        if ((st = qr_batched<double2>(ctx, m, l, Aq, m, lm, tau, F))) return st;
        const int warps = F * nrhs;
        admm_fwd_kernel<<<(warps + 7) / 8, 256, 0, ctx->stream>>>(m, l, nrhs, Aq, P, Bq, F);
        IA_LAUNCH_CHECK(ctx);
        if ((st = apply_q_batched<double2>(ctx, m, l, Aq, tau, nrhs, Bq, l, (long long)l * nrhs, x0,
                                           (long long)m * nrhs, F)))
            return st;
    }
    AdmmArgs a;
    a.l = l;
    a.m = m;
    a.nrhs = nrhs;
    a.norm = acfg->norm;
    a.nm = acfg->max_iters;
    a.gst = acfg->gst_iters;
    a.rho = acfg->rho;
    a.gamma = acfg->gamma;
    a.eps = acfg->epsilon;
    a.p = acfg->p;
    a.A = H;
    a.AT = AT;
    a.K = Ki;
    a.aa22 = aa22;
    a.lam0 = lam0;
    a.x0 = x0;
    a.c = c;
    a.iters = iters;
    a.info = info;
    const int cs = admm_cluster_size(l, m);
    const size_t smem = admm_smem_bytes(l, (m + cs - 1) / cs, dual);
    if (smem > 200 * 1024) return IA_ERR_TOO_LARGE;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)(F * nrhs * cs));
    lc.blockDim = dim3(ADMM_THREADS);
    lc.dynamicSmemBytes = smem;
    lc.stream = ctx->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    lc.attrs = at;
    lc.numAttrs = cs > 1 ? 1 : 0;
    if (dual) {
        IA_CUDA_TRY(cudaFuncSetAttribute(admm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        IA_CUDA_TRY(cudaLaunchKernelEx(&lc, admm_kernel<true>, a, cs));
    } else {
        IA_CUDA_TRY(cudaFuncSetAttribute(admm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        IA_CUDA_TRY(cudaLaunchKernelEx(&lc, admm_kernel<false>, a, 1));
    }
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

}  // namespace ia
