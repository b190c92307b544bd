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
// splitting the m columns of A and the l rows of K2 -- runs every iteration of
// one (frequency, right-hand side).  c, x, u, r stay in shared memory; A, A^T
// and K2 are read from L2 with one output entry per thread (coalesced matrix
// loads, the vector broadcast from shared memory, no cross-lane reductions).
// The l-vector A r, the rows of K2 y and the three stopping norms are combined
// across the cluster through distributed shared memory in rank order, so every
// CTA takes the same stopping decision.  cs depends on (l, m) only, so a
// problem's result does not depend on the rest of the batch.
//
// Arithmetic.  FP64, or (IA_PREC_MIXED) double-float: the matrices are split
// once into FP32 (hi, lo) pairs and the three matrix-vector products of each
// c-update run on the FP32 pipe with error-free products (~2^-48 relative),
// while r, the shrink, the dual update and the norms stay FP64.
#include <cooperative_groups.h>
#include "df32.cuh"
#include "ia_common.cuh"
#include "ia_internal.h"

namespace cg = cooperative_groups;

namespace ia {

constexpr int ADMM_THREADS = 256;
constexpr int ADMM_WARPS = ADMM_THREADS / 32;

struct AdmmF64 {
    typedef double2 M;
    typedef double2 V;
    typedef double2 Acc;
    static __device__ __forceinline__ V vec(double2 x) { return x; }
    static __device__ __forceinline__ Acc zero() { return make_double2(0.0, 0.0); }
    static __device__ __forceinline__ void mac(Acc &a, M m, V v) { zfma(a, m, v); }
    static __device__ __forceinline__ void cmac(Acc &a, M m, V v) { zcfma(a, m, v); }
    static __device__ __forceinline__ void norm(Acc &) {}
    static __device__ __forceinline__ double2 out(Acc a) { return a; }
};

// double-float complex: (re hi, im hi, re lo, im lo)
struct AdmmDF {
    typedef float4 M;
    typedef float4 V;
    struct Acc {
        dfl re, im;
    };
    static __device__ __forceinline__ V vec(double2 x)
    {
        const float rh = __double2float_rn(x.x), ih = __double2float_rn(x.y);
        return make_float4(rh, ih, __double2float_rn(x.x - (double)rh), __double2float_rn(x.y - (double)ih));
    }
    static __device__ __forceinline__ Acc zero() { return Acc{dfl{0.f, 0.f}, dfl{0.f, 0.f}}; }
    // a += m v
    static __device__ __forceinline__ void mac(Acc &a, M m, V v)
    {
        df_mac(a.re, dfl{m.x, m.z}, dfl{v.x, v.z});
        df_mac(a.re, dfl{-m.y, -m.w}, dfl{v.y, v.w});
        df_mac(a.im, dfl{m.x, m.z}, dfl{v.y, v.w});
        df_mac(a.im, dfl{m.y, m.w}, dfl{v.x, v.z});
    }
    // a += conj(m) v
    static __device__ __forceinline__ void cmac(Acc &a, M m, V v)
    {
        df_mac(a.re, dfl{m.x, m.z}, dfl{v.x, v.z});
        df_mac(a.re, dfl{m.y, m.w}, dfl{v.y, v.w});
        df_mac(a.im, dfl{m.x, m.z}, dfl{v.y, v.w});
        df_mac(a.im, dfl{-m.y, -m.w}, dfl{v.x, v.z});
    }
    static __device__ __forceinline__ void norm(Acc &a)
    {
        a.re = df_norm(a.re);
        a.im = df_norm(a.im);
    }
    static __device__ __forceinline__ double2 out(Acc a)
    {
        return make_double2((double)a.re.hi + (double)a.re.lo, (double)a.im.hi + (double)a.im.lo);
    }
};

template <class AR>
struct AdmmArgs {
    typedef typename AR::M M;
    int l, m, nrhs, norm, nm, gst;
    double rho, gamma, eps, p;
    const M *A;           // F x (l x m)     dual
    const M *AT;          // F x (m x l)     dual
    const M *K;           // dual: F x (l x l) K2; primal: F x (m x m) P
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

// sum_{k in [k0, k1)} op(Mat[row + k * ld]) vec[k], renormalising every 8 terms
template <class AR, bool CONJ>
__device__ __forceinline__ double2 admm_dot(const typename AR::M *__restrict__ mat, size_t ld, int k0, int k1,
                                            const typename AR::V *vec)
{
    typename AR::Acc acc = AR::zero();
    int k = k0;
    for (; k + 8 <= k1; k += 8) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const typename AR::M a = mat[(size_t)(k + q) * ld];
            if (CONJ) AR::cmac(acc, a, vec[k + q]);
            else AR::mac(acc, a, vec[k + q]);
        }
        AR::norm(acc);
    }
    for (; k < k1; ++k) {
        const typename AR::M a = mat[(size_t)k * ld];
        if (CONJ) AR::cmac(acc, a, vec[k]);
        else AR::mac(acc, a, vec[k]);
    }
    AR::norm(acc);
    return AR::out(acc);
}

// out[i] (i < rows) = sum_k Mat[row0 + i + k ld] vec[k], k < K: thread per
// (output, split of k) with the partial sums added in split order
template <class AR>
__device__ __forceinline__ void admm_matvec(const typename AR::M *__restrict__ mat, int ld, int row0, int rows, int K,
                                            const typename AR::V *vec, double2 *psum, double2 *out)
{
    const int tid = threadIdx.x;
    if (rows <= 0) {
        __syncthreads();
        return;
    }
    int nsp = rows <= ADMM_THREADS ? ADMM_THREADS / rows : 1;
    if (nsp > 8) nsp = 8;
    const int chunk = (K + nsp - 1) / nsp;
    for (int t = tid; t < nsp * rows; t += ADMM_THREADS) {
        const int i = t % rows, s = t / rows;
        const int k0 = s * chunk, k1 = min(K, k0 + chunk);
        psum[t] = admm_dot<AR, false>(mat + row0 + i, (size_t)ld, k0, k1, vec);
    }
    __syncthreads();
    for (int i = tid; i < rows; i += ADMM_THREADS) {
        double2 s = psum[i];
        for (int q = 1; q < nsp; ++q) s = zadd(s, psum[q * rows + i]);
        out[i] = s;
    }
}

// shared-memory bytes per CTA (all elements 16 bytes): c, x, u, r (FP64) and
// r as V (mloc each); partial sums max(threads, l); dual: y partials (2 l),
// y as V (l), z partials (2 lc), z as V (l); then norm partials
static size_t admm_smem_bytes(int l, int mloc, int lc, bool dual)
{
    size_t v = 5 * (size_t)mloc + (size_t)(l > ADMM_THREADS ? l : ADMM_THREADS);
    if (dual) v += 2 * (size_t)l + l + 2 * (size_t)lc + l;
    return v * 16 + (8 + 3 * ADMM_WARPS + 8) * sizeof(double);
}

template <class AR, bool DUAL>
__global__ void __launch_bounds__(ADMM_THREADS, 1) admm_kernel(AdmmArgs<AR> a, int cs)
{
    typedef typename AR::M M;
    typedef typename AR::V V;
    extern __shared__ double2 sm[];
    const int rank = DUAL && cs > 1 ? (int)cg::this_cluster().block_rank() : 0;
    const int pid = blockIdx.x / cs;
    const int f = pid / a.nrhs, rr = pid - f * a.nrhs;
    const int l = a.l, m = a.m;
    const int mloc = (m + cs - 1) / cs, j0 = rank * mloc;
    const int nloc = max(0, min(m, j0 + mloc) - j0);
    const int lc = (l + cs - 1) / cs, z0 = rank * lc, nz = max(0, min(l, z0 + lc) - z0);
    const int PS = l > ADMM_THREADS ? l : ADMM_THREADS;
    double2 *c = sm, *x = c + mloc, *u = x + mloc, *rd = u + mloc;
    V *rv = reinterpret_cast<V *>(rd + mloc);
    double2 *psum = reinterpret_cast<double2 *>(rv + mloc);
    double2 *ypart = psum + PS;                       // 2 x l      (dual)
    V *yv = reinterpret_cast<V *>(ypart + 2 * l);     // l
    double2 *zpart = reinterpret_cast<double2 *>(yv + l);   // 2 x lc
    V *zv = reinterpret_cast<V *>(zpart + 2 * lc);    // l
    double *red = reinterpret_cast<double *>(DUAL ? reinterpret_cast<double2 *>(zv + l) : psum + PS);   // 2 x 4
    double *wred = red + 8;                           // warps x 3
    int *flag = reinterpret_cast<int *>(wred + 3 * ADMM_WARPS);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;

    const M *A = a.A + (size_t)f * l * m;
    const M *AT = a.AT + (size_t)f * l * m;
    const M *K = a.K + (size_t)f * (DUAL ? (size_t)l * l : (size_t)m * m);
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
                const double2 r = make_double2(fma(rho, xv.x, bv.x) - uv.x, fma(rho, xv.y, bv.y) - uv.y);
                rd[j] = r;
                rv[j] = AR::vec(r);
            }
            __syncthreads();
            if (DUAL) {
                // this CTA's part of y = A r: rows 0..l-1 over its columns
                admm_matvec<AR>(A + (size_t)j0 * l, l, 0, l, nloc, rv, psum, ypart + buf * l);
                if (cs > 1) cg::this_cluster().sync();
                else __syncthreads();
                for (int i = tid; i < l; i += ADMM_THREADS) {
                    double2 s = make_double2(0.0, 0.0);
                    for (int q = 0; q < cs; ++q) {
                        const double2 *yp = cs > 1 ? cg::this_cluster().map_shared_rank(ypart, q) : ypart;
                        s = zadd(s, yp[buf * l + i]);
                    }
                    yv[i] = AR::vec(s);
                }
                __syncthreads();
                // this CTA's rows of z = K2 y
                admm_matvec<AR>(K, l, z0, nz, l, yv, psum, zpart + buf * lc);
                if (cs > 1) cg::this_cluster().sync();
                else __syncthreads();
                for (int i = tid; i < l; i += ADMM_THREADS) {
                    const int q = i / lc;
                    const double2 *zp = cs > 1 ? cg::this_cluster().map_shared_rank(zpart, q) : zpart;
                    zv[i] = AR::vec(zp[buf * lc + i - q * lc]);
                }
                __syncthreads();
            }
            // c_j, then the shrink and dual updates of entry j
            double dc = 0.0, dcx = 0.0, du = 0.0;
            for (int j = tid; j < nloc; j += ADMM_THREADS) {
                double2 cn;
                if (DUAL) {
                    // c_j = (r_j - sum_i conj(A[i, j]) z_i) / rho, A[i, j] = A^T[j + i m]
                    const double2 t = admm_dot<AR, true>(AT + j0 + j, (size_t)m, 0, l, zv);
                    cn = make_double2((rd[j].x - t.x) * inv_rho, (rd[j].y - t.y) * inv_rho);
                } else {
                    cn = admm_dot<AR, false>(K + j, (size_t)m, 0, m, rv);
                }
                const double2 co = c[j], uo = u[j];
                dc += zabs2(zsub(cn, co));
                double2 xn;
                if (a.norm == 2) {
                    xn = make_double2(fma(rho, cn.x, uo.x) / dlr, fma(rho, cn.y, uo.y) / dlr);
                } else {
                    const double2 yv2 = make_double2(fma(uo.x, inv_rho, cn.x), fma(uo.y, inv_rho, cn.y));
                    const double ay = hypot(yv2.x, yv2.y);
                    if (a.norm == 1) {
                        const double sc = ay > lr ? (ay - lr) / ay : 0.0;
                        xn = zscale(yv2, sc);
                    } else if (!(ay <= tau)) {
                        double s = ay;
                        for (int d = 0; d < a.gst; ++d) s = ay - lam_p * p * pow(s, p - 1.0);
                        xn = ay > 0.0 ? zscale(yv2, s / ay) : make_double2(0.0, 0.0);
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
            dc = warp_sum(dc);
            dcx = warp_sum(dcx);
            du = warp_sum(du);
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

// M += s I (n x n per batch entry); Id (if given) = id I
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
    while (cs < 8 && admm_smem_bytes(l, (m + cs - 1) / cs, (l + cs - 1) / cs, true) > 200 * 1024) cs *= 2;
    return cs;
}

size_t admm_ws_bytes(int l, int m, int F, int nrhs)
{
    const size_t L = l, M = m, FF = F, R = nrhs;
    const size_t kd = m <= l ? M * M : L * L;
    return 2 * ws_round(16 * L * M * FF) + 2 * ws_round(16 * kd * FF) + 2 * ws_round(16 * M * R * FF) +
           ws_round(16 * (L > M ? L : M) * R * FF) + ws_round(16 * (L < M ? L : M) * FF) +
           ws_round(4 * (L < M ? L : M) * FF) + 2 * ws_round(16 * L * M * FF) + ws_round(16 * kd * FF) + 4096;
}

template <class AR>
static int admm_launch(ia_context *ctx, bool dual, int cs, size_t smem, int blocks, const AdmmArgs<AR> &a)
{
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)blocks);
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
        IA_CUDA_TRY(cudaFuncSetAttribute(admm_kernel<AR, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024));
        IA_CUDA_TRY(cudaLaunchKernelEx(&lc, admm_kernel<AR, true>, a, cs));
    } else {
        IA_CUDA_TRY(cudaFuncSetAttribute(admm_kernel<AR, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024));
        IA_CUDA_TRY(cudaLaunchKernelEx(&lc, admm_kernel<AR, false>, a, 1));
    }
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

template <class AR>
static void admm_fill(AdmmArgs<AR> &a, int l, int m, int nrhs, const ia_admm_config *acfg, const double2 *aa22,
                      const double *lam0, const double2 *x0, double2 *c, int *iters, int *info)
{
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
    a.aa22 = aa22;
    a.lam0 = lam0;
    a.x0 = x0;
    a.c = c;
    a.iters = iters;
    a.info = info;
}

int admm_batched(ia_context *ctx, int l, int m, int F, const double2 *H, int nrhs, const double2 *P,
                 const double *lam0, const ia_admm_config *acfg, const double2 *x0_in, double2 *c, int *iters,
                 int *info, WsCursor &cur)
{
    const bool dual = m > l;
    const bool mixed = acfg->precision == IA_PREC_MIXED;
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
    // 2 A^H b, and the Gram matrix of the c-update inverse (dual K2 =
    // 2 (rho I + 2 A A^H)^-1, primal P = (2 A^H A + rho I)^-1); double-float
    // products on the mixed path
    const long long lr = (long long)l * nrhs, mr = (long long)m * nrhs;
    if (mixed) {
        if ((st = dfgemm_batched(ctx, OP_C, OP_N, m, nrhs, l, 2.0, H, l, lm, P, l, lr, 0.0, aa22, m, mr, F))) return st;
        if (dual) st = dfgemm_batched(ctx, OP_N, OP_C, l, l, m, 2.0, H, l, lm, H, l, lm, 0.0, Kf, l, n2, F);
        else st = dfgemm_batched(ctx, OP_C, OP_N, m, m, l, 2.0, H, l, lm, H, l, lm, 0.0, Kf, m, n2, F);
    } else {
        if ((st = zgemm_batched(ctx, OP_C, OP_N, m, nrhs, l, two, H, l, lm, P, l, lr, zero, aa22, m, mr, F))) return st;
        if (dual) st = zgemm_batched(ctx, OP_N, OP_C, l, l, m, two, H, l, lm, H, l, lm, zero, Kf, l, n2, F);
        else st = zgemm_batched(ctx, OP_C, OP_N, m, m, l, two, H, l, lm, H, l, lm, zero, Kf, m, n2, F);
    }
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
    const int cs = admm_cluster_size(l, m);
    const size_t smem = admm_smem_bytes(l, (m + cs - 1) / cs, (l + cs - 1) / cs, dual);
    if (smem > 200 * 1024) return IA_ERR_TOO_LARGE;
    const int blocks = F * nrhs * cs;
    if (!mixed) {
        AdmmArgs<AdmmF64> a;
        admm_fill(a, l, m, nrhs, acfg, aa22, lam0, x0, c, iters, info);
        a.A = H;
        a.AT = AT;
        a.K = Ki;
        return admm_launch(ctx, dual, cs, smem, blocks, a);
    }
    // double-float copies of A, A^T and the inverse
    float4 *Adf = cur.take<float4>(lm * F), *ATdf = cur.take<float4>(lm * F), *Kdf = cur.take<float4>(n2 * F);
    if (dual) {
        if ((st = split_df_batched(ctx, (size_t)lm * F, H, Adf))) return st;
        if ((st = split_df_batched(ctx, (size_t)lm * F, AT, ATdf))) return st;
    }
    if ((st = split_df_batched(ctx, (size_t)n2 * F, Ki, Kdf))) return st;
    AdmmArgs<AdmmDF> a;
    admm_fill(a, l, m, nrhs, acfg, aa22, lam0, x0, c, iters, info);
    a.A = Adf;
    a.AT = ATdf;
    a.K = Kdf;
    return admm_launch(ctx, dual, cs, smem, blocks, a);
}

}  // namespace ia
