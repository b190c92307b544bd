// Regularised solve of wide or square operators H (m x n, m <= n) -- the
// shape of every transfer matrix in the pipeline (microphones x unknowns).
//
//   Y = H^H (n x m)
//   Y = Q R                      Householder QR, reflectors kept (skipped if n == m)
//   [R; conj(b)^T] J             one-sided Jacobi on R (m x m); the appended
//                                rows ride along, so they end as conj(J^H b)^T
//   sigma_j, U_R = R J / sigma   (H = J S (Q U_R)^H: U_H = J, V_H = Q U_R)
//   beta = J^H b                 read off the appended rows
//   lambda, z = phi .* beta      GCV / TSVD / fixed (gcv.cuh)
//   x = Q [U_R z; 0]             small GEMM, then the reflectors
// Neither U_H nor V_H is formed.  This replaces the reference's csvd + gcvG +
// tikhonovG / tsvd chain (CUDA/tsvd.cuh:10-172, MATLAB/regtools) for the
// batched path; Jacobi work runs on m rows instead of n.
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

constexpr int QR_THREADS = 512;

// One CTA per matrix.  Column j: reflector H_j = I - tau v v^H, v(0) = 1
// (LAPACK zlarfg convention, beta = -sign(Re alpha) ||x||), stored below the
// diagonal; H_j^H applied to the trailing columns of A and to every column of
// B (B may be null).  tau may be null.
__global__ void __launch_bounds__(QR_THREADS) qr_kernel(int rows, int cols, double2 *A, int lda, long long sA,
                                                        double2 *tau, int nrhs, double2 *B, int ldb, long long sB)
{
    __shared__ double red[QR_THREADS / 32];
    __shared__ double2 s_tau;
    __shared__ double2 s_scale;   // 1/(alpha - beta)
    const int f = blockIdx.x;
    A += f * sA;
    if (B) B += f * sB;
    if (tau) tau += (size_t)f * cols;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = QR_THREADS / 32;
    for (int j = 0; j < cols && j < rows; ++j) {
        double2 *x = A + j + (size_t)j * lda;
        const int len = rows - j;
        double sg = 0.0;
        for (int i = 1 + tid; i < len; i += QR_THREADS) sg += zabs2(x[i]);
        sg = warp_sum(sg);
        if (lane == 0) red[wid] = sg;
        __syncthreads();
        if (tid == 0) {
            double sigma = 0.0;
            for (int w = 0; w < nw; ++w) sigma += red[w];
            double2 alpha = x[0];
            if (sigma == 0.0 && alpha.y == 0.0) {
                s_tau = make_double2(0.0, 0.0);
                s_scale = make_double2(0.0, 0.0);
            } else {
                double nrm = sqrt(zabs2(alpha) + sigma);
                double beta = alpha.x >= 0.0 ? -nrm : nrm;
                s_tau = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
                s_scale = zdiv(make_double2(1.0, 0.0), make_double2(alpha.x - beta, alpha.y));
                x[0] = make_double2(beta, 0.0);
            }
            if (tau) tau[j] = s_tau;
        }
        __syncthreads();
        const double2 tv = s_tau, sc = s_scale;
        if (tv.x == 0.0 && tv.y == 0.0) continue;
        for (int i = 1 + tid; i < len; i += QR_THREADS) x[i] = zmul(x[i], sc);
        __syncthreads();
        const double2 ctau = zconj(tv);
        const int ntrail = cols - j - 1;
        const int ntot = ntrail + (B ? nrhs : 0);
        for (int c = wid; c < ntot; c += nw) {
            double2 *col = c < ntrail ? A + j + (size_t)(j + 1 + c) * lda : B + j + (size_t)(c - ntrail) * ldb;
            double2 w = lane == 0 ? col[0] : make_double2(0.0, 0.0);
            for (int i = 1 + lane; i < len; i += 32) zcfma(w, x[i], col[i]);
            w = warp_sum2(w);
            w = zmul(ctau, w);
            if (lane == 0) col[0] = zsub(col[0], w);
            for (int i = 1 + lane; i < len; i += 32) zfms(col[i], x[i], w);
        }
        __syncthreads();
    }
}

int zgeqrs_batched(ia_context *ctx, int rows, int cols, double2 *A, int lda, long long sA, int nrhs, double2 *B,
                   int ldb, long long sB, int batch)
{
    qr_kernel<<<batch, QR_THREADS, 0, ctx->stream>>>(rows, cols, A, lda, sA, nullptr, nrhs, B, ldb, sB);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// Raug ((N + nrhs) x N): R (upper triangle of Y, or all of Y when full) over
// the rows conj(b_r)^T.
__global__ void build_raug_kernel(int N, int Mrows, int nrhs, const double2 *Y, const double2 *B, int full,
                                  double2 *R)
{
    const int f = blockIdx.y;
    const int ld = N + nrhs;
    const long long total = (long long)ld * N;
    Y += (size_t)f * Mrows * N;
    R += (size_t)f * ld * N;
    const double2 *b = B + (size_t)f * nrhs * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        int i = (int)(e % ld), j = (int)(e / ld);
        double2 v;
        if (i < N) v = (full || i <= j) ? Y[i + (size_t)j * Mrows] : make_double2(0.0, 0.0);
        else v = zconj(b[(size_t)(i - N) * N + j]);
        R[e] = v;
    }
}

// sigma (sorted), beta = conj(appended rows) (sorted), U_R = R/sigma (sorted).
__global__ void finalize_wide_kernel(int N, int nrhs, const double2 *R, double *S, double2 *BETA, double2 *UR,
                                     int *info)
{
    extern __shared__ double sm[];
    double *sig = sm;
    int *rank = reinterpret_cast<int *>(sm + N);
    const int f = blockIdx.x;
    const int ld = N + nrhs;
    R += (size_t)f * ld * N;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = wid; j < N; j += nw) {
        double a = 0.0;
        for (int r = lane; r < N; r += 32) a += zabs2(R[r + (size_t)j * ld]);
        a = warp_sum(a);
        if (lane == 0) sig[j] = sqrt(a);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        double sj = sig[j];
        int rk = 0;
        for (int i = 0; i < N; ++i) {
            double si = sig[i];
            if (si > sj || (si == sj && i < j)) rk++;
        }
        rank[j] = rk;
        S[(size_t)f * N + rk] = sj;
        if (info && (!(sj == sj) || isinf(sj))) atomicOr(&info[f], IA_INFO_NONFINITE);
        for (int r = 0; r < nrhs; ++r) BETA[((size_t)f * nrhs + r) * N + rk] = zconj(R[N + r + (size_t)j * ld]);
    }
    __syncthreads();
    for (int j = wid; j < N; j += nw) {
        double inv = sig[j] > 0.0 ? 1.0 / sig[j] : 0.0;
        double2 *dst = UR + (size_t)f * N * N + (size_t)rank[j] * N;
        for (int r = lane; r < N; r += 32) dst[r] = zscale(R[r + (size_t)j * ld], inv);
    }
}

// x (rows x nrhs) = H_0 H_1 ... H_{cols-1} [W; 0], reflectors from qr_kernel.
__global__ void apply_q_kernel(int rows, int cols, const double2 *Y, const double2 *TAU, int nrhs, const double2 *W,
                               double2 *X)
{
    const int f = blockIdx.x;
    Y += (size_t)f * rows * cols;
    TAU += (size_t)f * cols;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int r = wid; r < nrhs; r += nw) {
        double2 *x = X + ((size_t)f * nrhs + r) * rows;
        const double2 *w = W + ((size_t)f * nrhs + r) * cols;
        for (int i = lane; i < rows; i += 32) x[i] = i < cols ? w[i] : make_double2(0.0, 0.0);
        __syncwarp();
        for (int j = cols - 1; j >= 0; --j) {
            const double2 t = TAU[j];
            if (t.x == 0.0 && t.y == 0.0) continue;
            const double2 *v = Y + (size_t)j * rows;      // v(j) = 1, v(j+1:) below the diagonal
            double2 acc = lane == 0 ? x[j] : make_double2(0.0, 0.0);
            for (int i = j + 1 + lane; i < rows; i += 32) zcfma(acc, v[i], x[i]);
            acc = warp_sum2(acc);
            acc = zmul(t, acc);
            if (lane == 0) x[j] = zsub(x[j], acc);
            for (int i = j + 1 + lane; i < rows; i += 32) zfms(x[i], v[i], acc);
            __syncwarp();
        }
    }
}

size_t wide_solve_ws_bytes(int m, int n, int nrhs, int batch)
{
    const size_t F = batch, N = m, M = n, R = nrhs;
    return ws_round(16 * M * N * F) + ws_round(16 * N * F) + ws_round(16 * (N + R) * N * F) + ws_round(8 * N * F) +
           ws_round(16 * R * N * F) * 3 + ws_round(16 * N * N * F) + 2048;
}

int wide_solve_batched(ia_context *ctx, int m, int n, int batch, const double2 *A, bool transposed, int nrhs,
                       const double2 *b, const ia_config *cfg, double2 *x, double *lambda, double *s_out, int *info,
                       WsCursor &cur)
{
    const int N = m, Mr = n;
    const bool qr = n > m;
    double2 *Y = cur.take<double2>((size_t)Mr * N * batch);
    double2 *tau = cur.take<double2>((size_t)N * batch);
    double2 *R = cur.take<double2>((size_t)(N + nrhs) * N * batch);
    double *s = s_out ? s_out : cur.take<double>((size_t)N * batch);
    double2 *beta = cur.take<double2>((size_t)nrhs * N * batch);
    double2 *z = cur.take<double2>((size_t)nrhs * N * batch);
    double2 *w = cur.take<double2>((size_t)nrhs * N * batch);
    double2 *UR = cur.take<double2>((size_t)N * N * batch);
    const long long sA = (long long)m * n;
    int st;
    // Y = A^H
    if (transposed) st = zcopy2d_batched(ctx, n, m, A, n, sA, Y, Mr, (long long)Mr * N, true, batch);
    else st = ztranspose_batched(ctx, m, n, A, m, sA, Y, Mr, (long long)Mr * N, true, batch);
    if (st) return st;
    if (qr) {
        qr_kernel<<<batch, QR_THREADS, 0, ctx->stream>>>(Mr, N, Y, Mr, (long long)Mr * N, tau, 0, nullptr, 0, 0);
        IA_LAUNCH_CHECK(ctx);
    }
    {
        long long total = (long long)(N + nrhs) * N;
        int blocks = (int)((total + 255) / 256);
        if (blocks > 512) blocks = 512;
        build_raug_kernel<<<dim3(blocks, batch), 256, 0, ctx->stream>>>(N, Mr, nrhs, Y, b, qr ? 0 : 1, R);
        IA_LAUNCH_CHECK(ctx);
    }
    st = jacobi_rows_batched(ctx, N + nrhs, N, N, R, nullptr, batch, cfg->svd_max_sweeps, info);
    if (st) return st;
    finalize_wide_kernel<<<batch, 256, (size_t)N * (sizeof(double) + sizeof(int)), ctx->stream>>>(N, nrhs, R, s, beta,
                                                                                                 UR, info);
    IA_LAUNCH_CHECK(ctx);
    st = gcv_beta_batched(ctx, m, N, batch, s, nrhs, beta, nullptr, cfg, z, lambda);
    if (st) return st;
    // w = U_R z  (N x nrhs); directly into x when there is no Q
    st = zgemm_batched(ctx, OP_N, OP_N, N, nrhs, N, make_double2(1.0, 0.0), UR, N, (long long)N * N, z, N,
                       (long long)N * nrhs, make_double2(0.0, 0.0), qr ? w : x, N, (long long)N * nrhs, batch);
    if (st) return st;
    if (qr) {
        apply_q_kernel<<<batch, 256, 0, ctx->stream>>>(Mr, N, Y, tau, nrhs, w, x);
        IA_LAUNCH_CHECK(ctx);
    }
    return IA_OK;
}

}  // namespace ia
