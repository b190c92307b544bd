// Regularised solve of wide or square operators H (m x n, m <= n) -- the
// shape of every transfer matrix in the pipeline (microphones x unknowns).
//
// FP64 path (wide_solve_batched):
//   Y = H^H (n x m)
//   Y = Q R                      Householder QR, reflectors kept (skipped if n == m)
//   [R; conj(b)^T] J             one-sided Jacobi on R (m x m); the appended
//                                rows ride along, so they end as conj(J^H b)^T
//   sigma_j, U_R = R J / sigma   (H = J S (Q U_R)^H: U_H = J, V_H = Q U_R)
//   beta = J^H b                 read off the appended rows
//   lambda, z = phi .* beta      GCV / TSVD / fixed (gcv.cuh)
//   x = Q [U_R z; 0]             small GEMM, then the reflectors
// Neither U_H nor V_H is formed.
//
// Mixed path (wide_solve_mixed_batched): the same QR / Jacobi / GCV chain in
// FP32 (sigma, beta and lambda carried to FP64), V_H = Q [U_R; 0] formed in
// FP32, then x is recovered in FP64 by preconditioned iterative refinement of
// the Tikhonov normal equations (H^H H + lambda^2 I) x = H^H b: residuals with
// the FP64 operator, corrections through V_H diag(1/(s^2+lambda^2)) V_H^H.
//
// Both replace the reference's csvd + gcvG + tikhonovG / tsvd chain
// (CUDA/tsvd.cuh:10-172, MATLAB/regtools) for the batched path.
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

constexpr int QR_THREADS = 512;

// One CTA per matrix.  Column j: reflector H_j = I - tau v v^H, v(0) = 1
// (LAPACK zlarfg convention, beta = -sign(Re alpha) ||x||), stored below the
// diagonal; H_j^H applied to the trailing columns of A and to every column of
// B (B may be null).  tau may be null.
template <class T>
__global__ void __launch_bounds__(QR_THREADS) qr_kernel(int rows, int cols, T *A, int lda, long long sA, T *tau,
                                                        int nrhs, T *B, int ldb, long long sB)
{
    typedef typename ctraits<T>::R R;
    __shared__ R red[QR_THREADS / 32];
    __shared__ T s_tau;
    __shared__ T s_scale;   // 1/(alpha - beta)
    const int f = blockIdx.x;
    A += f * sA;
    if (B) B += f * sB;
    if (tau) tau += (size_t)f * cols;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = QR_THREADS / 32;
    const T zero = ctraits<T>::make(0, 0);
    for (int j = 0; j < cols && j < rows; ++j) {
        T *x = A + j + (size_t)j * lda;
        const int len = rows - j;
        R sg = 0;
        for (int i = 1 + tid; i < len; i += QR_THREADS) sg += zabs2(x[i]);
        sg = warp_sum(sg);
        if (lane == 0) red[wid] = sg;
        __syncthreads();
        if (tid == 0) {
            R sigma = 0;
            for (int w = 0; w < nw; ++w) sigma += red[w];
            T alpha = x[0];
            if (sigma == 0 && alpha.y == 0) {
                s_tau = zero;
                s_scale = zero;
            } else {
                R nrm = sqrt(zabs2(alpha) + sigma);
                R beta = alpha.x >= 0 ? -nrm : nrm;
                s_tau = ctraits<T>::make((beta - alpha.x) / beta, -alpha.y / beta);
                s_scale = zdiv(ctraits<T>::make(1, 0), ctraits<T>::make(alpha.x - beta, alpha.y));
                x[0] = ctraits<T>::make(beta, 0);
            }
            if (tau) tau[j] = s_tau;
        }
        __syncthreads();
        const T tv = s_tau, sc = s_scale;
        if (tv.x == 0 && tv.y == 0) continue;
        for (int i = 1 + tid; i < len; i += QR_THREADS) x[i] = zmul(x[i], sc);
        __syncthreads();
        const T ctau = zconj(tv);
        const int ntrail = cols - j - 1;
        const int ntot = ntrail + (B ? nrhs : 0);
        for (int c = wid; c < ntot; c += nw) {
            T *col = c < ntrail ? A + j + (size_t)(j + 1 + c) * lda : B + j + (size_t)(c - ntrail) * ldb;
            T w = lane == 0 ? col[0] : zero;
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
    qr_kernel<double2><<<batch, QR_THREADS, 0, ctx->stream>>>(rows, cols, A, lda, sA, nullptr, nrhs, B, ldb, sB);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// Raug ((N + nrhs) x N): R (upper triangle of Y, or all of Y when full) over
// the rows conj(b_r)^T.
template <class T>
__global__ void build_raug_kernel(int N, int Mrows, int nrhs, const T *Y, const double2 *B, int full, T *Rg)
{
    typedef typename ctraits<T>::R R;
    const int f = blockIdx.y;
    const int ld = N + nrhs;
    const long long total = (long long)ld * N;
    Y += (size_t)f * Mrows * N;
    Rg += (size_t)f * ld * N;
    const double2 *b = B + (size_t)f * nrhs * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        int i = (int)(e % ld), j = (int)(e / ld);
        T v;
        if (i < N) {
            v = (full || i <= j) ? Y[i + (size_t)j * Mrows] : ctraits<T>::make(0, 0);
        } else {
            double2 bb = b[(size_t)(i - N) * N + j];
            v = ctraits<T>::make((R)bb.x, -(R)bb.y);
        }
        Rg[e] = v;
    }
}

// sigma (sorted, FP64 out), beta = conj(appended rows) (sorted, FP64 out),
// U_R = R/sigma (sorted, element type T).
template <class T>
__global__ void finalize_wide_kernel(int N, int nrhs, const T *Rg, double *S, double2 *BETA, T *UR, int *info)
{
    typedef typename ctraits<T>::R R;
    extern __shared__ double sm[];
    double *sig = sm;
    int *rank = reinterpret_cast<int *>(sm + N);
    const int f = blockIdx.x;
    const int ld = N + nrhs;
    Rg += (size_t)f * ld * N;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = wid; j < N; j += nw) {
        R a = 0;
        for (int r = lane; r < N; r += 32) a += zabs2(Rg[r + (size_t)j * ld]);
        a = warp_sum(a);
        if (lane == 0) sig[j] = sqrt((double)a);
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
        for (int r = 0; r < nrhs; ++r) {
            T v = Rg[N + r + (size_t)j * ld];
            BETA[((size_t)f * nrhs + r) * N + rk] = make_double2((double)v.x, -(double)v.y);
        }
    }
    __syncthreads();
    for (int j = wid; j < N; j += nw) {
        R inv = sig[j] > 0.0 ? (R)(1.0 / sig[j]) : (R)0;
        T *dst = UR + (size_t)f * N * N + (size_t)rank[j] * N;
        for (int r = lane; r < N; r += 32) dst[r] = zscale(Rg[r + (size_t)j * ld], inv);
    }
}

// X (rows x ncol per frequency, column stride ldx) = H_0 H_1 ... H_{cols-1} [W; 0]
template <class T>
__global__ void apply_q_kernel(int rows, int cols, const T *Y, const T *TAU, int ncol, const T *W, int ldw,
                               long long sW, T *X, long long sX)
{
    const int f = blockIdx.x;
    Y += (size_t)f * rows * cols;
    TAU += (size_t)f * cols;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const T zero = ctraits<T>::make(0, 0);
    for (int r = wid; r < ncol; r += nw) {
        T *x = X + f * sX + (size_t)r * rows;
        const T *w = W + f * sW + (size_t)r * ldw;
        for (int i = lane; i < rows; i += 32) x[i] = i < cols ? w[i] : zero;
        __syncwarp();
        for (int j = cols - 1; j >= 0; --j) {
            const T t = TAU[j];
            if (t.x == 0 && t.y == 0) continue;
            const T *v = Y + (size_t)j * rows;      // v(j) = 1, v(j+1:) below the diagonal
            T acc = lane == 0 ? x[j] : zero;
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
    double2 *Rg = cur.take<double2>((size_t)(N + nrhs) * N * batch);
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
        qr_kernel<double2><<<batch, QR_THREADS, 0, ctx->stream>>>(Mr, N, Y, Mr, (long long)Mr * N, tau, 0, nullptr, 0,
                                                                  0);
        IA_LAUNCH_CHECK(ctx);
    }
    {
        long long total = (long long)(N + nrhs) * N;
        int blocks = (int)((total + 255) / 256);
        if (blocks > 512) blocks = 512;
        build_raug_kernel<double2><<<dim3(blocks, batch), 256, 0, ctx->stream>>>(N, Mr, nrhs, Y, b, qr ? 0 : 1, Rg);
        IA_LAUNCH_CHECK(ctx);
    }
    st = jacobi_rows_batched<double2>(ctx, N + nrhs, N, N, Rg, nullptr, batch, cfg->svd_max_sweeps, info);
    if (st) return st;
    finalize_wide_kernel<double2><<<batch, 256, (size_t)N * (sizeof(double) + sizeof(int)), ctx->stream>>>(
        N, nrhs, Rg, s, beta, UR, info);
    IA_LAUNCH_CHECK(ctx);
    st = gcv_beta_batched(ctx, m, N, batch, s, nrhs, beta, nullptr, cfg, z, lambda);
    if (st) return st;
    // w = U_R z  (N x nrhs); directly into x when there is no Q
    st = zgemm_batched(ctx, OP_N, OP_N, N, nrhs, N, make_double2(1.0, 0.0), UR, N, (long long)N * N, z, N,
                       (long long)N * nrhs, make_double2(0.0, 0.0), qr ? w : x, N, (long long)N * nrhs, batch);
    if (st) return st;
    if (qr) {
        apply_q_kernel<double2><<<batch, 256, 0, ctx->stream>>>(Mr, N, Y, tau, nrhs, w, N, (long long)N * nrhs, x,
                                                                (long long)Mr * nrhs);
        IA_LAUNCH_CHECK(ctx);
    }
    return IA_OK;
}

// --------------------------------------------------------------------------
// mixed path
// --------------------------------------------------------------------------
constexpr int REFINE_THREADS = 256;

// One CTA per (frequency, right-hand side).  H is m x n (FP64): given as H
// (column-major m x n) or as H^T (column-major n x m).  V (n x N, FP32) and
// s (N) approximate H's right singular vectors and values; lambda fixed.
// x_{k+1} = x_k + V diag(1/(s^2+lambda^2)) V^H (H^H (b - H x_k) - lambda^2 x_k)
__global__ void __launch_bounds__(REFINE_THREADS) tikhonov_refine_kernel(int m, int n, int N, const double2 *H,
                                                                           int transposed, const float2 *V,
                                                                           const double *S, const double *LAM,
                                                                           int nrhs, const double2 *Bv, int steps,
                                                                           double2 *X)
{
    extern __shared__ double2 smz[];
    double2 *x = smz;          // n
    double2 *g = x + n;        // n
    double2 *r1 = g + n;       // m
    double2 *t2 = r1 + m;      // N
    const int f = blockIdx.x, rr = blockIdx.y;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    H += (size_t)f * m * n;
    V += (size_t)f * n * N;
    S += (size_t)f * N;
    const double lam = LAM[(size_t)f * nrhs + rr], l2 = lam * lam;
    const double2 *b = Bv + ((size_t)f * nrhs + rr) * m;
    const double2 zero = make_double2(0.0, 0.0);
    for (int i = tid; i < n; i += blockDim.x) x[i] = zero;
    __syncthreads();
    for (int it = 0; it < steps; ++it) {
        // r1 = b - H x
        if (transposed) {
            // H(i, j) = Ht[j + i n]: column i of Ht is row i of H -> warp per row
            for (int i = wid; i < m; i += nw) {
                double2 acc = zero;
                const double2 *col = H + (size_t)i * n;
                for (int j = lane; j < n; j += 32) zfma(acc, col[j], x[j]);
                acc = warp_sum2(acc);
                if (lane == 0) r1[i] = zsub(b[i], acc);
            }
        } else {
            for (int i = tid; i < m; i += blockDim.x) {
                double2 acc = zero;
                for (int j = 0; j < n; ++j) zfma(acc, H[i + (size_t)j * m], x[j]);
                r1[i] = zsub(b[i], acc);
            }
        }
        __syncthreads();
        // g = H^H r1 - lambda^2 x
        if (transposed) {
            for (int j = tid; j < n; j += blockDim.x) {
                double2 acc = zero;
                for (int i = 0; i < m; ++i) zcfma(acc, H[j + (size_t)i * n], r1[i]);
                g[j] = zsub(acc, zscale(x[j], l2));
            }
        } else {
            for (int j = wid; j < n; j += nw) {
                double2 acc = zero;
                const double2 *col = H + (size_t)j * m;
                for (int i = lane; i < m; i += 32) zcfma(acc, col[i], r1[i]);
                acc = warp_sum2(acc);
                if (lane == 0) g[j] = zsub(acc, zscale(x[j], l2));
            }
        }
        __syncthreads();
        // preconditioner V diag(1/(s^2+l^2)) V^H + (I - V V^H)/l^2:
        // t2 = (1/(s^2+l^2) - 1/l^2) V^H g, correction V t2 + g/l^2
        const double il2 = l2 > 0.0 ? 1.0 / l2 : 0.0;
        for (int k = wid; k < N; k += nw) {
            double2 acc = zero;
            const float2 *vc = V + (size_t)k * n;
            for (int j = lane; j < n; j += 32) {
                float2 v = vc[j];
                zcfma(acc, make_double2(v.x, v.y), g[j]);
            }
            acc = warp_sum2(acc);
            if (lane == 0) {
                double sk = S[k];
                double d = sk * sk + l2;
                t2[k] = zscale(acc, d > 0.0 ? 1.0 / d - il2 : 0.0);
            }
        }
        __syncthreads();
        // x += V t2 + g / l^2
        for (int j = tid; j < n; j += blockDim.x) {
            double2 acc = zadd(x[j], zscale(g[j], il2));
            for (int k = 0; k < N; ++k) {
                float2 v = V[j + (size_t)k * n];
                zfma(acc, make_double2(v.x, v.y), t2[k]);
            }
            x[j] = acc;
        }
        __syncthreads();
    }
    double2 *xo = X + ((size_t)f * nrhs + rr) * n;
    for (int j = tid; j < n; j += blockDim.x) xo[j] = x[j];
}

size_t wide_solve_mixed_ws_bytes(int m, int n, int nrhs, int batch)
{
    const size_t F = batch, N = m, M = n, R = nrhs;
    return ws_round(16 * M * N * F) + ws_round(8 * M * N * F) + ws_round(8 * N * F) + ws_round(8 * (N + R) * N * F) +
           ws_round(8 * N * F) + ws_round(16 * R * N * F) * 2 + ws_round(8 * N * N * F) + ws_round(8 * M * N * F) +
           4096;
}

int wide_solve_mixed_batched(ia_context *ctx, int m, int n, int batch, const double2 *A, bool transposed, int nrhs,
                             const double2 *b, const ia_config *cfg, double2 *x, double *lambda, double *s_out,
                             int *info, WsCursor &cur)
{
    const int N = m, Mr = n;
    const bool qr = n > m;
    double2 *Yd = transposed ? nullptr : cur.take<double2>((size_t)Mr * N * batch);
    float2 *Y = cur.take<float2>((size_t)Mr * N * batch);
    float2 *tau = cur.take<float2>((size_t)N * batch);
    float2 *Rg = cur.take<float2>((size_t)(N + nrhs) * N * batch);
    double *s = s_out ? s_out : cur.take<double>((size_t)N * batch);
    double2 *beta = cur.take<double2>((size_t)nrhs * N * batch);
    double2 *z = cur.take<double2>((size_t)nrhs * N * batch);
    float2 *UR = cur.take<float2>((size_t)N * N * batch);
    float2 *V = cur.take<float2>((size_t)Mr * N * batch);
    double *lam = lambda ? lambda : cur.take<double>((size_t)nrhs * batch);
    const long long sA = (long long)m * n, sY = (long long)Mr * N;
    int st;
    // Y = A^H in FP32
    if (transposed) {
        st = copy2d_batched<double2, float2>(ctx, n, m, A, n, sA, Y, Mr, sY, true, batch);
    } else {
        st = ztranspose_batched(ctx, m, n, A, m, sA, Yd, Mr, sY, true, batch);
        if (!st) st = copy2d_batched<double2, float2>(ctx, Mr, N, Yd, Mr, sY, Y, Mr, sY, false, batch);
    }
    if (st) return st;
    if (qr) {
        qr_kernel<float2><<<batch, QR_THREADS, 0, ctx->stream>>>(Mr, N, Y, Mr, sY, tau, 0, nullptr, 0, 0);
        IA_LAUNCH_CHECK(ctx);
    }
    {
        long long total = (long long)(N + nrhs) * N;
        int blocks = (int)((total + 255) / 256);
        if (blocks > 512) blocks = 512;
        build_raug_kernel<float2><<<dim3(blocks, batch), 256, 0, ctx->stream>>>(N, Mr, nrhs, Y, b, qr ? 0 : 1, Rg);
        IA_LAUNCH_CHECK(ctx);
    }
    st = jacobi_rows_batched<float2>(ctx, N + nrhs, N, N, Rg, nullptr, batch, cfg->svd_max_sweeps, info);
    if (st) return st;
    finalize_wide_kernel<float2><<<batch, 256, (size_t)N * (sizeof(double) + sizeof(int)), ctx->stream>>>(
        N, nrhs, Rg, s, beta, UR, info);
    IA_LAUNCH_CHECK(ctx);
    st = gcv_beta_batched(ctx, m, N, batch, s, nrhs, beta, nullptr, cfg, z, lam);
    if (st) return st;
    // V_H = Q [U_R; 0] (n x N, FP32)
    if (qr) {
        apply_q_kernel<float2><<<batch, 256, 0, ctx->stream>>>(Mr, N, Y, tau, N, UR, N, (long long)N * N, V, sY);
        IA_LAUNCH_CHECK(ctx);
    } else {
        st = copy2d_batched<float2, float2>(ctx, N, N, UR, N, (long long)N * N, V, N, (long long)N * N, false, batch);
        if (st) return st;
    }
    if (cfg->method == IA_METHOD_TSVD) {
        // TSVD keeps the FP32 factors: x = V (phi .* beta), phi from gcv_beta_batched (lambda = 0)
        double2 *Vd = cur.take<double2>((size_t)Mr * N * batch);
        st = copy2d_batched<float2, double2>(ctx, Mr, N, V, Mr, sY, Vd, Mr, sY, false, batch);
        if (st) return st;
        return zgemm_batched(ctx, OP_N, OP_N, Mr, nrhs, N, make_double2(1.0, 0.0), Vd, Mr, sY, z, N,
                             (long long)N * nrhs, make_double2(0.0, 0.0), x, Mr, (long long)Mr * nrhs, batch);
    }
    size_t smem = sizeof(double2) * (2 * (size_t)n + (size_t)m + (size_t)N);
    if (smem > 200 * 1024) return IA_ERR_TOO_LARGE;
    IA_CUDA_TRY(cudaFuncSetAttribute(tikhonov_refine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    tikhonov_refine_kernel<<<dim3(batch, nrhs), REFINE_THREADS, smem, ctx->stream>>>(
        m, n, N, A, transposed ? 1 : 0, V, s, lam, nrhs, b, cfg->refine_steps + 1, x);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

}  // namespace ia
