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
// Mixed path (wide_solve_mixed_batched): QR of H^H and one-sided Jacobi on R
// in FP32 give X ~ U_H (eigenvectors of E = H H^H) to ~1e-5; E is formed by
// the double-float GEMM; Ogita-Aishima refinement steps (all products in
// double-float) bring separated eigenpairs to that level; a two-sided FP64
// Jacobi on S = X^H E X (an FP64 product) separates the near-equal pairs
// those steps leave coupled; then s = sqrt(eig E), beta = U^H b, GCV in FP64, and
// x = H^H U diag(phi / s) beta against the FP64 operator.
//
// Both replace the reference's csvd + gcvG + tikhonovG / tsvd chain
// (CUDA/tsvd.cuh:10-172, MATLAB/regtools) for the batched path.
#include <cooperative_groups.h>
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

namespace cg = cooperative_groups;

constexpr int QR_THREADS = 512;

// One CTA per matrix.  Column j: reflector H_j = I - tau v v^H, v(0) = 1
// (LAPACK zlarfg convention, beta = -sign(Re alpha) ||x||), stored below the
// diagonal; H_j^H applied to the trailing columns of A and to every column of
// B (B may be null).  tau may be null.  KPL > 0 (rows <= 1 + 32 KPL, dynamic
// shared memory of rows elements): the reflector is kept in shared memory and
// each trailing column's segment in registers, so a column costs one round of
// independent loads instead of a dependent load per element; the arithmetic
// and its order are those of KPL = 0.  PIV: column pivoting (perm).
template <class T, int KPL, bool PIV>
__global__ void __launch_bounds__(QR_THREADS) qr_kernel(int rows, int cols, T *A, int lda, long long sA, T *tau,
                                                        int nrhs, T *B, int ldb, long long sB, int *perm)
{
    typedef typename ctraits<T>::R R;
    extern __shared__ __align__(16) unsigned char qr_smem[];
    T *xs = reinterpret_cast<T *>(qr_smem);   // the scaled reflector (KPL > 0)
    R *cn = reinterpret_cast<R *>(qr_smem + (KPL > 0 ? sizeof(T) * (size_t)rows : 0));   // pivoting: column norms^2
    int *idx = reinterpret_cast<int *>(cn + cols);                                        // pivoting: column order
    __shared__ R red[QR_THREADS / 32];
    __shared__ T s_tau;
    __shared__ T s_scale;   // 1/(alpha - beta)
    __shared__ int s_piv;
    const int f = blockIdx.x;
    A += f * sA;
    if (B) B += f * sB;
    if (tau) tau += (size_t)f * cols;
    if (PIV) perm += (size_t)f * cols;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = QR_THREADS / 32;
    const T zero = ctraits<T>::make(0, 0);
    if (PIV) {
        for (int c = wid; c < cols; c += nw) {
            R a = 0;
            for (int i = lane; i < rows; i += 32) a += zabs2(A[i + (size_t)c * lda]);
            a = warp_sum(a);
            if (lane == 0) {
                cn[c] = a;
                idx[c] = c;
            }
        }
        __syncthreads();
    }
    for (int j = 0; j < cols && j < rows; ++j) {
        if (PIV) {
            // column pivoting: the remaining column of largest norm (first on
            // ties) moves to position j, whole column (Businger-Golub)
            if (wid == 0) {
                R best = -1;
                int bi = j;
                for (int c = j + lane; c < cols; c += 32)
                    if (cn[c] > best) {
                        best = cn[c];
                        bi = c;
                    }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const R ov = __shfl_xor_sync(0xffffffffu, best, o);
                    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                    if (ov > best || (ov == best && oi < bi)) {
                        best = ov;
                        bi = oi;
                    }
                }
                if (lane == 0) s_piv = bi;
            }
            __syncthreads();
            const int p = s_piv;
            if (p != j) {
                for (int i = tid; i < rows; i += QR_THREADS) {
                    const T t = A[i + (size_t)j * lda];
                    A[i + (size_t)j * lda] = A[i + (size_t)p * lda];
                    A[i + (size_t)p * lda] = t;
                }
                if (tid == 0) {
                    const R tn = cn[j];
                    cn[j] = cn[p];
                    cn[p] = tn;
                    const int ti = idx[j];
                    idx[j] = idx[p];
                    idx[p] = ti;
                }
            }
            __syncthreads();
        }
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
        if (tv.x == 0 && tv.y == 0) {
            // no reflector: the trailing columns' norms lose their row j
            if (PIV) {
                for (int c = j + 1 + tid; c < cols; c += QR_THREADS) {
                    const R v = cn[c] - zabs2(A[j + (size_t)c * lda]);
                    cn[c] = v > 0 ? v : 0;
                }
                __syncthreads();
            }
            continue;
        }
        for (int i = 1 + tid; i < len; i += QR_THREADS) {
            const T xv = zmul(x[i], sc);
            x[i] = xv;
            if (KPL > 0) xs[i] = xv;
        }
        __syncthreads();
        const T ctau = zconj(tv);
        const int ntrail = cols - j - 1;
        const int ntot = ntrail + (B ? nrhs : 0);
        for (int c = wid; c < ntot; c += nw) {
            T *col = c < ntrail ? A + j + (size_t)(j + 1 + c) * lda : B + j + (size_t)(c - ntrail) * ldb;
            T w = lane == 0 ? col[0] : zero;
            if (KPL > 0) {
                T v[KPL > 0 ? KPL : 1];
#pragma unroll
                for (int t = 0; t < KPL; ++t) {
                    const int i = 1 + lane + 32 * t;
                    v[t] = i < len ? col[i] : zero;
                }
#pragma unroll
                for (int t = 0; t < KPL; ++t) {
                    const int i = 1 + lane + 32 * t;
                    if (i < len) zcfma(w, xs[i], v[t]);
                }
                w = warp_sum2(w);
                w = zmul(ctau, w);
                if (lane == 0) col[0] = zsub(col[0], w);
                R nr = 0;
#pragma unroll
                for (int t = 0; t < KPL; ++t) {
                    const int i = 1 + lane + 32 * t;
                    if (i < len) {
                        zfms(v[t], xs[i], w);
                        col[i] = v[t];
                        nr += zabs2(v[t]);
                    }
                }
                // pivoting: the norm of the rows below j, exact from the
                // updated segment
                if (PIV && c < ntrail) {
                    nr = warp_sum(nr);
                    if (lane == 0) cn[j + 1 + c] = nr;
                }
            } else {
                for (int i = 1 + lane; i < len; i += 32) zcfma(w, x[i], col[i]);
                w = warp_sum2(w);
                w = zmul(ctau, w);
                if (lane == 0) col[0] = zsub(col[0], w);
                R nr = 0;
                for (int i = 1 + lane; i < len; i += 32) {
                    zfms(col[i], x[i], w);
                    nr += zabs2(col[i]);
                }
                if (PIV && c < ntrail) {
                    nr = warp_sum(nr);
                    if (lane == 0) cn[j + 1 + c] = nr;
                }
            }
        }
        __syncthreads();
    }
    if (PIV)
        for (int c = tid; c < cols; c += QR_THREADS) perm[c] = idx[c];
}

// KPL = 24 covers rows <= 769 (the bench's 642-row H^H)
constexpr int QR_KPL = 24;

// perm (batch x cols, may be null): column pivoting, perm[k] = the input
// column that ends in position k
// ---- column-pivoted QR of one FP32 matrix over a cluster of QRC_CS CTAs ---
// The single-CTA kernel above is a chain of `cols` latency-bound reflector
// steps on one SM.  Here CTA r of a bin's cluster owns columns [r cw, (r+1) cw)
// in its shared memory; per step the owner of column j forms the reflector
// and every CTA applies it to its own columns, so four SMs share the trailing
// updates.  Per step, through distributed shared memory: each CTA's pivot
// candidate (largest remaining norm, first on ties) is read by all, which
// take the same decision; a pivot in another CTA is swapped in by copying the
// two columns across; the reflector is copied from its owner.  Three cluster
// barriers per step (two without a swap).  The arithmetic per column is the
// single-CTA kernel's (warp per column, the same reductions), except the
// reflector's norm, a reduction over the owner's threads.  Mixed path only
// (FP32, pivoted, no right-hand sides); tau may be null.
constexpr int QRC_CS = 4;
constexpr int QRC_THREADS = 512;

__global__ void __launch_bounds__(QRC_THREADS) qr_cluster_kernel(int rows, int cols, float2 *A, int lda, long long sA,
                                                                 float2 *tau, int *perm)
{
    typedef float R;
    constexpr int KPL = QR_KPL;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int f = blockIdx.x / QRC_CS;
    const int cw = (cols + QRC_CS - 1) / QRC_CS;
    const int c0 = rank * cw, c1 = c0 + cw < cols ? c0 + cw : cols, nown = c1 > c0 ? c1 - c0 : 0;
    extern __shared__ __align__(16) unsigned char qrc_smem[];
    float2 *colbuf = reinterpret_cast<float2 *>(qrc_smem);      // nown columns of `rows`
    float2 *xs = colbuf + (size_t)cw * rows;                      // the current reflector (rows)
    float2 *tmp = xs + rows;                                      // a column arriving by a swap (rows)
    R *cn = reinterpret_cast<R *>(tmp + rows);                    // norms^2 of the owned columns' remaining rows
    int *idx = reinterpret_cast<int *>(cn + cw);                  // original index of each owned column
    __shared__ R red[QRC_THREADS / 32];
    __shared__ R cand_v;
    __shared__ int cand_i;
    __shared__ float2 s_tau;
    __shared__ float2 s_scale;
    __shared__ R s_swap_cn;
    __shared__ int s_swap_idx;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = QRC_THREADS / 32;
    const float2 zero = make_float2(0.f, 0.f);
    A += f * sA;
    const long long aext = (long long)cols * lda;
    for (int e = tid; e < nown * rows; e += QRC_THREADS) {
        const int c = e / rows, i = e % rows;
        colbuf[e] = IA_IDX_OK(i + (long long)(c0 + c) * lda, aext) ? A[i + (size_t)(c0 + c) * lda] : zero;
    }
    __syncthreads();
    for (int c = wid; c < nown; c += nw) {
        R a = 0;
        for (int i = lane; i < rows; i += 32) a += zabs2(colbuf[i + (size_t)c * rows]);
        a = warp_sum(a);
        if (lane == 0) {
            cn[c] = a;
            idx[c] = c0 + c;
        }
    }
    __syncthreads();
    const int steps = cols < rows ? cols : rows;
    for (int j = 0; j < steps; ++j) {
        // pivot: this CTA's candidate among its columns >= j, then the cluster's
        if (wid == 0) {
            R best = -1;
            int bi = cols;
            for (int c = lane; c < nown; c += 32)
                if (c0 + c >= j && cn[c] > best) {
                    best = cn[c];
                    bi = c0 + c;
                }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const R ov = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov > best || (ov == best && oi < bi)) {
                    best = ov;
                    bi = oi;
                }
            }
            if (lane == 0) {
                cand_v = best;
                cand_i = bi;
            }
        }
        cluster.sync();
        R pv = -1;
        int p = cols;
        for (int q = 0; q < QRC_CS; ++q) {
            const R v = *cluster.map_shared_rank(&cand_v, q);
            const int i = *cluster.map_shared_rank(&cand_i, q);
            if (v > pv || (v == pv && i < p)) {
                pv = v;
                p = i;
            }
        }
        const int oj = j / cw, op = p / cw;
        if (p != j) {
            if (oj == op) {
                if (rank == oj) {
                    float2 *a = colbuf + (size_t)(j - c0) * rows, *b = colbuf + (size_t)(p - c0) * rows;
                    for (int i = tid; i < rows; i += QRC_THREADS) {
                        const float2 t = a[i];
                        a[i] = b[i];
                        b[i] = t;
                    }
                    if (tid == 0) {
                        const R tn = cn[j - c0];
                        cn[j - c0] = cn[p - c0];
                        cn[p - c0] = tn;
                        const int ti = idx[j - c0];
                        idx[j - c0] = idx[p - c0];
                        idx[p - c0] = ti;
                    }
                }
            } else {
                // each of the two owners copies the other's column in, then
                // (after the barrier) over its own
                if (rank == oj || rank == op) {
                    const int mine = rank == oj ? j : p, other = rank == oj ? p : j;
                    const int orank = rank == oj ? op : oj;
                    const float2 *src = cluster.map_shared_rank(colbuf, orank) + (size_t)(other - orank * cw) * rows;
                    for (int i = tid; i < rows; i += QRC_THREADS) tmp[i] = src[i];
                    if (tid == 0) {
                        s_swap_cn = *cluster.map_shared_rank(cn + (other - orank * cw), orank);
                        s_swap_idx = *cluster.map_shared_rank(idx + (other - orank * cw), orank);
                    }
                    (void)mine;
                }
                cluster.sync();
                if (rank == oj || rank == op) {
                    const int mine = rank == oj ? j : p;
                    float2 *dst = colbuf + (size_t)(mine - c0) * rows;
                    for (int i = tid; i < rows; i += QRC_THREADS) dst[i] = tmp[i];
                    if (tid == 0) {
                        cn[mine - c0] = s_swap_cn;
                        idx[mine - c0] = s_swap_idx;
                    }
                }
            }
        }
        // the reflector of column j, by its owner
        if (rank == oj) {
            __syncthreads();
            float2 *x = colbuf + (size_t)(j - c0) * rows + j;
            const int len = rows - j;
            R sg = 0;
            for (int i = 1 + tid; i < len; i += QRC_THREADS) sg += zabs2(x[i]);
            sg = warp_sum(sg);
            if (lane == 0) red[wid] = sg;
            __syncthreads();
            if (tid == 0) {
                R sigma = 0;
                for (int w = 0; w < nw; ++w) sigma += red[w];
                const float2 alpha = x[0];
                if (sigma == 0 && alpha.y == 0) {
                    s_tau = zero;
                    s_scale = zero;
                } else {
                    const R nrm = sqrtf(zabs2(alpha) + sigma);
                    const R beta = alpha.x >= 0 ? -nrm : nrm;
                    s_tau = make_float2((beta - alpha.x) / beta, -alpha.y / beta);
                    s_scale = zdiv(make_float2(1.f, 0.f), make_float2(alpha.x - beta, alpha.y));
                    x[0] = make_float2(beta, 0.f);
                }
                if (tau) tau[(size_t)f * cols + j] = s_tau;
            }
            __syncthreads();
            const float2 sc = s_scale;
            const bool none = s_tau.x == 0 && s_tau.y == 0;
            for (int i = 1 + tid; i < len; i += QRC_THREADS) {
                const float2 v = none ? x[i] : zmul(x[i], sc);
                if (!none) x[i] = v;
                xs[j + i] = v;
            }
        }
        cluster.sync();
        // every CTA: the reflector (and tau) from the owner, then its columns > j
        float2 tv;
        {
            const float2 *oxs = cluster.map_shared_rank(xs, oj);
            if (rank != oj)
                for (int i = j + 1 + tid; i < rows; i += QRC_THREADS) xs[i] = oxs[i];
            tv = *cluster.map_shared_rank(&s_tau, oj);
        }
        __syncthreads();
        const int len = rows - j;
        const bool none = tv.x == 0 && tv.y == 0;
        const float2 ctau = zconj(tv);
        for (int c = wid; c < nown; c += nw) {
            if (c0 + c <= j) continue;
            float2 *col = colbuf + (size_t)c * rows + j;
            if (none) {
                // no reflector: the norm loses its row j
                if (lane == 0) {
                    const R v = cn[c] - zabs2(col[0]);
                    cn[c] = v > 0 ? v : 0;
                }
                continue;
            }
            float2 w = lane == 0 ? col[0] : zero;
            float2 v[KPL];
#pragma unroll
            for (int t = 0; t < KPL; ++t) {
                const int i = 1 + lane + 32 * t;
                v[t] = i < len ? col[i] : zero;
            }
#pragma unroll
            for (int t = 0; t < KPL; ++t) {
                const int i = 1 + lane + 32 * t;
                if (i < len) zcfma(w, xs[j + i], v[t]);
            }
            w = warp_sum2(w);
            w = zmul(ctau, w);
            if (lane == 0) col[0] = zsub(col[0], w);
            R nr = 0;
#pragma unroll
            for (int t = 0; t < KPL; ++t) {
                const int i = 1 + lane + 32 * t;
                if (i < len) {
                    zfms(v[t], xs[j + i], w);
                    col[i] = v[t];
                    nr += zabs2(v[t]);
                }
            }
            nr = warp_sum(nr);
            if (lane == 0) cn[c] = nr;
        }
        __syncthreads();
    }
    cluster.sync();   // no CTA leaves while another may still read its shared memory
    for (int e = tid; e < nown * rows; e += QRC_THREADS) {
        const int c = e / rows, i = e % rows;
        if (IA_IDX_OK(i + (long long)(c0 + c) * lda, aext)) A[i + (size_t)(c0 + c) * lda] = colbuf[e];
    }
    if (perm)
        for (int c = tid; c < nown; c += QRC_THREADS) perm[(size_t)f * cols + c0 + c] = idx[c];
}

static size_t qr_cluster_smem(int rows, int cols)
{
    const int cw = (cols + QRC_CS - 1) / QRC_CS;
    return sizeof(float2) * ((size_t)cw * rows + 2 * (size_t)rows) + (sizeof(float) + sizeof(int)) * (size_t)cw;
}

template <class T, bool PIV>
static int qr_launch_t(ia_context *ctx, int rows, int cols, T *A, int lda, long long sA, T *tau, int nrhs, T *B,
                       int ldb, long long sB, int batch, int *perm)
{
    typedef typename ctraits<T>::R R;
    const size_t piv = PIV ? (sizeof(R) + sizeof(int)) * (size_t)cols : 0;
    if constexpr (std::is_same<T, float2>::value && PIV) {
        // the cluster form shortens one bin's chain but holds four SMs for
        // ~60 % of the one-CTA form's time (2.3x its SM time): for batches
        // that leave most of the GPU idle (at most a quarter of the SMs in
        // clusters) and for the last part of a staggered pipeline, whose
        // chain ends the pass; the other 16-bin parts of the 64-bin pass take
        // the one-CTA form.  Both forms give bitwise the same factors (the
        // same reductions in the same order, the same pivot rule).
        const size_t csm = qr_cluster_smem(rows, cols);
        if (!B && rows <= 1 + 32 * QR_KPL && cols >= 2 * QRC_CS && csm <= 227 * 1024 &&
            (4 * QRC_CS * batch <= ctx->sm_count || ctx->tail_part)) {
            IA_CUDA_TRY(cudaFuncSetAttribute(qr_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm));
            cudaLaunchConfig_t lc = {};
            lc.gridDim = dim3((unsigned)(QRC_CS * batch));
            lc.blockDim = dim3(QRC_THREADS);
            lc.dynamicSmemBytes = csm;
            lc.stream = ctx->stream;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = QRC_CS;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            lc.attrs = at;
            lc.numAttrs = 1;
            IA_CUDA_TRY(cudaLaunchKernelEx(&lc, qr_cluster_kernel, rows, cols, (float2 *)A, lda, sA, (float2 *)tau,
                                           perm));
            IA_LAUNCH_CHECK(ctx);
            return IA_OK;
        }
    }
    if (rows <= 1 + 32 * QR_KPL) {
        const size_t smem = sizeof(T) * (size_t)rows + piv;
        if (smem > 48 * 1024) {
            if (smem > 227 * 1024) return IA_ERR_TOO_LARGE;
            IA_CUDA_TRY(cudaFuncSetAttribute(qr_kernel<T, QR_KPL, PIV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem));
        }
        qr_kernel<T, QR_KPL, PIV><<<batch, QR_THREADS, smem, ctx->stream>>>(rows, cols, A, lda, sA, tau, nrhs, B,
                                                                           ldb, sB, perm);
    } else {
        if (piv > 48 * 1024) {
            if (piv > 227 * 1024) return IA_ERR_TOO_LARGE;
            IA_CUDA_TRY(cudaFuncSetAttribute(qr_kernel<T, 0, PIV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)piv));
        }
        qr_kernel<T, 0, PIV><<<batch, QR_THREADS, piv, ctx->stream>>>(rows, cols, A, lda, sA, tau, nrhs, B, ldb, sB,
                                                                     perm);
    }
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

template <class T>
static int qr_launch(ia_context *ctx, int rows, int cols, T *A, int lda, long long sA, T *tau, int nrhs, T *B,
                     int ldb, long long sB, int batch, int *perm = nullptr)
{
    if (perm) return qr_launch_t<T, true>(ctx, rows, cols, A, lda, sA, tau, nrhs, B, ldb, sB, batch, perm);
    return qr_launch_t<T, false>(ctx, rows, cols, A, lda, sA, tau, nrhs, B, ldb, sB, batch, nullptr);
}

int zgeqrs_batched(ia_context *ctx, int rows, int cols, double2 *A, int lda, long long sA, int nrhs, double2 *B,
                   int ldb, long long sB, int batch)
{
    return qr_launch<double2>(ctx, rows, cols, A, lda, sA, nullptr, nrhs, B, ldb, sB, batch);
}

template <class T>
int qr_batched(ia_context *ctx, int rows, int cols, T *A, int lda, long long sA, T *tau, int batch)
{
    return qr_launch<T>(ctx, rows, cols, A, lda, sA, tau, 0, nullptr, 0, 0, batch);
}
template int qr_batched<float2>(ia_context *, int, int, float2 *, int, long long, float2 *, int);
template int qr_batched<double2>(ia_context *, int, int, double2 *, int, long long, double2 *, int);

// R^H (N x N) from the QR'd Y: R is the upper triangle of Y (all of Y when full)
__global__ void build_rh_kernel(int N, int Mrows, const float2 *Y, int full, float2 *RH)
{
    const int f = blockIdx.y;
    const long long total = (long long)N * N;
    Y += (size_t)f * Mrows * N;
    RH += (size_t)f * N * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % N), j = (int)(e / N);     // RH(i, j) = conj(R(j, i))
        float2 v = make_float2(0.f, 0.f);
        if (full || j <= i) {
            const float2 r = Y[j + (size_t)i * Mrows];
            v = make_float2(r.x, -r.y);
        }
        RH[e] = v;
    }
}

// unit columns of Y (N x N per matrix); a zero column becomes e_j
__global__ void normalize_cols_kernel(int N, const float2 *Y, float2 *X, const int *perm)
{
    const int f = blockIdx.x;
    Y += (size_t)f * N * N;
    X += (size_t)f * N * N;
    if (perm) perm += (size_t)f * N;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = wid; j < N; j += nw) {
        const float2 *y = Y + (size_t)j * N;
        float a = 0.f;
        for (int r = lane; r < N; r += 32) a += y[r].x * y[r].x + y[r].y * y[r].y;
        a = warp_sum(a);
        const float inv = a > 0.f ? rsqrtf(a) : 0.f;
        for (int r = lane; r < N; r += 32)
            X[(perm ? perm[r] : r) + (size_t)j * N] =
                a > 0.f ? make_float2(y[r].x * inv, y[r].y * inv) : make_float2(r == j ? 1.f : 0.f, 0.f);
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

template <class T>
int apply_q_batched(ia_context *ctx, int rows, int cols, const T *Y, const T *tau, int ncol, const T *W, int ldw,
                    long long sW, T *X, long long sX, int batch)
{
    apply_q_kernel<T><<<batch, 256, 0, ctx->stream>>>(rows, cols, Y, tau, ncol, W, ldw, sW, X, sX);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}
template int apply_q_batched<float2>(ia_context *, int, int, const float2 *, const float2 *, int, const float2 *, int,
                                     long long, float2 *, long long, int);
template int apply_q_batched<double2>(ia_context *, int, int, const double2 *, const double2 *, int, const double2 *,
                                      int, long long, double2 *, long long, int);

__global__ void eig_backproject_kernel(int m, int n, int N, const double2 *H, int transposed, const double2 *X,
                                       int conj_u, const int *RANK, const double *S, const double2 *Z, int nrhs,
                                       double2 *Xout);

// Raug ((N + nrhs) x N) of the pivoted-QR solve: R^H (R: upper triangle of
// Y P = Q R) over the rows conj(v_r)^T, v_r = R P^T b_r, so that the
// one-sided Jacobi's column rotations J carry J^H v_r along.
__global__ void build_rh_aug_kernel(int N, int Mrows, int nrhs, const double2 *Y, const int *perm,
                                    const double2 *B, double2 *Rg)
{
    const int f = blockIdx.y;
    const int ld = N + nrhs;
    Y += (size_t)f * Mrows * N;
    Rg += (size_t)f * ld * N;
    perm += (size_t)f * N;
    const double2 *b = B + (size_t)f * nrhs * N;
    const long long total = (long long)N * N;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % N), j = (int)(e / N);     // R^H(i, j) = conj(R(j, i)), R upper
        double2 v = make_double2(0.0, 0.0);
        if (j <= i) {
            const double2 r = Y[j + (size_t)i * Mrows];
            v = make_double2(r.x, -r.y);
        }
        Rg[i + (size_t)j * ld] = v;
    }
    // v_r(i) = sum_{j >= i} R(i, j) b_r(perm[j]); the appended row holds conj(v_r)
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)nrhs * N;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % N), r = (int)(e / N);
        const double2 *br = b + (size_t)r * N;
        double2 acc = make_double2(0.0, 0.0);
        for (int j = i; j < N; ++j) zfma(acc, Y[i + (size_t)j * Mrows], br[perm[j]]);
        Rg[N + r + (size_t)i * ld] = make_double2(acc.x, -acc.y);
    }
}

// After the Jacobi on Raug: sigma_i = |column i of R^H J| (sorted, S), the
// rank of each column (RANK), beta = Sigma^-1 J^H v (sorted, BETA) and the
// left singular vectors U = P W, W = (R^H J) Sigma^-1, in the columns' own
// order (X, N x N).
__global__ void finalize_dv_kernel(int N, int nrhs, const double2 *Rg, const int *perm, double *S, double2 *BETA,
                                   double2 *X, int *RANK, int *info)
{
    extern __shared__ double sm_dv[];
    double *sig = sm_dv;
    const int f = blockIdx.x;
    const int ld = N + nrhs;
    Rg += (size_t)f * ld * N;
    perm += (size_t)f * N;
    X += (size_t)f * N * N;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = wid; j < N; j += nw) {
        double a = 0.0;
        for (int r = lane; r < N; r += 32) a += zabs2(Rg[r + (size_t)j * ld]);
        a = warp_sum(a);
        if (lane == 0) sig[j] = sqrt(a);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const double sj = sig[j];
        int rk = 0;
        for (int i = 0; i < N; ++i) {
            const double si = sig[i];
            if (si > sj || (si == sj && i < j)) rk++;
        }
        RANK[(size_t)f * N + j] = rk;
        S[(size_t)f * N + rk] = sj;
        if (info && (!(sj == sj) || isinf(sj))) atomicOr(&info[f], IA_INFO_NONFINITE);
        const double inv = sj > 0.0 ? 1.0 / sj : 0.0;
        for (int r = 0; r < nrhs; ++r) {
            const double2 v = Rg[N + r + (size_t)j * ld];
            BETA[((size_t)f * nrhs + r) * N + rk] = make_double2(v.x * inv, -v.y * inv);
        }
    }
    for (int j = wid; j < N; j += nw) {
        const double inv = sig[j] > 0.0 ? 1.0 / sig[j] : 0.0;
        for (int r = lane; r < N; r += 32) X[perm[r] + (size_t)j * N] = zscale(Rg[r + (size_t)j * ld], inv);
    }
}

size_t wide_solve_ws_bytes(int m, int n, int nrhs, int batch)
{
    const size_t F = batch, N = m, M = n, R = nrhs;
    return ws_round(16 * M * N * F) + ws_round(16 * N * F) + ws_round(16 * (N + R) * N * F) + ws_round(8 * N * F) +
           ws_round(16 * R * N * F) * 2 + ws_round(16 * N * N * F) + 2 * ws_round(4 * N * F) + 2048;
}

// FP64 wide solve (Drmac-Veselic preconditioned one-sided Jacobi):
// Y = A^H (n x m), column-pivoted Householder QR Y P = Q R, one-sided Jacobi
// on R^H (its columns converge to W Sigma with A = (P W) Sigma (Q J)^H): the
// pivoting grades R's rows, and Jacobi on R^H then needs 7-10 sweeps where
// the plain iteration on A^H needed 12-13 (and on a numerically
// rank-deficient operator, such as an order-15 spherical-harmonic expansion
// at low kr, did not settle within 40).  beta = U^H b rides along the
// rotations as the appended rows conj(R P^T b)^T; GCV / Tikhonov in FP64;
// x = A^H U (z / sigma) against the caller's A.
int wide_solve_batched(ia_context *ctx, int m, int n, int batch, const double2 *A, bool transposed, int nrhs,
                       const double2 *b, const ia_config *cfg, double2 *x, double *lambda, double *s_out, int *info,
                       WsCursor &cur)
{
    const int N = m, Mr = n;
    double2 *Y = cur.take<double2>((size_t)Mr * N * batch);
    double2 *tau = cur.take<double2>((size_t)N * batch);
    double2 *Rg = cur.take<double2>((size_t)(N + nrhs) * N * batch);
    double *s = s_out ? s_out : cur.take<double>((size_t)N * batch);
    double2 *beta = cur.take<double2>((size_t)nrhs * N * batch);
    double2 *z = cur.take<double2>((size_t)nrhs * N * batch);
    double2 *X = cur.take<double2>((size_t)N * N * batch);
    int *perm = cur.take<int>((size_t)N * batch);
    int *rank = cur.take<int>((size_t)N * batch);
    if (cur.off > cur.cap) return IA_ERR_TOO_LARGE;   // the carve would run past the caller's scratch
    const long long sA = (long long)m * n;
    int st;
    // Y = A^H
    if (transposed) st = zcopy2d_batched(ctx, n, m, A, n, sA, Y, Mr, (long long)Mr * N, true, batch);
    else st = ztranspose_batched(ctx, m, n, A, m, sA, Y, Mr, (long long)Mr * N, true, batch);
    if (st) return st;
    if ((st = qr_launch<double2>(ctx, Mr, N, Y, Mr, (long long)Mr * N, tau, 0, nullptr, 0, 0, batch, perm)))
        return st;
    {
        long long total = (long long)N * N;
        int blocks = (int)((total + 255) / 256);
        if (blocks > 512) blocks = 512;
        build_rh_aug_kernel<<<dim3(blocks, batch), 256, 0, ctx->stream>>>(N, Mr, nrhs, Y, perm, b, Rg);
        IA_LAUNCH_CHECK(ctx);
    }
    st = jacobi_rows_batched<double2>(ctx, N + nrhs, N, N, Rg, nullptr, batch, cfg->svd_max_sweeps, info);
    if (st) return st;
    finalize_dv_kernel<<<batch, 256, (size_t)N * sizeof(double), ctx->stream>>>(N, nrhs, Rg, perm, s, beta, X, rank,
                                                                                 info);
    IA_LAUNCH_CHECK(ctx);
    st = gcv_beta_batched(ctx, m, N, batch, s, nrhs, beta, nullptr, cfg, z, lambda);
    if (st) return st;
    const size_t smem = sizeof(double2) * ((size_t)N + (size_t)m);
    eig_backproject_kernel<<<dim3(batch, nrhs), 256, smem, ctx->stream>>>(m, n, N, A, transposed ? 1 : 0, X, 0, rank,
                                                                         s, z, nrhs, x);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// --------------------------------------------------------------------------
// mixed path: FP32 start, FP64-accurate finish in data space.
//
// H H^H = U S^2 U^H (m x m) holds everything GCV and Tikhonov need:
//   beta = U^H b, s, and x = V diag(phi) beta = H^H U diag(phi/s) beta.
// 1. FP32: Y = H^H = Q R, one-sided Jacobi R J = U_R S with J accumulated;
//    J approximates U.
// 2. E = H H^H in FP64.
// 3. Eigen-refinement of E from X = J (Ogita & Aishima 2018, Hermitian form):
//      R = I - X^H X, S = X^H E X, lambda_i = S_ii / (1 - R_ii),
//      F_ij = (S_ij + lambda_j R_ij) / (lambda_j - lambda_i)  (separated pairs)
//      F_ij = R_ij / 2                                         (clustered pairs,
//             |lambda_i - lambda_j| <= 2 (||S - diag(lambda)|| + max|lambda| ||R||))
//      X <- X (I + F)
//    E X and X^H (E X) in FP64, X^H X and X F in double-float; each step
//    squares the error of X.
// 4. s = sqrt(lambda) sorted, beta = U^H b, GCV in FP64, x = H^H U (phi/s .* beta).
// For H given as H^T, E is formed as (H^T)^H H^T = conj(H H^H), whose
// eigenvectors are conj(U).
// --------------------------------------------------------------------------
constexpr int OA_THREADS = 256;

__global__ void __launch_bounds__(OA_THREADS) oa_update_kernel(int N, const double2 *S, const double2 *Rm,
                                                                 double2 *Fc, double *LAM)
{
    __shared__ double red[2][OA_THREADS / 32];
    __shared__ double s_delta;
    extern __shared__ double lam[];   // N
    const int f = blockIdx.x;
    const size_t off = (size_t)f * N * N;
    S += off;
    Rm += off;
    Fc += off;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    for (int i = tid; i < N; i += blockDim.x) {
        double l = S[i + (size_t)i * N].x / Rm[i + (size_t)i * N].x;
        lam[i] = l;
        LAM[(size_t)f * N + i] = l;
    }
    __syncthreads();
    double so = 0.0, ro = 0.0;
    for (int e = tid; e < N * N; e += blockDim.x) {
        int i = e % N, j = e / N;
        double2 sv = S[e], rv = Rm[e];
        if (i == j) {
            sv.x -= lam[i];
            rv.x = 1.0 - rv.x;
            rv.y = -rv.y;
        } else {
            rv.x = -rv.x;
            rv.y = -rv.y;
        }
        so += zabs2(sv);
        ro += zabs2(rv);
    }
    so = warp_sum(so);
    ro = warp_sum(ro);
    if (lane == 0) { red[0][wid] = so; red[1][wid] = ro; }
    __syncthreads();
    if (tid == 0) {
        double a = 0.0, b = 0.0, lmax = 0.0;
        for (int w = 0; w < nw; ++w) { a += red[0][w]; b += red[1][w]; }
        for (int i = 0; i < N; ++i) lmax = fmax(lmax, fabs(lam[i]));
        s_delta = 2.0 * (sqrt(a) + lmax * sqrt(b));
    }
    __syncthreads();
    const double delta = s_delta;
    for (int e = tid; e < N * N; e += blockDim.x) {
        int i = e % N, j = e / N;
        double2 r = Rm[e];
        double2 R = (i == j) ? make_double2(1.0 - r.x, -r.y) : make_double2(-r.x, -r.y);
        double2 v;
        double gap = lam[j] - lam[i];
        if (i != j && fabs(gap) > delta) {
            double2 num = zadd(S[e], zscale(R, lam[j]));
            v = zscale(num, 1.0 / gap);
        } else {
            v = zscale(R, 0.5);
        }
        Fc[e] = v;
    }
}

// Two-sided FP64 Jacobi on the projected matrix S = X^H E X (N x N Hermitian,
// nearly diagonal after the refinement steps), one CTA per frequency, S in
// global memory, the rotations applied to the columns of X as well.  Only
// pairs coupled above the rounding level of S (|S_ij| > 2 N eps
// max|S_ii|) rotate, so the cost follows the clustered pairs the first-order
// refinement cannot separate (near-degenerate eigenvalues of symmetric
// geometries).  Round-robin ordering: in a round the pairs are disjoint, their
// rotations are computed from the current S, then applied to all pair columns,
// then to all pair rows (left and right rotations commute).  The rotation
//   G = [[c, s e], [-s conj(e), c]],  e = S_ij/|S_ij|,  t = tan(theta) from
//   zeta = (S_jj - S_ii) / (2 |S_ij|)   (Rutishauser's stable form)
// zeroes S_ij; S <- G^H S G on the pair, X <- X G.  LAM <- diag(S).
// Each sweep first checks every pair at once and runs only the rounds that
// hold a coupled pair; a round's rotations are applied with every (pair,
// matrix, row) and (pair, column) update spread over the whole CTA, one round
// of memory latency per phase.  (Applied warp per pair, with the global-memory
// updates in sequence while the other warps waited at the barrier, the kernel
// stalled on barriers: 68 cycles per issue.)
// Pairs whose two diagonal entries both lie below the Gram floor N eps
// max|S_ii| (half of tol) do not rotate: eigenvalues there are not resolved
// by a Gram matrix and are reported at the floor (eig_beta_kernel), so all
// such components get the same filter factor and enter the solution only as
// a subspace, which rotations inside it leave unchanged.  On operators
// spanning many decades (an order-15 spherical-harmonic expansion at low kr)
// that noise-level block holds most of the coupled pairs.
constexpr int HJ_THREADS = 512;

__device__ __forceinline__ void hj_pair(int N2, int round, int k, int &i, int &j)
{
    if (k == 0) {
        i = round;
        j = N2 - 1;
    } else {
        // (round + k) mod (N2 - 1) and (round - k + N2 - 1) mod (N2 - 1):
        // both operands lie in [0, 2 (N2 - 1)), so one conditional
        // subtraction replaces the integer division
        i = round + k;
        if (i >= N2 - 1) i -= N2 - 1;
        j = round - k + N2 - 1;
        if (j >= N2 - 1) j -= N2 - 1;
    }
    if (i > j) { int t = i; i = j; j = t; }
}

// SM: S (N <= 120) held in shared memory for the whole run, read from
// global memory once (its final state is not needed: LAM and X are the
// results); the pair slots and round flags then take 16- and 8-bit types and
// the diagonal is read from S directly, so that S fits beside them.
template <bool SM>
__global__ void __launch_bounds__(HJ_THREADS) herm_jacobi_kernel(int N, double2 *Sg, double2 *X, double *LAM,
                                                                  int max_sweeps, int *info)
{
    typedef typename std::conditional<SM, unsigned short, int>::type PIdx;
    typedef typename std::conditional<SM, unsigned char, int>::type RFlag;
    extern __shared__ __align__(16) double hj_sm[];
    const int N2 = N + (N & 1), P = N2 / 2;
    double2 *S = SM ? reinterpret_cast<double2 *>(hj_sm) : Sg;          // SM: N x N
    double *cs = hj_sm + (SM ? 2 * (size_t)N * N : 0);   // P
    double2 *se = reinterpret_cast<double2 *>(cs + P + (P & 1));   // P, 16-byte aligned
    PIdx *pi = reinterpret_cast<PIdx *>(se + P);          // P
    PIdx *pj = pi + P;                                    // P
    RFlag *rflag = reinterpret_cast<RFlag *>(pj + P);     // N2 - 1: rounds with a coupled pair
    __shared__ double red[HJ_THREADS / 32];
    __shared__ int s_rot;
    __shared__ int s_nact;   // rotating pairs of the current round (cs, se, pi, pj slots)
    const int f = blockIdx.x;
    Sg += (size_t)f * N * N;
    if (!SM) S = Sg;
    X += (size_t)f * N * N;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    if (SM) {
        for (int e = tid; e < N * N; e += blockDim.x) S[e] = Sg[e];
        __syncthreads();
    }
    double lm = 0.0;
    for (int i = tid; i < N; i += blockDim.x) lm = fmax(lm, fabs(S[i + (size_t)i * N].x));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lm = fmax(lm, __shfl_xor_sync(0xffffffffu, lm, o));
    if (lane == 0) red[wid] = lm;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; ++w) t = fmax(t, red[w]);
        red[0] = t;
    }
    __syncthreads();
    const double tol = 2.0 * (double)N * 2.220446049250313e-16 * red[0];
    const double floor2 = 0.5 * tol;
    // N: diag(S) at the sweep's start, after rflag's N2 ints (N2 even: 8-byte
    // aligned); with S in shared memory the diagonal is read from S
    double *dg = SM ? nullptr : reinterpret_cast<double *>(rflag + N2);
    auto diag = [&](int i) { return SM ? S[i + (size_t)i * N].x : dg[i]; };
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        // every pair of the sweep checked at once (independent loads): only
        // rounds holding a pair above tol run; couplings that rotations of
        // this sweep raise in skipped rounds are met by the next sweep's check,
        // and a converged S costs one pass instead of N2 - 1 serial rounds
        for (int r = tid; r < N2 - 1; r += blockDim.x) rflag[r] = 0;
        if (!SM)
            for (int i = tid; i < N; i += blockDim.x) dg[i] = S[i + (size_t)i * N].x;
        if (tid == 0) {
            s_rot = 0;
            s_nact = 0;
        }
        __syncthreads();
        for (int e = tid; e < (N2 - 1) * P; e += blockDim.x) {
            const int round = e / P, k = e - round * P;
            int i, j;
            hj_pair(N2, round, k, i, j);
            if (j >= N) continue;
            if (diag(i) < floor2 && diag(j) < floor2) continue;
            const double2 s = S[i + (size_t)j * N];
            if (sqrt(s.x * s.x + s.y * s.y) > tol) rflag[round] = 1;
        }
        __syncthreads();
        for (int round = 0; round < N2 - 1; ++round) {
            if (!rflag[round]) continue;
            int mine = 0;
            for (int k = tid; k < P; k += blockDim.x) {
                int i, j;
                hj_pair(N2, round, k, i, j);
                if (j >= N) continue;
                const double2 s = S[i + (size_t)j * N];
                const double g = sqrt(s.x * s.x + s.y * s.y);
                if (!(g > tol)) continue;
                const double a = S[i + (size_t)i * N].x, b = S[j + (size_t)j * N].x;
                if (a < floor2 && b < floor2) continue;
                const double zeta = (b - a) / (2.0 * g);
                const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / sqrt(1.0 + t * t);
                const double sn = t * c;
                const int slot = atomicAdd(&s_nact, 1);
                cs[slot] = c;
                se[slot] = make_double2(sn * s.x / g, sn * s.y / g);   // s e
                pi[slot] = (PIdx)i;
                pj[slot] = (PIdx)j;
                ++mine;
            }
            if (mine) atomicAdd(&s_rot, mine);
            // a round without rotations skips both apply phases and their barriers
            if (!__syncthreads_or(mine)) continue;
            const int nact = s_nact;
            // the round's pairs are disjoint: every (pair, matrix, row) of the
            // column phase and every (pair, column) of the row phase is an
            // independent update, spread over the whole CTA
            // columns of S and X: [u v] <- [u v] G
            for (int e = tid; e < nact * 2 * N; e += blockDim.x) {
                const int q = e / (2 * N), rem = e - q * 2 * N, mat = rem / N, r = rem - mat * N;
                const int i = pi[q], j = pj[q];
                const double c = cs[q];
                const double2 w = se[q];
                double2 *M = mat == 0 ? S : X;
                double2 *ci = M + (size_t)i * N, *cj = M + (size_t)j * N;
                const double2 u = ci[r], v = cj[r];
                double2 nu = zscale(u, c), nv = zscale(v, c);
                zfms(nu, zconj(w), v);                 // c u - conj(s e) v
                zfma(nv, w, u);                        // c v + s e u
                ci[r] = nu;
                cj[r] = nv;
            }
            __syncthreads();
            if (tid == 0) s_nact = 0;                  // every thread has read it
            // rows of S: [u; v] <- G^H [u; v]
            for (int e = tid; e < nact * N; e += blockDim.x) {
                const int q = e / N, col = e - q * N;
                const int i = pi[q], j = pj[q];
                const double c = cs[q];
                const double2 w = se[q];
                double2 *a = S + i + (size_t)col * N, *b = S + j + (size_t)col * N;
                const double2 u = *a, v = *b;
                double2 nu = zscale(u, c), nv = zscale(v, c);
                zfms(nu, w, v);                            // c u - s e v
                zfma(nv, zconj(w), u);                     // c v + conj(s e) u
                *a = nu;
                *b = nv;
            }
            __syncthreads();
        }
        const int total = s_rot;
        __syncthreads();
        if (total == 0) break;
    }
    if (tid == 0 && sweep >= max_sweeps && info) atomicOr(&info[f], IA_INFO_NOCONV);
    for (int i = tid; i < N; i += blockDim.x) LAM[(size_t)f * N + i] = S[i + (size_t)i * N].x;
}

// s (sorted descending), beta = U^H b (sorted like s), rank of every column;
// U = X, or conj(X) when conj_u.  Eigenvalues of the FP64 E = H H^H carry an
// absolute error ~ N eps lambda_max, so singular values below
// sqrt(N eps) s_1 are not resolved by this path: they are reported at that
// floor (an exact 0 would otherwise extend the GCV grid, whose lower end is
// max(s_p, 16 eps s_1), into a spurious lambda -> 0 minimum).  Filter factors
// of such components are below (floor / lambda)^2 for any useful lambda.
__global__ void eig_beta_kernel(int m, int N, const double *LAM, const double2 *X, int conj_u, int nrhs,
                                const double2 *Bv, double *S, double2 *BETA, int *RANK)
{
    __shared__ double red[32];
    const int f = blockIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    LAM += (size_t)f * N;
    X += (size_t)f * N * N;
    double lm = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) lm = fmax(lm, LAM[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lm = fmax(lm, __shfl_xor_sync(0xffffffffu, lm, o));
    if (lane == 0) red[wid] = lm;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < nw; ++w) t = fmax(t, red[w]);
        red[0] = t;
    }
    __syncthreads();
    const double floor2 = (double)N * 2.220446049250313e-16 * red[0];
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double li = LAM[i];
        int rk = 0;
        for (int j = 0; j < N; ++j) {
            double lj = LAM[j];
            if (lj > li || (lj == li && j < i)) rk++;
        }
        RANK[(size_t)f * N + i] = rk;
        S[(size_t)f * N + rk] = sqrt(fmax(li, floor2));
    }
    __syncthreads();
    for (int r = 0; r < nrhs; ++r) {
        const double2 *b = Bv + ((size_t)f * nrhs + r) * m;
        for (int i = wid; i < N; i += nw) {
            double2 acc = make_double2(0.0, 0.0);
            const double2 *xc = X + (size_t)i * N;
            for (int j = lane; j < m; j += 32) {
                if (conj_u) zfma(acc, xc[j], b[j]);       // conj(conj(X)) b
                else zcfma(acc, xc[j], b[j]);
            }
            acc = warp_sum2(acc);
            if (lane == 0) BETA[((size_t)f * nrhs + r) * N + RANK[(size_t)f * N + i]] = acc;
        }
    }
}

// x = H^H U (z / s), one CTA per (frequency, right-hand side)
__global__ void eig_backproject_kernel(int m, int n, int N, const double2 *H, int transposed, const double2 *X,
                                       int conj_u, const int *RANK, const double *S, const double2 *Z, int nrhs,
                                       double2 *Xout)
{
    extern __shared__ double2 smw[];
    double2 *coef = smw;       // N, original column order
    double2 *w = smw + N;      // m
    const int f = blockIdx.x, rr = blockIdx.y;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    X += (size_t)f * N * N;
    H += (size_t)f * m * n;
    const double2 *z = Z + ((size_t)f * nrhs + rr) * N;
    for (int i = tid; i < N; i += blockDim.x) {
        int rk = RANK[(size_t)f * N + i];
        double s = S[(size_t)f * N + rk];
        coef[i] = s > 0.0 ? zscale(z[rk], 1.0 / s) : make_double2(0.0, 0.0);
    }
    __syncthreads();
    for (int j = tid; j < m; j += blockDim.x) {
        double2 acc = make_double2(0.0, 0.0);
        for (int i = 0; i < N; ++i) {
            double2 u = X[j + (size_t)i * N];
            if (conj_u) u.y = -u.y;
            zfma(acc, u, coef[i]);
        }
        w[j] = acc;
    }
    __syncthreads();
    double2 *x = Xout + ((size_t)f * nrhs + rr) * n;
    if (transposed) {
        for (int k = tid; k < n; k += blockDim.x) {
            double2 acc = make_double2(0.0, 0.0);
            for (int j = 0; j < m; ++j) zcfma(acc, H[k + (size_t)j * n], w[j]);
            x[k] = acc;
        }
    } else {
        for (int k = wid; k < n; k += nw) {
            double2 acc = make_double2(0.0, 0.0);
            const double2 *col = H + (size_t)k * m;
            for (int j = lane; j < m; j += 32) zcfma(acc, col[j], w[j]);
            acc = warp_sum2(acc);
            if (lane == 0) x[k] = acc;
        }
    }
}

// FP64-level products of the mixed eigensolver (E = H H^H and the
// Ogita-Aishima / Newton-Schulz products): the tensor-core GEMM on 8 BF16
// slices when cfg->gemm_slices turns the tensor cores on and the product's K
// keeps the slice sums exact (K <= 1024 at 8 slices), else the double-float
// CUDA-core GEMM.  E's error reaches x as |dE| / lambda^2, so these products
// take 8 slices (bound 1.4e-13 of the row and column maxima per term) whatever
// the transfer uses.  The slice planes of both operands live in one scratch
// region that each product reuses (products run in stream order).
constexpr int EIG_SLICES = 8;

static bool eig_tc(const ia_config *cfg, int K)
{
    return cfg->gemm_slices >= TC_SLICES_MIN && cfg->gemm_slices <= TC_SLICES_MAX &&
           (long long)EIG_SLICES * 1024 * ((2 * K + 7) & ~7) <= (1ll << 24);
}

static size_t eig_gemm_ws_bytes(int N, int K, int batch)
{
    return tc_planes_bytes(N, K, EIG_SLICES, false, batch) + tc_planes_bytes(N, K, EIG_SLICES, true, batch) + 1024;
}

struct EigGemm {
    ia_context *ctx;
    const ia_config *cfg;
    char *ws;
    size_t bytes;
    int *info;
    int operator()(Op opa, Op opb, int M, int N, int K, double alpha, const double2 *A, int lda, long long sA,
                   const double2 *B, int ldb, long long sB, double beta, double2 *C, int ldc, long long sC,
                   int batch) const
    {
        if (!eig_tc(cfg, K))
            return dfgemm_batched(ctx, opa, opb, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch);
        WsCursor cur{ws, 0, bytes};
        TcPlanes Pa{}, Pb{};
        int st = tc_slice_pair(ctx, opa, A, lda, sA, M, opb, B, ldb, sB, N, K, EIG_SLICES, batch, Pa, Pb, cur);
        if (!st) st = tc_gemm(ctx, Pa, Pb, M, N, alpha, beta, C, ldc, sC, batch, info);
        return st;
    }
};

// CTAs per bin of the statistics pass (bin_stats_kernel)
constexpr int BIN_STAT_BLOCKS = 16;

static size_t gram_eig_mixed_ws_bytes(int m, int n, int batch)
{
    const size_t F = batch, N = m, M = n;
    return ws_round(16 * M * N * F) + ws_round(8 * M * N * F) + ws_round(8 * N * F) + 2 * ws_round(8 * N * N * F) +
           7 * ws_round(16 * N * N * F) + ws_round(8 * N * F) + ws_round(4 * N * F) + ws_round(16 * M * N * F) +
           ws_round(4 * F) + ws_round(8 * F) + 2 * ws_round(8 * (size_t)BIN_STAT_BLOCKS * F) +
           eig_gemm_ws_bytes(m, n > m ? n : m, batch) + 4096;
}

// Range of the FP32 and double-float stages.  Their high words are FP32, so
// |A| above ~1e19 overflows the Gram matrix and the column norms (an
// order-15 spherical-harmonic operator reaches 1e30 at kr = 0.14).  Those
// stages work on A 2^-e_f, e_f per bin with max(|Re|, |Im|) < 2^e_f; a power
// of two commutes with every rounding, so the scaled run is the unscaled one
// times 2^-e_f (bitwise, wherever the unscaled one stays in range).  The
// eigenvalues come back multiplied by 4^e_f; everything after (s, beta, GCV,
// x) works on the caller's A in FP64.
// Per-bin statistics of A in one pass over all SMs: BIN_STAT_BLOCKS CTAs per
// bin, each over a contiguous chunk, write the chunk's largest |Re|, |Im| (as
// an order-preserving key) and its sum of |a|^2; bin_stats_finish_kernel
// combines the chunks in chunk order (deterministic) into the exponent e_f
// with max(|Re|, |Im|) < 2^e_f and ||A_f||_F^2.

__global__ void bin_stats_kernel(size_t count, const double2 *__restrict__ A, unsigned long long *__restrict__ keys,
                                 double *__restrict__ sums)
{
    __shared__ unsigned long long s_key[8];
    __shared__ double s_sum[8];
    const int f = blockIdx.y, c = blockIdx.x;
    const size_t chunk = (count + BIN_STAT_BLOCKS - 1) / BIN_STAT_BLOCKS;
    const size_t e0 = (size_t)c * chunk, e1 = e0 + chunk < count ? e0 + chunk : count;
    A += (size_t)f * count;
    unsigned long long key = 0ull;
    double sum = 0.0;
    for (size_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
        const double2 v = A[e];
        const unsigned long long a = __double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFull;
        const unsigned long long b = __double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFull;
        key = a > key ? a : key;
        key = b > key ? b : key;
        sum += v.x * v.x + v.y * v.y;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long k2 = __shfl_xor_sync(0xffffffffu, key, o);
        key = k2 > key ? k2 : key;
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        s_key[wid] = key;
        s_sum[wid] = sum;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            key = s_key[w] > key ? s_key[w] : key;
            sum += s_sum[w];
        }
        keys[(size_t)f * BIN_STAT_BLOCKS + c] = key;
        sums[(size_t)f * BIN_STAT_BLOCKS + c] = sum;
    }
}

__global__ void bin_stats_finish_kernel(int F, const unsigned long long *__restrict__ keys,
                                        const double *__restrict__ sums, int *__restrict__ ex, double *__restrict__ fro2)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    unsigned long long k = 0ull;
    double sum = 0.0;
    for (int c = 0; c < BIN_STAT_BLOCKS; ++c) {
        const unsigned long long kc = keys[(size_t)f * BIN_STAT_BLOCKS + c];
        k = kc > k ? kc : k;
        sum += sums[(size_t)f * BIN_STAT_BLOCKS + c];
    }
    // exponent of the largest magnitude (non-finite input keeps e = 0 and
    // surfaces downstream as IA_INFO_NONFINITE or in the guard's trace check)
    ex[f] = (k && k < 0x7FF0000000000000ull) ? (int)(k >> 52) - 1022 : 0;
    fro2[f] = sum;
}

__global__ void scale_bins_kernel(size_t count, const double2 *__restrict__ A, const int *__restrict__ ex,
                                  double2 *__restrict__ As)
{
    const int f = blockIdx.y;
    const double sc = ldexp(1.0, -ex[f]);
    A += (size_t)f * count;
    As += (size_t)f * count;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        const double2 v = A[e];
        As[e] = make_double2(v.x * sc, v.y * sc);
    }
}

__global__ void unscale_eig_kernel(int N, double *__restrict__ lam, const int *__restrict__ ex)
{
    const int f = blockIdx.x;
    const double sc = ldexp(1.0, 2 * ex[f]);
    for (int i = threadIdx.x; i < N; i += blockDim.x) lam[(size_t)f * N + i] *= sc;
}

size_t wide_solve_mixed_ws_bytes(int m, int n, int nrhs, int batch)
{
    const size_t F = batch, N = m, R = nrhs;
    return gram_eig_mixed_ws_bytes(m, n, batch) + ws_round(8 * N * F) + ws_round(4 * N * F) +
           2 * ws_round(16 * R * N * F) + ws_round(8 * R * F) + 4096;
}

// Steps 1-4 of the mixed solve: eigenvectors X (m x m, columns in no
// particular order) and eigenvalues lam_e (m) of E = A A^H for A (m x n,
// column-major), or of conj(E) for the transposed input (A^T stored, n x m):
// FP32 QR (n > m) and one-sided Jacobi, double-float E and Ogita-Aishima steps,
// Newton-Schulz, FP64 S = X^H E X and the two-sided Jacobi on its coupled
// pairs.  *Xout and *lam_out point into the workspace taken from cur.
static int gram_eig_mixed(ia_context *ctx, int m, int n, int batch, const double2 *A, bool transposed,
                          const ia_config *cfg, double2 **Xout, double **lam_out, double **fro2_out, int *info,
                          WsCursor &cur)
{
    const int N = m, Mr = n;
    const bool qr = n > m;
    const size_t NN = (size_t)N * N;
    double2 *Yd = transposed ? nullptr : cur.take<double2>((size_t)Mr * N * batch);
    float2 *Y = cur.take<float2>((size_t)Mr * N * batch);
    float2 *tau = cur.take<float2>((size_t)N * batch);
    float2 *R32 = cur.take<float2>(NN * batch);
    float2 *J32 = cur.take<float2>(NN * batch);
    double2 *E = cur.take<double2>(NN * batch);
    double2 *X = cur.take<double2>(NN * batch);
    double2 *Xn = cur.take<double2>(NN * batch);
    double2 *T1 = cur.take<double2>(NN * batch);
    double2 *Sm = cur.take<double2>(NN * batch);
    double2 *Rm = cur.take<double2>(NN * batch);
    double2 *Fc = cur.take<double2>(NN * batch);
    double *lam_e = cur.take<double>((size_t)N * batch);
    int *perm = qr ? cur.take<int>((size_t)N * batch) : nullptr;
    double2 *As = cur.take<double2>((size_t)m * n * batch);
    int *ex = cur.take<int>((size_t)batch);
    double *fro2 = cur.take<double>((size_t)batch);
    unsigned long long *keys = cur.take<unsigned long long>((size_t)BIN_STAT_BLOCKS * batch);
    double *sums = cur.take<double>((size_t)BIN_STAT_BLOCKS * batch);
    const size_t eg_bytes = eig_gemm_ws_bytes(N, n > m ? n : m, batch);
    const EigGemm eg{ctx, cfg, cur.take<char>(eg_bytes), eg_bytes, info};
    if (cur.off > cur.cap) return IA_ERR_ALLOC;
    const long long sA = (long long)m * n, sY = (long long)Mr * N, sN = (long long)NN;
    int st;
    // the FP32 and double-float stages (1-3) work on A 2^-e_f
    bin_stats_kernel<<<dim3(BIN_STAT_BLOCKS, batch), 256, 0, ctx->stream>>>((size_t)sA, A, keys, sums);
    IA_LAUNCH_CHECK(ctx);
    bin_stats_finish_kernel<<<(batch + 127) / 128, 128, 0, ctx->stream>>>(batch, keys, sums, ex, fro2);
    IA_LAUNCH_CHECK(ctx);
    *fro2_out = fro2;
    {
        int blocks = (int)((sA + 255) / 256);
        if (blocks > 256) blocks = 256;
        scale_bins_kernel<<<dim3(blocks, batch), 256, 0, ctx->stream>>>((size_t)sA, A, ex, As);
        IA_LAUNCH_CHECK(ctx);
    }
    A = As;
    // 1. FP32 start: Y = H^H, QR with column pivoting (Y P = Q R), one-sided
    // Jacobi on R^H.  Pivoting orders R's diagonal by decreasing size, which
    // cuts the Jacobi's sweeps from 12-13 to 7-8 on the bench's transfer
    // matrices (Drmac-Veselic preconditioning); H H^H = P R^H R P^T, so the
    // Jacobi's vectors come back through P.
    if (transposed) {
        st = copy2d_batched<double2, float2>(ctx, n, m, A, n, sA, Y, Mr, sY, true, batch);
    } else {
        st = ztranspose_batched(ctx, m, n, A, m, sA, Yd, Mr, sY, true, batch);
        if (!st) st = copy2d_batched<double2, float2>(ctx, Mr, N, Yd, Mr, sY, Y, Mr, sY, false, batch);
    }
    if (st) return st;
    if (qr && (st = qr_launch<float2>(ctx, Mr, N, Y, Mr, sY, tau, 0, nullptr, 0, 0, batch, perm))) return st;
    {
        long long total = (long long)N * N;
        int blocks = (int)((total + 255) / 256);
        if (blocks > 512) blocks = 512;
        build_rh_kernel<<<dim3(blocks, batch), 256, 0, ctx->stream>>>(N, Mr, Y, qr ? 0 : 1, R32);
        IA_LAUNCH_CHECK(ctx);
    }
    // one-sided Jacobi on R^H: its columns end as U_E diag(sigma) with E = R^H R
    // = H H^H, so no rotation accumulator is needed
    st = jacobi_rows_batched<float2>(ctx, N, N, N, R32, nullptr, batch, cfg->svd_max_sweeps, info);
    if (st) return st;
    normalize_cols_kernel<<<batch, 256, 0, ctx->stream>>>(N, R32, J32, perm);
    IA_LAUNCH_CHECK(ctx);
    // 2. E = H H^H (or its conjugate for H^T input) at FP64 level (EigGemm):
    // H reaches this path from the mixed transfer (~1e-11 relative), so an
    // FP64 product would not make E more accurate.
    if (transposed) st = eg(OP_C, OP_N, N, N, n, 1.0, A, n, sA, A, n, sA, 0.0, E, N, sN, batch);
    else st = eg(OP_N, OP_C, N, N, n, 1.0, A, m, sA, A, m, sA, 0.0, E, N, sN, batch);
    if (st) return st;
    // 3. eigen-refinement from X = J (conj(J) for H^T input)
    if ((st = copy2d_batched<float2, double2>(ctx, N, N, J32, N, sN, X, N, sN, transposed, batch))) return st;
    // the FP32 Jacobi leaves X accurate to ~1e-5 (its stopping threshold sits
    // above FP32 rounding noise); the quadratic steps reach the double-float
    // level of their products, and step 4's FP64 S = X^H E X with the
    // two-sided Jacobi finishes at FP64 level.  Two steps: emulated on the
    // bench's transfer matrices they leave 27-143 pairs coupled above that
    // Jacobi's threshold and three steps 0-6, but the third step's four
    // double-float products cost more than the Jacobi sweeps they save
    // (measured 14.3 -> 14.9 ms per 64-bin solve).
    const int steps = cfg->refine_steps > 2 ? cfg->refine_steps : 2;
    for (int it = 0; it < steps; ++it) {
        if ((st = eg(OP_N, OP_N, N, N, N, 1.0, E, N, sN, X, N, sN, 0.0, T1, N, sN, batch))) return st;
        if ((st = eg(OP_C, OP_N, N, N, N, 1.0, X, N, sN, T1, N, sN, 0.0, Sm, N, sN, batch))) return st;
        if ((st = eg(OP_C, OP_N, N, N, N, 1.0, X, N, sN, X, N, sN, 0.0, Rm, N, sN, batch))) return st;
        oa_update_kernel<<<batch, OA_THREADS, sizeof(double) * (size_t)N, ctx->stream>>>(N, Sm, Rm, Fc, lam_e);
        IA_LAUNCH_CHECK(ctx);
        if ((st = zcopy2d_batched(ctx, N, N, X, N, sN, Xn, N, sN, false, batch))) return st;
        if ((st = eg(OP_N, OP_N, N, N, N, 1.0, X, N, sN, Fc, N, sN, 1.0, Xn, N, sN, batch))) return st;
        double2 *t = X;
        X = Xn;
        Xn = t;
    }
    // 4. pairs of near-equal eigenvalues stay coupled through the first-order
    // steps (the refinement treats them as a cluster): orthonormalise X
    // (Newton-Schulz, X <- 1.5 X - 0.5 X X^H X), form S = X^H E X at FP64
    // level (EigGemm; FP64 CUDA-core GEMMs cost 0.5 ms per 16 bins here) and
    // rotate the coupled pairs apart with two-sided Jacobi; lam_e <- diag(S).
    // Suited to spectra with few clusters (a transfer matrix's decaying
    // singular values): on a dense clustered spectrum (the radiation operator
    // of a sphere) the first-order steps stall and the Jacobi does a full sweep.
    if ((st = eg(OP_C, OP_N, N, N, N, 1.0, X, N, sN, X, N, sN, 0.0, Rm, N, sN, batch))) return st;
    if ((st = zcopy2d_batched(ctx, N, N, X, N, sN, Xn, N, sN, false, batch))) return st;
    if ((st = eg(OP_N, OP_N, N, N, N, -0.5, X, N, sN, Rm, N, sN, 1.5, Xn, N, sN, batch))) return st;
    {
        double2 *t = X;
        X = Xn;
        Xn = t;
    }
    if ((st = eg(OP_N, OP_N, N, N, N, 1.0, E, N, sN, X, N, sN, 0.0, T1, N, sN, batch))) return st;
    if ((st = eg(OP_C, OP_N, N, N, N, 1.0, X, N, sN, T1, N, sN, 0.0, Sm, N, sN, batch))) return st;
    if ((st = herm_jacobi_batched(ctx, N, Sm, X, lam_e, cfg->svd_max_sweeps < 16 ? cfg->svd_max_sweeps : 16, batch,
                                  info)))
        return st;
    unscale_eig_kernel<<<batch, 128, 0, ctx->stream>>>(N, lam_e, ex);
    IA_LAUNCH_CHECK(ctx);
    *Xout = X;
    *lam_out = lam_e;
    return IA_OK;
}

// Precision guard, one thread per bin: ||A_f||_F^2 (from the statistics pass)
// against sum s_i^2 (IA_INFO_UNRESOLVED), and the smallest regularisation
// level against s_1 (IA_INFO_PRECISION).  The
// mixed eigensolver reaches FP64-level eigenpairs of H H^H (errors ~eps
// s_1^2), so a Tikhonov solution is good to ~eps (s_1 / lambda)^2 and needs
// lambda well above sqrt(eps) s_1; below cfg->mixed_guard the bin is marked
// for the FP64 path.  A broken eigen-decomposition (an eigenvalue lost or
// doubled) shows in the trace.
__global__ void precision_guard_kernel(int F, const double *__restrict__ fro2, int p, const double *__restrict__ s,
                                       int nrhs, const double *__restrict__ lam, const double2 *__restrict__ beta,
                                       int method, int tsvd_k, double ratio, int *__restrict__ info)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= F) return;
    const double *sf = s + (size_t)f * p;
    double s2 = 0.0, s1 = 0.0, smin = INFINITY;
    for (int i = 0; i < p; ++i) {
        s2 += sf[i] * sf[i];
        s1 = fmax(s1, sf[i]);
        smin = fmin(smin, sf[i]);
    }
    // eig_beta_kernel reports the values a Gram matrix cannot resolve at
    // sqrt(N eps) s_1; "unresolved" here: at most twice that
    const double floor_s = sqrt((double)p * 2.220446049250313e-16) * s1;
    const bool reaches_floor = smin <= 10.0 * floor_s;
    double level;
    if (method == IA_METHOD_TSVD) {
        level = sf[tsvd_k - 1];
    } else {
        level = lam[(size_t)f * nrhs];
        for (int r = 1; r < nrhs; ++r) level = fmin(level, lam[(size_t)f * nrhs + r]);
    }
    const double a2 = fro2[f];
    // a successful decomposition meets the trace to ~1e-10 (X orthonormal to
    // that level after Newton-Schulz); a lost or doubled eigenpair shows at
    // 1e-8 and above
    if (!(a2 > 0.0 && a2 < INFINITY && fabs(s2 - a2) <= 1e-9 * a2)) {
        info[f] |= IA_INFO_UNRESOLVED;
        // more refinement steps can settle the eigenpairs of a spectrum that
        // reaches the floor, but not resolve the values below it
        if (reaches_floor) info[f] |= IA_INFO_PRECISION;
    }
    if (!(level >= ratio * s1)) info[f] |= IA_INFO_PRECISION;
    // GCV and the unresolved subspace: the data's energy per unresolved
    // component (their sum |beta|^2 is exact as a subspace quantity) against
    // the mean energy of the components the chosen lambda filters out.  Where
    // the unresolved components carry ten times that, they hold signal, and
    // the true GCV minimum may lie among the values the mixed path cannot
    // resolve (an order-15 spherical-harmonic operator at low kr: the mixed
    // GCV settles on a large-lambda local minimum, FP64's is 1e-11 s_1); where
    // they hold the noise level (the IBEM sphere at 30 dB) the choice stands.
    // A choice at the top of the grid (lambda ~ s_1: everything filtered)
    // over such a spectrum says only that no resolved level beats filtering
    // all; the comparison below is then empty, and the true minimum may lie
    // among the unresolved values (the order-15 HELS operator at kr 3.6:
    // mixed lambda = s_1, FP64's 3e-8 s_1), so that too goes to FP64.
    if (method != IA_METHOD_TSVD && reaches_floor) {
        for (int r = 0; r < nrhs; ++r) {
            const double lm = lam[(size_t)f * nrhs + r], l2 = lm * lm;
            if (lm >= 0.5 * s1) info[f] |= IA_INFO_PRECISION;
            const double2 *bt = beta + ((size_t)f * nrhs + r) * p;
            double bu = 0.0, num = 0.0, den = 0.0;
            int nu = 0;
            for (int i = 0; i < p; ++i) {
                const double b2 = bt[i].x * bt[i].x + bt[i].y * bt[i].y;
                if (sf[i] <= 2.0 * floor_s) {
                    bu += b2;
                    ++nu;
                } else {
                    const double fi = l2 / (sf[i] * sf[i] + l2);
                    num += fi * fi * b2;
                    den += fi;
                }
            }
            if (nu > 0 && den > 0.0 && bu / nu > 10.0 * (num / den)) info[f] |= IA_INFO_PRECISION;
        }
    }
}

int herm_jacobi_batched(ia_context *ctx, int N, double2 *S, double2 *X, double *LAM, int max_sweeps, int batch,
                        int *info)
{
    const int P = (N + (N & 1)) / 2, N2 = 2 * P;
    // S in shared memory when it fits beside the pair slots (N <= 120 with
    // 16-bit slot indices and 8-bit round flags): the device's per-CTA limit
    // less the kernel's static shared memory
    const size_t smem_s = sizeof(double2) * (size_t)N * N + sizeof(double) * (size_t)(P + (P & 1)) +
                          sizeof(double2) * P + 2 * sizeof(unsigned short) * P + (size_t)N2;
    static size_t smem_cap = 0;   // per process: one device type
    if (!smem_cap) {
        int optin = 0;
        cudaFuncAttributes fa{};
        if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device) == cudaSuccess &&
            cudaFuncGetAttributes(&fa, herm_jacobi_kernel<true>) == cudaSuccess && (size_t)optin > fa.sharedSizeBytes)
            smem_cap = (size_t)optin - fa.sharedSizeBytes;
        else
            smem_cap = 1;
    }
    if (smem_s <= smem_cap && N < 65536) {
        IA_CUDA_TRY(cudaFuncSetAttribute(herm_jacobi_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem_s));
        herm_jacobi_kernel<true><<<batch, HJ_THREADS, smem_s, ctx->stream>>>(N, S, X, LAM, max_sweeps, info);
        IA_LAUNCH_CHECK(ctx);
        return IA_OK;
    }
    const size_t smem = sizeof(double) * (size_t)(P + (P & 1)) + sizeof(double2) * P + 2 * sizeof(int) * P +
                        sizeof(int) * (size_t)N2 + sizeof(double) * (size_t)N;
    if (smem > 227 * 1024 - 512) return IA_ERR_TOO_LARGE;
    if (smem > 48 * 1024)
        IA_CUDA_TRY(cudaFuncSetAttribute(herm_jacobi_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
    herm_jacobi_kernel<false><<<batch, HJ_THREADS, smem, ctx->stream>>>(N, S, X, LAM, max_sweeps, info);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

int wide_solve_mixed_batched(ia_context *ctx, int m, int n, int batch, const double2 *A, bool transposed, int nrhs,
                             const double2 *b, const ia_config *cfg, double2 *x, double *lambda, double *s_out,
                             int *info, WsCursor &cur)
{
    const int N = m;
    double2 *X;
    double *lam_e;
    double *fro2;
    int st = gram_eig_mixed(ctx, m, n, batch, A, transposed, cfg, &X, &lam_e, &fro2, info, cur);
    if (st) return st;
    double *s = s_out ? s_out : cur.take<double>((size_t)N * batch);
    int *rank = cur.take<int>((size_t)N * batch);
    double2 *beta = cur.take<double2>((size_t)nrhs * N * batch);
    double2 *z = cur.take<double2>((size_t)nrhs * N * batch);
    double *lam = lambda ? lambda : cur.take<double>((size_t)nrhs * batch);
    // 5. s, beta, GCV, back-projection
    eig_beta_kernel<<<batch, 256, 0, ctx->stream>>>(m, N, lam_e, X, transposed ? 1 : 0, nrhs, b, s, beta, rank);
    IA_LAUNCH_CHECK(ctx);
    st = gcv_beta_batched(ctx, m, N, batch, s, nrhs, beta, nullptr, cfg, z, lam);
    if (st) return st;
    size_t smem = sizeof(double2) * ((size_t)N + (size_t)m);
    eig_backproject_kernel<<<dim3(batch, nrhs), 256, smem, ctx->stream>>>(m, n, N, A, transposed ? 1 : 0, X,
                                                                         transposed ? 1 : 0, rank, s, z, nrhs, x);
    IA_LAUNCH_CHECK(ctx);
    // 6. precision guard (IA_INFO_PRECISION for the FP64 fallback)
    precision_guard_kernel<<<(batch + 127) / 128, 128, 0, ctx->stream>>>(batch, fro2, N, s, nrhs, lam, beta,
                                                                         cfg->method, cfg->tsvd_k, cfg->mixed_guard,
                                                                         info);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

IA_BOUNDS_READER(bounds_read_wide)

}  // namespace ia
