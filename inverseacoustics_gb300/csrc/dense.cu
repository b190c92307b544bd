// Batched complex dense kernels: GEMM, LU with partial pivoting, triangular
// solves, transposes -- templated on the element type (double2 for the FP64
// path, float2 for the FP32 stages of the mixed path).  These replace the
// reference's cuBLAS / cuSOLVER / LAPACK calls on the hot path
// (cusolverDnZZgels CUDA/ibem.cuh:391, CUDA/esm.cuh:75; zgels_
// CUDA/ibem.cuh:755; cublasZgemm CUDA/ibem.cuh:398; cublasZgeam
// CUDA/esm.cuh:79).  Every launch covers the whole frequency batch (grid.z or
// grid.x = batch).
#include <type_traits>
#include "ia_common.cuh"
#include "ia_internal.h"
#include "tune.h"

namespace ia {

// --------------------------------------------------------------------------
// GEMM: C = alpha op(A) op(B) + beta C.  A BM x BN tile per CTA of 256
// threads, each thread a TM x TN block of outputs strided by BM/TM rows and
// BN/TN columns so shared-memory reads are conflict free; K in steps of 8
// (a step of 16 measured slower for the FP32 LU updates).
// Every variant sums k in the same order (0..K-1, one thread per output), so
// the autotuner's choice of tile does not change results.
// --------------------------------------------------------------------------
constexpr int GB_K = 8;

template <class T>
__device__ __forceinline__ T ld_op(const T *P, int ld, int r, int c, int R, int Cc, int op)
{
    // element (r, c) of op(P) where op(P) is R x Cc
    if (r >= R || c >= Cc) return ctraits<T>::make(0, 0);
    if (op == OP_N) return P[r + (size_t)c * ld];
    T v = P[c + (size_t)r * ld];
    if (op == OP_C) v.y = -v.y;
    return v;
}

template <class T, int BM, int BN, int TM, int TN>
__global__ void __launch_bounds__(256) gemm_kernel(int opa, int opb, int M, int N, int K, T alpha,
                                                   const T *__restrict__ A, int lda, long long sA,
                                                   const T *__restrict__ B, int ldb, long long sB, T beta,
                                                   T *__restrict__ C, int ldc, long long sC)
{
    constexpr int NTX = BN / TN, NTY = BM / TM;
    static_assert(NTX * NTY == 256, "256 threads per tile");
    constexpr int KC = GB_K;
    __shared__ T As[KC][BM];
    __shared__ T Bs[KC][BN];
    const int f = blockIdx.z;
    A += f * sA;
    B += f * sB;
    C += f * sC;
    const int tx = threadIdx.x % NTX, ty = threadIdx.x / NTX;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = ctraits<T>::make(0, 0);

    for (int k0 = 0; k0 < K; k0 += KC) {
#pragma unroll
        for (int e = threadIdx.x; e < KC * BM; e += 256) {
            int r, kk;
            if (opa == OP_N) { r = e % BM; kk = e / BM; }
            else { kk = e % KC; r = e / KC; }
            As[kk][r] = ld_op(A, lda, m0 + r, k0 + kk, M, K, opa);
        }
#pragma unroll
        for (int e = threadIdx.x; e < KC * BN; e += 256) {
            int kk, c;
            if (opb == OP_N) { kk = e % KC; c = e / KC; }
            else { c = e % BN; kk = e / BN; }
            Bs[kk][c] = ld_op(B, ldb, k0 + kk, n0 + c, K, N, opb);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < KC; ++kk) {
            T a[TM], b[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + NTY * i];
#pragma unroll
            for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + NTX * j];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) zfma(acc[i][j], a[i], b[j]);
        }
        __syncthreads();
    }
    const bool beta0 = (beta.x == 0 && beta.y == 0);
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        int r = m0 + ty + NTY * i;
        if (r >= M) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            int c = n0 + tx + NTX * j;
            if (c >= N) continue;
            T v = zmul(alpha, acc[i][j]);
            T *p = C + r + (size_t)c * ldc;
            if (!beta0) v = zadd(v, zmul(beta, *p));
            *p = v;
        }
    }
}

// Rank-K update for K <= GP_K with both operands untransposed (the blocked
// LU's A22 -= L21 U12 and the blocked solves' B -= L X): the whole A and B
// panels are staged once (one barrier instead of two per 8-wide K step, and
// every thread's global loads in flight together), B's rows padded by one
// element so the column-major panel stores are conflict free.  Same thread
// layout and the same k order per output as gemm_kernel: bitwise the same
// results.
constexpr int GP_K = 32;

template <class T, int BM, int BN, int TM, int TN>
__global__ void __launch_bounds__(256) gemm_nn_panel_kernel(int M, int N, int K, T alpha,
                                                            const T *__restrict__ A, int lda, long long sA,
                                                            const T *__restrict__ B, int ldb, long long sB, T beta,
                                                            T *__restrict__ C, int ldc, long long sC)
{
    constexpr int NTX = BN / TN, NTY = BM / TM;
    static_assert(NTX * NTY == 256, "256 threads per tile");
    __shared__ T As[GP_K][BM];
    __shared__ T Bs[GP_K][BN + 1];
    const int f = blockIdx.z;
    A += f * sA;
    B += f * sB;
    C += f * sC;
    const int tx = threadIdx.x % NTX, ty = threadIdx.x / NTX;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const T zero = ctraits<T>::make(0, 0);
#pragma unroll
    for (int e = threadIdx.x; e < GP_K * BM; e += 256) {
        const int r = e % BM, kk = e / BM;
        As[kk][r] = (m0 + r < M && kk < K) ? A[(m0 + r) + (size_t)kk * lda] : zero;
    }
#pragma unroll
    for (int e = threadIdx.x; e < GP_K * BN; e += 256) {
        const int kk = e % GP_K, c = e / GP_K;
        Bs[kk][c] = (n0 + c < N && kk < K) ? B[kk + (size_t)(n0 + c) * ldb] : zero;
    }
    __syncthreads();
    T acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = zero;
#pragma unroll 8
    for (int kk = 0; kk < K; ++kk) {
        T a[TM], b[TN];
#pragma unroll
        for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + NTY * i];
#pragma unroll
        for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + NTX * j];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j) zfma(acc[i][j], a[i], b[j]);
    }
    const bool beta0 = (beta.x == 0 && beta.y == 0);
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        int r = m0 + ty + NTY * i;
        if (r >= M) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            int c = n0 + tx + NTX * j;
            if (c >= N) continue;
            T v = zmul(alpha, acc[i][j]);
            T *p = C + r + (size_t)c * ldc;
            if (!beta0) v = zadd(v, zmul(beta, *p));
            *p = v;
        }
    }
}

template <class T, int BM, int BN, int TM, int TN>
static int gemm_launch(ia_context *ctx, Op opa, Op opb, int M, int N, int K, T alpha, const T *A, int lda,
                       long long sA, const T *B, int ldb, long long sB, T beta, T *C, int ldc, long long sC, int batch)
{
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, batch);
    gemm_kernel<T, BM, BN, TM, TN>
        <<<grid, 256, 0, ctx->stream>>>(opa, opb, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

template <class T, int BM, int BN, int TM, int TN>
static int gemm_panel_launch(ia_context *ctx, int M, int N, int K, T alpha, const T *A, int lda, long long sA,
                             const T *B, int ldb, long long sB, T beta, T *C, int ldc, long long sC, int batch)
{
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, batch);
    gemm_nn_panel_kernel<T, BM, BN, TM, TN>
        <<<grid, 256, 0, ctx->stream>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// tile variants: 64x64 (4x4 per thread), 32x32 (2x2), 128x64 (8x4); for
// untransposed operands with K <= GP_K also the staged-panel forms 32x32
// (2x2) and, FP32 only, 64x64 (4x4)
constexpr int GEMM_VARIANTS = 3;
constexpr int GEMM_VARIANTS_PANEL = 5;

template <class T>
int gemm_batched(ia_context *ctx, Op opa, Op opb, int M, int N, int K, T alpha, const T *A, int lda, long long sA,
                 const T *B, int ldb, long long sB, T beta, T *C, int ldc, long long sC, int batch)
{
    if (M <= 0 || N <= 0 || batch <= 0) return IA_OK;
    auto launch = [&](int v, T *Cout) -> int {
        switch (v) {
        case 1: return gemm_launch<T, 32, 32, 2, 2>(ctx, opa, opb, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, Cout,
                                                    ldc, sC, batch);
        case 2: return gemm_launch<T, 128, 64, 8, 4>(ctx, opa, opb, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta,
                                                     Cout, ldc, sC, batch);
        case 3: return gemm_panel_launch<T, 32, 32, 2, 2>(ctx, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, Cout,
                                                          ldc, sC, batch);
        case 4:
            // 64x64 panels of double2 would take 66 KB, above the static shared-memory limit
            if constexpr (std::is_same<T, float2>::value)
                return gemm_panel_launch<T, 64, 64, 4, 4>(ctx, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, Cout,
                                                          ldc, sC, batch);
            return IA_ERR_ARG;
        default: return gemm_launch<T, 64, 64, 4, 4>(ctx, opa, opb, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta,
                                                     Cout, ldc, sC, batch);
        }
    };
    TuneKey key{};
    key.kernel = sizeof(T) == sizeof(double2) ? TK_GEMM_Z : TK_GEMM_C;
    key.v[0] = opa;
    key.v[1] = opb;
    key.v[2] = M;
    key.v[3] = N;
    key.v[4] = K;
    key.v[5] = batch;
    const size_t cbytes = sizeof(T) * ((size_t)(batch - 1) * sC + (size_t)ldc * (N - 1) + M);
    TuneScratch scratch{ctx};
    const bool panel = opa == OP_N && opb == OP_N && K <= GP_K;
    const int nvar = !panel                               ? GEMM_VARIANTS
                     : std::is_same<T, float2>::value ? GEMM_VARIANTS_PANEL
                                                      : GEMM_VARIANTS_PANEL - 1;
    const int v = tune_select(ctx, key, nvar, [&](int vv) -> int {
        if (!scratch.p) {
            int st = scratch.init(C, cbytes);
            if (st) return st;
        }
        return launch(vv, (T *)scratch.p);
    });
    return launch(v, C);
}

// --------------------------------------------------------------------------
// LU with partial pivoting (LAPACK zgetrf semantics: pivot = largest
// |re|+|im| in the column, first index on ties; row interchanges applied to
// whole rows; ipiv 0-based).  Blocked right-looking: panel (one CTA per
// matrix), U12 = L11^-1 A12 (trsm), A22 -= L21 U12 (gemm).
// --------------------------------------------------------------------------
constexpr int LU_NB = 32;
constexpr int PANEL_THREADS = 256;

template <class T>
__global__ void __launch_bounds__(PANEL_THREADS) lu_panel_kernel(int n, T *A, int lda, long long sA, int *ipiv,
                                                                   int k0, int kend, int *info)
{
    typedef typename ctraits<T>::R R;
    __shared__ R sval[PANEL_THREADS / 32];
    __shared__ int sidx[PANEL_THREADS / 32];
    __shared__ int s_piv;
    const int f = blockIdx.x;
    A += f * sA;
    ipiv += (size_t)f * n;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int j = k0; j < kend; ++j) {
        R best = -1;
        int bi = n;
        for (int i = j + tid; i < n; i += PANEL_THREADS) {
            T a = A[i + (size_t)j * lda];
            R v = fabs(a.x) + fabs(a.y);
            if (v > best) { best = v; bi = i; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            R ov = __shfl_xor_sync(0xffffffffu, best, o);
            int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) { sval[wid] = best; sidx[wid] = bi; }
        __syncthreads();
        if (tid == 0) {
            R bv = sval[0];
            int bidx = sidx[0];
            for (int w = 1; w < PANEL_THREADS / 32; ++w)
                if (sval[w] > bv || (sval[w] == bv && sidx[w] < bidx)) { bv = sval[w]; bidx = sidx[w]; }
            if (!(bv > 0)) {
                if (!(bv == 0)) info[f] |= IA_INFO_NONFINITE;
                else info[f] |= IA_INFO_SINGULAR;
                bidx = j;
            }
            s_piv = bidx;
            ipiv[j] = bidx;
        }
        __syncthreads();
        const int piv = s_piv;
        if (piv != j) {
            for (int c = tid; c < n; c += PANEL_THREADS) {
                T t = A[j + (size_t)c * lda];
                A[j + (size_t)c * lda] = A[piv + (size_t)c * lda];
                A[piv + (size_t)c * lda] = t;
            }
        }
        __syncthreads();
        T d = A[j + (size_t)j * lda];
        if (d.x != 0 || d.y != 0) {
            T inv = zdiv(ctraits<T>::make(1, 0), d);
            for (int i = j + 1 + tid; i < n; i += PANEL_THREADS)
                A[i + (size_t)j * lda] = zmul(A[i + (size_t)j * lda], inv);
        }
        __syncthreads();
        // rank-1 update, thread per row (coalesced down each column)
        for (int r = j + 1 + tid; r < n; r += PANEL_THREADS) {
            const T l = A[r + (size_t)j * lda];
            for (int c = j + 1; c < kend; ++c) {
                T v = A[r + (size_t)c * lda];
                zfms(v, l, A[j + (size_t)c * lda]);
                A[r + (size_t)c * lda] = v;
            }
        }
        __syncthreads();
    }
}

// The same panel factorisation with the panel (rows k0..n-1 of columns
// k0..kend-1) held in shared memory: identical arithmetic in the same order,
// so the factors are bitwise those of lu_panel_kernel.  Row interchanges are
// applied inside the panel only; lu_laswp_kernel applies them to the other
// columns afterwards.
template <class T>
__global__ void __launch_bounds__(PANEL_THREADS) lu_panel_smem_kernel(int n, T *A, int lda, long long sA, int *ipiv,
                                                                        int k0, int kend, int *info)
{
    typedef typename ctraits<T>::R R;
    extern __shared__ unsigned char lu_smem[];
    T *P = reinterpret_cast<T *>(lu_smem);          // P[c * pr + (i - k0)]
    __shared__ R sval[PANEL_THREADS / 32];
    __shared__ int sidx[PANEL_THREADS / 32];
    const int f = blockIdx.x;
    A += f * sA;
    ipiv += (size_t)f * n;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int pr = n - k0, nb = kend - k0;
    for (int e = tid; e < pr * nb; e += PANEL_THREADS) {
        const int i = e % pr, c = e / pr;
        P[e] = A[k0 + i + (size_t)(k0 + c) * lda];
    }
    __syncthreads();
    // A(i, c) of the panel is P[(c - k0) * pr + i - k0].  The pivot search of
    // column j + 1 rides in column j's rank-1 update (the threads that update
    // column j + 1 keep the running maximum of the new values), so a column
    // costs three barriers: interchange, scale, update.  Every thread decides
    // the pivot from the per-warp maxima itself.  Same values, same order of
    // comparison, so the pivots are those of a separate search.
    auto warp_best = [&](R best, int bi) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            R ov = __shfl_xor_sync(0xffffffffu, best, o);
            int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) { sval[wid] = best; sidx[wid] = bi; }
    };
    {
        const T *col = P;                                   // column k0
        R best = -1;
        int bi = n;
        for (int i = k0 + tid; i < n; i += PANEL_THREADS) {
            T a = col[i - k0];
            R v = fabs(a.x) + fabs(a.y);
            if (v > best) { best = v; bi = i; }
        }
        warp_best(best, bi);
        __syncthreads();
    }
    for (int j = k0; j < kend; ++j) {
        R bv = sval[0];
        int piv = sidx[0];
        for (int w = 1; w < PANEL_THREADS / 32; ++w)
            if (sval[w] > bv || (sval[w] == bv && sidx[w] < piv)) { bv = sval[w]; piv = sidx[w]; }
        if (!(bv > 0)) piv = j;
        if (tid == 0) {
            if (!(bv > 0)) info[f] |= (bv == 0) ? IA_INFO_SINGULAR : IA_INFO_NONFINITE;
            ipiv[j] = piv;
        }
        if (piv != j) {
            for (int c = tid; c < nb; c += PANEL_THREADS) {
                T *pc = P + (size_t)c * pr;
                T t = pc[j - k0];
                pc[j - k0] = pc[piv - k0];
                pc[piv - k0] = t;
            }
        }
        __syncthreads();
        T *cj = P + (size_t)(j - k0) * pr;
        T d = cj[j - k0];
        if (d.x != 0 || d.y != 0) {
            T inv = zdiv(ctraits<T>::make(1, 0), d);
            for (int i = j + 1 + tid; i < n; i += PANEL_THREADS) cj[i - k0] = zmul(cj[i - k0], inv);
        }
        __syncthreads();
        // rank-1 update, thread per row: the row's multiplier once, then the
        // remaining columns in order (each element sees the same operations
        // in the same order as any other work split)
        const int ncols = kend - j - 1;
        R best = -1;
        int bi = n;
        if (ncols > 0) {
            for (int r = j + 1 + tid; r < n; r += PANEL_THREADS) {
                const T l = cj[r - k0];
                {
                    T *pc = P + (size_t)(j + 1 - k0) * pr;
                    T v = pc[r - k0];
                    zfms(v, l, pc[j - k0]);
                    pc[r - k0] = v;
                    const R av = fabs(v.x) + fabs(v.y);
                    if (av > best) { best = av; bi = r; }
                }
                for (int c = j + 2; c < kend; ++c) {
                    T *pc = P + (size_t)(c - k0) * pr;
                    T v = pc[r - k0];
                    zfms(v, l, pc[j - k0]);
                    pc[r - k0] = v;
                }
            }
            warp_best(best, bi);
        }
        __syncthreads();
    }
    for (int e = tid; e < pr * nb; e += PANEL_THREADS) {
        const int i = e % pr, c = e / pr;
        A[k0 + i + (size_t)(k0 + c) * lda] = P[e];
    }
}

// apply the interchanges ipiv[k0..kend) to every column outside [k0, kend)
template <class T>
__global__ void lu_laswp_kernel(int n, T *A, int lda, long long sA, const int *ipiv, int k0, int kend)
{
    const int f = blockIdx.y;
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n - (kend - k0)) return;
    if (c >= k0) c += kend - k0;
    T *a = A + f * sA + (size_t)c * lda;
    const int *pv = ipiv + (size_t)f * n;
    for (int j = k0; j < kend; ++j) {
        const int p = pv[j];
        if (p != j) {
            T t = a[j];
            a[j] = a[p];
            a[p] = t;
        }
    }
}

// Solve T X = X in place for an nbk x nbk diagonal block T (lower unit or
// upper non-unit) and X = nbk x ncols; one thread per column.
template <class T, bool UPPER>
__global__ void __launch_bounds__(128) trsm_block_kernel(int nbk, const T *Tm, int ldt, long long sT, T *X, int ldx,
                                                           long long sX, int ncols)
{
    __shared__ T Ts[LU_NB][LU_NB + 1];
    const int f = blockIdx.y;
    Tm += f * sT;
    X += f * sX;
    for (int e = threadIdx.x; e < nbk * nbk; e += blockDim.x) {
        int r = e % nbk, c = e / nbk;
        Ts[r][c] = Tm[r + (size_t)c * ldt];
    }
    __syncthreads();
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= ncols) return;
    T x[LU_NB];
#pragma unroll
    for (int r = 0; r < LU_NB; ++r)
        if (r < nbk) x[r] = X[r + (size_t)col * ldx];
    if (!UPPER) {
#pragma unroll
        for (int r = 0; r < LU_NB; ++r) {
            if (r >= nbk) break;
            T v = x[r];
#pragma unroll
            for (int t = 0; t < LU_NB; ++t)
                if (t < r) zfms(v, Ts[r][t], x[t]);
            x[r] = v;
        }
    } else {
#pragma unroll
        for (int r = LU_NB - 1; r >= 0; --r) {
            if (r >= nbk) continue;
            T v = x[r];
#pragma unroll
            for (int t = 0; t < LU_NB; ++t)
                if (t > r && t < nbk) zfms(v, Ts[r][t], x[t]);
            x[r] = zdiv(v, Ts[r][r]);
        }
    }
#pragma unroll
    for (int r = 0; r < LU_NB; ++r)
        if (r < nbk) X[r + (size_t)col * ldx] = x[r];
}

template <class T>
int getrf_batched(ia_context *ctx, int n, T *A, int lda, long long sA, int *ipiv, int *info, int batch)
{
    const T one = ctraits<T>::make(1, 0), mone = ctraits<T>::make(-1, 0);
    constexpr size_t kPanelSmemMax = 200 * 1024;
    const bool smem_panel = (size_t)n * LU_NB * sizeof(T) <= kPanelSmemMax;
    if (smem_panel)
        IA_CUDA_TRY(cudaFuncSetAttribute(lu_panel_smem_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kPanelSmemMax));
    for (int k0 = 0; k0 < n; k0 += LU_NB) {
        int kend = k0 + LU_NB < n ? k0 + LU_NB : n;
        int nb = kend - k0;
        if (smem_panel) {
            const size_t smem = (size_t)(n - k0) * nb * sizeof(T);
            lu_panel_smem_kernel<T><<<batch, PANEL_THREADS, smem, ctx->stream>>>(n, A, lda, sA, ipiv, k0, kend, info);
            IA_LAUNCH_CHECK(ctx);
            if (n > nb) {
                dim3 gs((n - nb + 127) / 128, batch);
                lu_laswp_kernel<T><<<gs, 128, 0, ctx->stream>>>(n, A, lda, sA, ipiv, k0, kend);
                IA_LAUNCH_CHECK(ctx);
            }
        } else {
            lu_panel_kernel<T><<<batch, PANEL_THREADS, 0, ctx->stream>>>(n, A, lda, sA, ipiv, k0, kend, info);
            IA_LAUNCH_CHECK(ctx);
        }
        int rest = n - kend;
        if (rest <= 0) break;
        dim3 g((rest + 127) / 128, batch);
        trsm_block_kernel<T, false><<<g, 128, 0, ctx->stream>>>(nb, A + k0 + (size_t)k0 * lda, lda, sA,
                                                                 A + k0 + (size_t)kend * lda, lda, sA, rest);
        IA_LAUNCH_CHECK(ctx);
        int r = gemm_batched<T>(ctx, OP_N, OP_N, rest, rest, nb, mone, A + kend + (size_t)k0 * lda, lda, sA,
                                A + k0 + (size_t)kend * lda, lda, sA, one, A + kend + (size_t)kend * lda, lda, sA,
                                batch);
        if (r) return r;
    }
    return IA_OK;
}

template <class T>
__global__ void apply_pivots_kernel(int n, int nrhs, const int *ipiv, T *B, int ldb, long long sB)
{
    const int f = blockIdx.y;
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= nrhs) return;
    ipiv += (size_t)f * n;
    T *b = B + f * sB + (size_t)col * ldb;
    for (int j = 0; j < n; ++j) {
        int p = ipiv[j];
        if (p != j) {
            T t = b[j];
            b[j] = b[p];
            b[p] = t;
        }
    }
}

template <class T>
int backsolve_upper_batched(ia_context *ctx, int n, int nrhs, const T *LU, int lda, long long sA, T *B, int ldb,
                            long long sB, int batch)
{
    const T one = ctraits<T>::make(1, 0), mone = ctraits<T>::make(-1, 0);
    dim3 g((nrhs + 127) / 128, batch);
    int nblk = (n + LU_NB - 1) / LU_NB;
    for (int bi = nblk - 1; bi >= 0; --bi) {
        int k0 = bi * LU_NB;
        int kend = k0 + LU_NB < n ? k0 + LU_NB : n;
        int nb = kend - k0;
        trsm_block_kernel<T, true><<<g, 128, 0, ctx->stream>>>(nb, LU + k0 + (size_t)k0 * lda, lda, sA, B + k0, ldb,
                                                                sB, nrhs);
        IA_LAUNCH_CHECK(ctx);
        if (k0 > 0) {
            int r = gemm_batched<T>(ctx, OP_N, OP_N, k0, nrhs, nb, mone, LU + (size_t)k0 * lda, lda, sA, B + k0, ldb,
                                    sB, one, B, ldb, sB, batch);
            if (r) return r;
        }
    }
    return IA_OK;
}

// Fused LU solve (FP32 complex): the row interchanges, the unit-lower L solve
// and the upper U solve for GETRS_RB right-hand-side columns of one matrix per
// CTA, in one launch, the n x GETRS_RB block of B in shared memory (columns of
// even stride, so two consecutive entries load as one 16-byte word).  Block
// steps of LU_NB rows: the diagonal block is staged in shared memory, zero
// outside the block (a partial last block needs no masks), with the
// reciprocals of U's diagonal computed in parallel; it is solved warp per
// column, lane per row, each solved entry broadcast by shuffle, branch-free
// (a select per step in place of the lane tests and the division).  The rows
// below (forward) or above (backward) are then updated thread per row, the
// block's LU_NB entries of the row of L or U loaded together from global
// memory (L2), the solved entries read in pairs.  Full blocks run without
// per-entry predicates.  Replaces 2 n / LU_NB dependent small launches (a
// diagonal-block solve and a GEMM update per step) by one.

__device__ __forceinline__ float2 shfl_c(float2 v, int src)
{
    return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// X rows [lo, hi) -= T(:, 0:nb) X(k0:k0+nb, :), thread per row (T: the L or
// U block column, leading dimension lda, starting at row 0 of the matrix)
template <int RB, int NT, bool FULL>
__device__ __forceinline__ void getrs_update(const float2 *__restrict__ T, int lda, long long text, float2 *X, int xs,
                                             int k0, int nb, int lo, int hi)
{
    // the row's entries in two halves (register budget: two CTAs per SM);
    // two threads per row, each with half of the right-hand sides (twice the
    // warps to hide the row loads' L2 latency: 25.9 -> 25.75 ms per pass)
    constexpr int TH = LU_NB / 2;
    constexpr int SPLIT = 2, RBT = RB / SPLIT, NR = NT / SPLIT;
    const int cbase = ((int)threadIdx.x / NR) * RBT;
    X += (size_t)cbase * xs;
    for (int i = lo + (int)threadIdx.x % NR; i < hi; i += NR) {
        const float2 *tp = T + i;
        float2 acc[RBT];
#pragma unroll
        for (int c = 0; c < RBT; ++c) acc[c] = X[i + (size_t)c * xs];
#pragma unroll
        for (int h = 0; h < LU_NB; h += TH) {
            float2 trow[TH];
#pragma unroll
            for (int t = 0; t < TH; ++t)
                trow[t] = (FULL || h + t < nb) && IA_IDX_OK(i + (long long)(h + t) * lda, text)
                              ? tp[(size_t)(h + t) * lda]
                              : make_float2(0.f, 0.f);
#pragma unroll
            for (int t = 0; t < TH; t += 2) {
                if (FULL || h + t < nb) {
#pragma unroll
                    for (int c = 0; c < RBT; ++c) {
                        // X(k0 + h + t, c) and the entry below: k0, h, t and xs even
                        const float4 x2 = *reinterpret_cast<const float4 *>(X + k0 + h + t + (size_t)c * xs);
                        zfms(acc[c], trow[t], make_float2(x2.x, x2.y));
                        zfms(acc[c], trow[t + 1], make_float2(x2.z, x2.w));
                    }
                }
            }
        }
#pragma unroll
        for (int c = 0; c < RBT; ++c) X[i + (size_t)c * xs] = acc[c];
    }
}

template <int GETRS_RB, int NT>
__global__ void __launch_bounds__(NT, 2) getrs_fused_kernel(int n, int nrhs, const float2 *__restrict__ LU,
                                                                     int lda, long long sA,
                                                                     const int *__restrict__ ipiv, float2 *B, int ldb,
                                                                     long long sB)
{
    extern __shared__ __align__(16) unsigned char gf_smem[];
    const int xs = (n + 1) & ~1;
    float2 *X = reinterpret_cast<float2 *>(gf_smem);                                  // xs x GETRS_RB
    float2(*D)[LU_NB + 1] = reinterpret_cast<float2(*)[LU_NB + 1]>(X + (size_t)xs * GETRS_RB);
    float2 *Dinv = reinterpret_cast<float2 *>(D + LU_NB);                              // LU_NB
    int *piv = reinterpret_cast<int *>(Dinv + LU_NB);                                  // n
    const int f = blockIdx.y, c0 = blockIdx.x * GETRS_RB;
    const int nc = nrhs - c0 < GETRS_RB ? nrhs - c0 : GETRS_RB;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    LU += f * sA;
    ipiv += (size_t)f * n;
    B += f * sB + (size_t)c0 * ldb;
    const float2 zero = make_float2(0.f, 0.f);
    const long long lext = (long long)n * lda, bext = (long long)nc * ldb;   // this matrix's LU, this CTA's B columns
    for (int e = tid; e < xs * GETRS_RB; e += NT) {
        const int i = e % xs, c = e / xs;
        X[e] = c < nc && i < n && IA_IDX_OK(i + (long long)c * ldb, bext) ? B[i + (size_t)c * ldb] : zero;
    }
    for (int j = tid; j < n; j += NT) piv[j] = ipiv[j];
    __syncthreads();
    if (tid < GETRS_RB) {
        float2 *x = X + (size_t)tid * xs;
        for (int j = 0; j < n; ++j) {
            const int p = piv[j];
            if (p != j && IA_IDX_OK(p, n)) {
                const float2 t = x[j];
                x[j] = x[p];
                x[p] = t;
            }
        }
    }
    __syncthreads();
    // forward: L Y = P B
    for (int k0 = 0; k0 < n; k0 += LU_NB) {
        const int nb = n - k0 < LU_NB ? n - k0 : LU_NB, kend = k0 + nb;
        for (int e = tid; e < LU_NB * LU_NB; e += NT) {
            const int r = e % LU_NB, cc = e / LU_NB;
            D[r][cc] = r < nb && cc < nb && IA_IDX_OK(k0 + r + (long long)(k0 + cc) * lda, lext)
                           ? LU[k0 + r + (size_t)(k0 + cc) * lda]
                           : zero;
        }
        __syncthreads();
        if (wid < GETRS_RB) {
            // lanes >= nb hold zero and, with D zero there, stay zero
            float2 *x = X + (size_t)wid * xs + k0;
            float2 v = lane < nb ? x[lane] : zero;
#pragma unroll
            for (int r = 0; r < LU_NB; ++r) {
                const float2 xr = shfl_c(v, r);
                const float2 d = lane > r ? D[lane][r] : zero;
                zfms(v, d, xr);
            }
            if (lane < nb) x[lane] = v;
        }
        __syncthreads();
        const long long text = lext - (long long)k0 * lda;
        if (nb == LU_NB) getrs_update<GETRS_RB, NT, true>(LU + (size_t)k0 * lda, lda, text, X, xs, k0, nb, kend, n);
        else getrs_update<GETRS_RB, NT, false>(LU + (size_t)k0 * lda, lda, text, X, xs, k0, nb, kend, n);
        __syncthreads();
    }
    // backward: U X = Y
    for (int k0 = ((n - 1) / LU_NB) * LU_NB; k0 >= 0; k0 -= LU_NB) {
        const int nb = n - k0 < LU_NB ? n - k0 : LU_NB;
        for (int e = tid; e < LU_NB * LU_NB; e += NT) {
            const int r = e % LU_NB, cc = e / LU_NB;
            D[r][cc] = r < nb && cc < nb && IA_IDX_OK(k0 + r + (long long)(k0 + cc) * lda, lext)
                           ? LU[k0 + r + (size_t)(k0 + cc) * lda]
                           : zero;
        }
        if (tid < LU_NB) {
            const float2 d = tid < nb && IA_IDX_OK(k0 + tid + (long long)(k0 + tid) * lda, lext)
                                 ? LU[k0 + tid + (size_t)(k0 + tid) * lda]
                                 : zero;
            Dinv[tid] = tid < nb ? zdiv(make_float2(1.f, 0.f), d) : zero;
        }
        __syncthreads();
        if (wid < GETRS_RB) {
            float2 *x = X + (size_t)wid * xs + k0;
            float2 v = lane < nb ? x[lane] : zero;
#pragma unroll
            for (int r = LU_NB - 1; r >= 0; --r) {
                const float2 sv = zmul(v, Dinv[r]);
                v = lane == r ? sv : v;
                const float2 xr = shfl_c(v, r);
                const float2 d = lane < r ? D[lane][r] : zero;
                zfms(v, d, xr);
            }
            if (lane < nb) x[lane] = v;
        }
        __syncthreads();
        const long long text = lext - (long long)k0 * lda;
        if (nb == LU_NB) getrs_update<GETRS_RB, NT, true>(LU + (size_t)k0 * lda, lda, text, X, xs, k0, nb, 0, k0);
        else getrs_update<GETRS_RB, NT, false>(LU + (size_t)k0 * lda, lda, text, X, xs, k0, nb, 0, k0);
        __syncthreads();
    }
    for (int e = tid; e < n * nc; e += NT) {
        const int i = e % n, c = e / n;
        if (IA_IDX_OK(i + (long long)c * ldb, bext)) B[i + (size_t)c * ldb] = X[i + (size_t)c * xs];
    }
}

static size_t getrs_fused_smem(int n, int GETRS_RB)
{
    const size_t xs = (size_t)((n + 1) & ~1);
    return sizeof(float2) * (xs * GETRS_RB + (size_t)LU_NB * (LU_NB + 1) + LU_NB) + sizeof(int) * (size_t)n;
}

template <class T>
int getrs_batched(ia_context *ctx, int n, int nrhs, const T *LU, int lda, long long sA, const int *ipiv, T *B,
                  int ldb, long long sB, int batch)
{
    if (n <= 0 || nrhs <= 0 || batch <= 0) return IA_OK;
    if constexpr (std::is_same<T, float2>::value) {
        // 8 right-hand sides per CTA (4 and 16 measured slower: with 16, the
        // 64-bin pass 28.4 against 28.0 ms)
        constexpr int rb = 8;
        const size_t smem = getrs_fused_smem(n, rb);
        // 512 threads: a warp per right-hand side in the diagonal solves, two
        // threads per row in the updates
        constexpr int nt = 64 * rb;
        if (smem <= 200 * 1024) {
            auto kern = getrs_fused_kernel<rb, nt>;
            if (smem > 48 * 1024)
                IA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
            dim3 gf((nrhs + rb - 1) / rb, batch);
            kern<<<gf, nt, smem, ctx->stream>>>(n, nrhs, LU, lda, sA, ipiv, B, ldb, sB);
            IA_LAUNCH_CHECK(ctx);
            return IA_OK;
        }
    }
    const T one = ctraits<T>::make(1, 0), mone = ctraits<T>::make(-1, 0);
    dim3 g((nrhs + 127) / 128, batch);
    apply_pivots_kernel<T><<<g, 128, 0, ctx->stream>>>(n, nrhs, ipiv, B, ldb, sB);
    IA_LAUNCH_CHECK(ctx);
    // forward: L Y = B
    for (int k0 = 0; k0 < n; k0 += LU_NB) {
        int kend = k0 + LU_NB < n ? k0 + LU_NB : n;
        int nb = kend - k0;
        trsm_block_kernel<T, false><<<g, 128, 0, ctx->stream>>>(nb, LU + k0 + (size_t)k0 * lda, lda, sA, B + k0, ldb,
                                                                 sB, nrhs);
        IA_LAUNCH_CHECK(ctx);
        if (kend < n) {
            int r = gemm_batched<T>(ctx, OP_N, OP_N, n - kend, nrhs, nb, mone, LU + kend + (size_t)k0 * lda, lda, sA,
                                    B + k0, ldb, sB, one, B + kend, ldb, sB, batch);
            if (r) return r;
        }
    }
    return backsolve_upper_batched<T>(ctx, n, nrhs, LU, lda, sA, B, ldb, sB, batch);
}

// --------------------------------------------------------------------------
// transposes / copies through a 32x32 shared tile
// --------------------------------------------------------------------------
template <class T>
__global__ void transpose_kernel(int rows, int cols, const T *in, int ldi, long long si, T *out, int ldo, long long so,
                                 int conj)
{
    __shared__ T tile[32][33];
    const int f = blockIdx.z;
    in += f * si;
    out += f * so;
    int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
    for (int t = threadIdx.y; t < 32; t += blockDim.y) {
        int r = r0 + threadIdx.x, c = c0 + t;
        if (r < rows && c < cols) tile[t][threadIdx.x] = in[r + (size_t)c * ldi];
    }
    __syncthreads();
    for (int t = threadIdx.y; t < 32; t += blockDim.y) {
        int oc = r0 + t, orow = c0 + threadIdx.x;  // out(orow, oc) = in(oc, orow)
        if (oc < rows && orow < cols) {
            T v = tile[threadIdx.x][t];
            if (conj) v.y = -v.y;
            out[orow + (size_t)oc * ldo] = v;
        }
    }
}

template <class T>
int transpose_batched(ia_context *ctx, int rows, int cols, const T *in, int ldi, long long si, T *out, int ldo,
                      long long so, bool conj, int batch)
{
    dim3 g((cols + 31) / 32, (rows + 31) / 32, batch);
    transpose_kernel<T><<<g, dim3(32, 8), 0, ctx->stream>>>(rows, cols, in, ldi, si, out, ldo, so, conj ? 1 : 0);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// 2-D copy with optional conjugation and element-type conversion
template <class TI, class TO>
__global__ void copy2d_kernel(int rows, int cols, const TI *in, int ldi, long long si, TO *out, int ldo, long long so,
                              int conj)
{
    typedef typename ctraits<TO>::R RO;
    const int f = blockIdx.y;
    long long total = (long long)rows * cols;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        int r = (int)(e % rows), c = (int)(e / rows);
        TI v = in[f * si + r + (size_t)c * ldi];
        out[f * so + r + (size_t)c * ldo] = ctraits<TO>::make((RO)v.x, conj ? -(RO)v.y : (RO)v.y);
    }
}

template <class TI, class TO>
int copy2d_batched(ia_context *ctx, int rows, int cols, const TI *in, int ldi, long long si, TO *out, int ldo,
                   long long so, bool conj, int batch)
{
    long long total = (long long)rows * cols;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 1024) blocks = 1024;
    dim3 g(blocks, batch);
    copy2d_kernel<TI, TO><<<g, 256, 0, ctx->stream>>>(rows, cols, in, ldi, si, out, ldo, so, conj ? 1 : 0);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

template <class TI>
__global__ void add2d_kernel(int rows, int cols, const TI *in, int ldi, long long si, double2 *out, int ldo,
                             long long so)
{
    const int f = blockIdx.y;
    long long total = (long long)rows * cols;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        int r = (int)(e % rows), c = (int)(e / rows);
        TI v = in[f * si + r + (size_t)c * ldi];
        double2 *o = out + f * so + r + (size_t)c * ldo;
        *o = make_double2(o->x + (double)v.x, o->y + (double)v.y);
    }
}

template <class TI>
int add2d_batched(ia_context *ctx, int rows, int cols, const TI *in, int ldi, long long si, double2 *out, int ldo,
                  long long so, int batch)
{
    long long total = (long long)rows * cols;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 1024) blocks = 1024;
    add2d_kernel<TI><<<dim3(blocks, batch), 256, 0, ctx->stream>>>(rows, cols, in, ldi, si, out, ldo, so);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}
template int add2d_batched<float2>(ia_context *, int, int, const float2 *, int, long long, double2 *, int, long long,
                                   int);
template int add2d_batched<double2>(ia_context *, int, int, const double2 *, int, long long, double2 *, int,
                                    long long, int);

// ---- instantiations ------------------------------------------------------
#define IA_DENSE_INST(T)                                                                                              \
    template int gemm_batched<T>(ia_context *, Op, Op, int, int, int, T, const T *, int, long long, const T *, int,   \
                                 long long, T, T *, int, long long, int);                                            \
    template int getrf_batched<T>(ia_context *, int, T *, int, long long, int *, int *, int);                         \
    template int getrs_batched<T>(ia_context *, int, int, const T *, int, long long, const int *, T *, int, long long, \
                                  int);                                                                               \
    template int backsolve_upper_batched<T>(ia_context *, int, int, const T *, int, long long, T *, int, long long,    \
                                            int);                                                                     \
    template int transpose_batched<T>(ia_context *, int, int, const T *, int, long long, T *, int, long long, bool,   \
                                      int);
IA_DENSE_INST(double2)
IA_DENSE_INST(float2)
template int copy2d_batched<double2, double2>(ia_context *, int, int, const double2 *, int, long long, double2 *, int,
                                              long long, bool, int);
template int copy2d_batched<float2, float2>(ia_context *, int, int, const float2 *, int, long long, float2 *, int,
                                            long long, bool, int);
template int copy2d_batched<double2, float2>(ia_context *, int, int, const double2 *, int, long long, float2 *, int,
                                             long long, bool, int);
template int copy2d_batched<float2, double2>(ia_context *, int, int, const float2 *, int, long long, double2 *, int,
                                             long long, bool, int);

IA_BOUNDS_READER(bounds_read_dense)

}  // namespace ia
