// Radiation modes of baffled radiators (plates, panels): the sinc radiation
// resistance matrix, its leading eigenpairs, and sound power v^H R v.
//
//   R_f(i,j) = omega^2 rho A^2 / (4 pi c) * sinc(k_f r_ij),  omega = k_f c
//
// The reference names this model for its radiation-mode configuration but
// ships no code for it; its BEM variant (CUDA/invr.cuh:457, MATLAB/invrV.m:65-119)
// forms the resistance matrix from R = Re(G Z) instead.  Sound power follows
// the reference's 1/2 Re(v^H p) convention (CUDA/utils.cuh:265-280) with
// p = R v.
//
// R is real symmetric positive semidefinite with a spectrum that falls off
// faster than exponentially past roughly area k^2 / (4 pi) modes (the
// radiating ones), so its numerical rank is small (under 200 for a 1280
// element plate at ka ~ 18).  The leading modes are found by block subspace
// iteration (Rutishauser; Saad, "Numerical Methods for Large Eigenvalue
// Problems", ch. 5) on b = nmodes + oversample vectors with Householder
// re-orthonormalisation, then one Rayleigh-Ritz projection in FP64.  In the
// mixed path the iterations run in FP32 and are followed by FP64 power steps
// whose products use double-float arithmetic on the FP32 pipe.
#include "df32.cuh"
#include <cooperative_groups.h>
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

// --------------------------------------------------------------------------
// R assembly.  CTA: a 64 x 64 tile of (i, j) for SR_FB frequencies; thread t
// owns row i0 + (t & 63) and columns j0 + (t >> 6) + 4 q, so each warp stores
// 32 consecutive rows of one column (coalesced, column-major).  For evenly
// spaced wavenumbers the phase advances by exp(i dk r) from frequency to
// frequency (two sincos per entry per block instead of SR_FB).
// --------------------------------------------------------------------------
constexpr int SR_TILE = 64;
constexpr int SR_FB = 8;

__global__ void __launch_bounds__(256) sinc_r_kernel(int n, const double *__restrict__ x, int F,
                                                     const double *__restrict__ kv, double pref,
                                                     double *__restrict__ R, float *__restrict__ R32)
{
    __shared__ double sx[SR_TILE], sy[SR_TILE], sz[SR_TILE];
    const int j0 = blockIdx.x * SR_TILE;
    const int i = blockIdx.y * SR_TILE + (threadIdx.x & 63);
    const int f0 = blockIdx.z * SR_FB;
    if (threadIdx.x < SR_TILE) {
        const int j = min(j0 + (int)threadIdx.x, n - 1);
        sx[threadIdx.x] = x[j];
        sy[threadIdx.x] = x[j + n];
        sz[threadIdx.x] = x[j + 2 * n];
    }
    __syncthreads();
    if (i >= n) return;
    const int nf = min(SR_FB, F - f0);
    double kf[SR_FB];
#pragma unroll
    for (int f = 0; f < SR_FB; ++f) kf[f] = kv[f0 + (f < nf ? f : nf - 1)];
    const double dk = nf > 1 ? kf[1] - kf[0] : 0.0;
    bool uniform = true;
#pragma unroll
    for (int f = 2; f < SR_FB; ++f)
        if (f < nf && fabs(kf[f] - (kf[0] + f * dk)) > 1e-12 * fabs(kf[f])) uniform = false;
    const double xi = x[i], yi = x[i + n], zi = x[i + 2 * n];
    const size_t nn = (size_t)n * n;
    for (int q = 0; q < SR_TILE / 4; ++q) {
        const int jl = (threadIdx.x >> 6) + 4 * q;
        const int j = j0 + jl;
        if (j >= n) break;
        const double dx = xi - sx[jl], dy = yi - sy[jl], dz = zi - sz[jl];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        double val[SR_FB];
        if (r == 0.0) {
#pragma unroll
            for (int f = 0; f < SR_FB; ++f) val[f] = pref * kf[f] * kf[f];
        } else {
            const double invr = 1.0 / r;
            double s, c, sd = 0.0, cd = 1.0;
            sincos(kf[0] * r, &s, &c);
            if (uniform && nf > 1) sincos(dk * r, &sd, &cd);
#pragma unroll
            for (int f = 0; f < SR_FB; ++f) {
                if (f > 0) {
                    if (uniform) {
                        const double s1 = fma(s, cd, c * sd);
                        c = fma(c, cd, -s * sd);
                        s = s1;
                    } else {
                        sincos(kf[f] * r, &s, &c);
                    }
                }
                // omega^2 rho A^2/(4 pi c) sin(kr)/(kr) = (c rho A^2/(4 pi)) k sin(kr)/r
                val[f] = pref * kf[f] * s * invr;
            }
        }
        const size_t o = (size_t)i + (size_t)j * n;
#pragma unroll
        for (int f = 0; f < SR_FB; ++f) {
            if (f >= nf) break;
            R[(size_t)(f0 + f) * nn + o] = val[f];
            if (R32) R32[(size_t)(f0 + f) * nn + o] = (float)val[f];
        }
    }
}

int sinc_resistance_batched(ia_context *ctx, int n, const double *x, int F, const double *k, double area, double c,
                            double rho, double *R, float *R32)
{
    if (n <= 0 || F <= 0) return IA_OK;
    const double pref = c * rho * area * area * IA_INV4PI;
    dim3 grid((n + SR_TILE - 1) / SR_TILE, (n + SR_TILE - 1) / SR_TILE, (F + SR_FB - 1) / SR_FB);
    sinc_r_kernel<<<grid, 256, 0, ctx->stream>>>(n, x, F, k, pref, R, R32);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// --------------------------------------------------------------------------
// Real GEMM C = alpha op(A) B + beta C, op(A) in {N, T}; 64 x 64 tiles, K tile
// 16, 256 threads with a 4 x 4 block each (outputs strided by 16).
// --------------------------------------------------------------------------
constexpr int RG_M = 64, RG_N = 64, RG_K = 16;

template <class T>
__global__ void __launch_bounds__(256) rgemm_kernel(int opa, int M, int N, int K, T alpha, const T *__restrict__ A,
                                                    int lda, long long sA, const T *__restrict__ B, int ldb,
                                                    long long sB, T beta, T *__restrict__ C, int ldc, long long sC)
{
    __shared__ T As[RG_K][RG_M + 1];
    __shared__ T Bs[RG_K][RG_N + 1];
    const int f = blockIdx.z;
    A += f * sA;
    B += f * sB;
    C += f * sC;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * RG_M, n0 = blockIdx.x * RG_N;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0;
    for (int k0 = 0; k0 < K; k0 += RG_K) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int e = threadIdx.x + t * 256;
            int r, kk;
            if (opa == OP_N) { r = e % RG_M; kk = e / RG_M; }
            else { kk = e % RG_K; r = e / RG_K; }
            const int gr = m0 + r, gk = k0 + kk;
            T v = 0;
            if (gr < M && gk < K) v = opa == OP_N ? A[gr + (size_t)gk * lda] : A[gk + (size_t)gr * lda];
            As[kk][r] = v;
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int e = threadIdx.x + t * 256;
            const int kk = e % RG_K, c = e / RG_K;
            const int gk = k0 + kk, gc = n0 + c;
            Bs[kk][c] = (gk < K && gc < N) ? B[gk + (size_t)gc * ldb] : T(0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < RG_K; ++kk) {
            T a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = m0 + ty + 16 * i;
        if (r >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = n0 + tx + 16 * j;
            if (c >= N) continue;
            T *p = C + r + (size_t)c * ldc;
            T v = alpha * acc[i][j];
            if (beta != T(0)) v = fma(beta, *p, v);
            *p = v;
        }
    }
}

template <class T>
static int rgemm_batched(ia_context *ctx, Op opa, int M, int N, int K, T alpha, const T *A, int lda, long long sA,
                         const T *B, int ldb, long long sB, T beta, T *C, int ldc, long long sC, int batch)
{
    if (M <= 0 || N <= 0 || batch <= 0) return IA_OK;
    dim3 grid((N + RG_N - 1) / RG_N, (M + RG_M - 1) / RG_M, batch);
    rgemm_kernel<T><<<grid, 256, 0, ctx->stream>>>(opa, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// Real double-float GEMM: FP64 operands split to (hi, lo) FP32 pairs on the
// way into shared memory, products and sums in double-float, FP64 output.
__global__ void __launch_bounds__(256) rdfgemm_kernel(int opa, int M, int N, int K, const double *__restrict__ A,
                                                      int lda, long long sA, const double *__restrict__ B, int ldb,
                                                      long long sB, double *__restrict__ C, int ldc, long long sC)
{
    __shared__ float2 As[RG_K][RG_M + 1];
    __shared__ float2 Bs[RG_K][RG_N + 1];
    const int f = blockIdx.z;
    A += f * sA;
    B += f * sB;
    C += f * sC;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * RG_M, n0 = blockIdx.x * RG_N;
    dfl acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = dfl{0.f, 0.f};
    for (int k0 = 0; k0 < K; k0 += RG_K) {
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int e = threadIdx.x + t * 256;
            int r, kk;
            if (opa == OP_N) { r = e % RG_M; kk = e / RG_M; }
            else { kk = e % RG_K; r = e / RG_K; }
            const int gr = m0 + r, gk = k0 + kk;
            double v = 0.0;
            if (gr < M && gk < K) v = opa == OP_N ? A[gr + (size_t)gk * lda] : A[gk + (size_t)gr * lda];
            const dfl d = df_from_double(v);
            As[kk][r] = make_float2(d.hi, d.lo);
        }
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int e = threadIdx.x + t * 256;
            const int kk = e % RG_K, c = e / RG_K;
            const int gk = k0 + kk, gc = n0 + c;
            const dfl d = df_from_double((gk < K && gc < N) ? B[gk + (size_t)gc * ldb] : 0.0);
            Bs[kk][c] = make_float2(d.hi, d.lo);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < RG_K; ++kk) {
            float2 a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) df_mac(acc[i][j], dfl{a[i].x, a[i].y}, dfl{b[j].x, b[j].y});
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = df_norm(acc[i][j]);
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = m0 + ty + 16 * i;
        if (r >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = n0 + tx + 16 * j;
            if (c >= N) continue;
            C[r + (size_t)c * ldc] = df_to_double(acc[i][j]);
        }
    }
}

static int rdfgemm_batched(ia_context *ctx, Op opa, int M, int N, int K, const double *A, int lda, long long sA,
                           const double *B, int ldb, long long sB, double *C, int ldc, long long sC, int batch)
{
    if (M <= 0 || N <= 0 || batch <= 0) return IA_OK;
    dim3 grid((N + RG_N - 1) / RG_N, (M + RG_M - 1) / RG_M, batch);
    rdfgemm_kernel<<<grid, 256, 0, ctx->stream>>>(opa, M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// C = op(A) B at FP64 accuracy: FP64 GEMM, or double-float on the FP32 pipe
static int prod64(ia_context *ctx, bool df, Op opa, int M, int N, int K, const double *A, int lda, long long sA,
                  const double *B, int ldb, long long sB, double *C, int ldc, long long sC, int batch)
{
    if (df) return rdfgemm_batched(ctx, opa, M, N, K, A, lda, sA, B, ldb, sB, C, ldc, sC, batch);
    return rgemm_batched<double>(ctx, opa, M, N, K, 1.0, A, lda, sA, B, ldb, sB, 0.0, C, ldc, sC, batch);
}

// --------------------------------------------------------------------------
// Real Householder QR of a tall block (rows x cols, one CTA per matrix):
// H_j = I - tau v v^T, v(j) = 1, beta = -sign(alpha) ||x|| (LAPACK dlarfg
// convention), reflectors stored below the diagonal.  Then the explicit
// thin Q = H_0 ... H_{cols-1} [I; 0], warp per column.
// --------------------------------------------------------------------------
constexpr int RQR_THREADS = 512;

template <class T>
__global__ void __launch_bounds__(RQR_THREADS) rqr_kernel(int rows, int cols, T *A, T *tau)
{
    __shared__ T red[RQR_THREADS / 32];
    __shared__ T s_tau, s_scale;
    const int f = blockIdx.x;
    A += (size_t)f * rows * cols;
    tau += (size_t)f * cols;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = RQR_THREADS / 32;
    for (int j = 0; j < cols && j < rows; ++j) {
        T *x = A + j + (size_t)j * rows;
        const int len = rows - j;
        T sg = 0;
        for (int i = 1 + tid; i < len; i += RQR_THREADS) sg = fma(x[i], x[i], sg);
        sg = warp_sum(sg);
        if (lane == 0) red[wid] = sg;
        __syncthreads();
        if (tid == 0) {
            T sigma = 0;
            for (int w = 0; w < nw; ++w) sigma += red[w];
            const T alpha = x[0];
            if (sigma == 0) {
                s_tau = 0;
                s_scale = 0;
            } else {
                const T nrm = sqrt(alpha * alpha + sigma);
                const T beta = alpha >= 0 ? -nrm : nrm;
                s_tau = (beta - alpha) / beta;
                s_scale = T(1) / (alpha - beta);
                x[0] = beta;
            }
            tau[j] = s_tau;
        }
        __syncthreads();
        const T tv = s_tau, sc = s_scale;
        if (tv == 0) continue;
        for (int i = 1 + tid; i < len; i += RQR_THREADS) x[i] *= sc;
        __syncthreads();
        for (int c = j + 1 + wid; c < cols; c += nw) {
            T *col = A + j + (size_t)c * rows;
            T w = lane == 0 ? col[0] : T(0);
            for (int i = 1 + lane; i < len; i += 32) w = fma(x[i], col[i], w);
            w = warp_sum(w) * tv;
            if (lane == 0) col[0] -= w;
            for (int i = 1 + lane; i < len; i += 32) col[i] = fma(-x[i], w, col[i]);
        }
        __syncthreads();
    }
}

template <class T>
__global__ void __launch_bounds__(512) rform_q_kernel(int rows, int cols, const T *__restrict__ Y,
                                                      const T *__restrict__ tau, T *__restrict__ Q)
{
    const int f = blockIdx.x;
    Y += (size_t)f * rows * cols;
    tau += (size_t)f * cols;
    Q += (size_t)f * rows * cols;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int c = wid; c < cols; c += nw) {
        T *q = Q + (size_t)c * rows;
        for (int i = lane; i < rows; i += 32) q[i] = i == c ? T(1) : T(0);
        __syncwarp();
        // H_j leaves e_c alone for j > c
        for (int j = min(c, rows - 1); j >= 0; --j) {
            const T t = tau[j];
            if (t == 0) continue;
            const T *v = Y + (size_t)j * rows;
            T acc = lane == 0 ? q[j] : T(0);
            for (int i = j + 1 + lane; i < rows; i += 32) acc = fma(v[i], q[i], acc);
            acc = warp_sum(acc) * t;
            if (lane == 0) q[j] -= acc;
            for (int i = j + 1 + lane; i < rows; i += 32) q[i] = fma(-v[i], acc, q[i]);
            __syncwarp();
        }
    }
}

// The same QR over a cluster of CS CTAs per bin: CTA r owns columns
// [r cw, (r + 1) cw) in shared memory; per step the owner of column j forms the
// reflector and publishes it with tau (double-buffered by step parity), and
// after one cluster barrier every CTA copies it and updates its own columns
// > j.  rqr_kernel's arithmetic in the same order (512 threads, the same
// reductions): bitwise the same factors, with the trailing updates of a bin
// on CS SMs and in shared memory instead of on one SM from L2.
template <class T, int CS>
__global__ void __launch_bounds__(RQR_THREADS) rqr_cluster_kernel(int rows, int cols, T *A, T *tau)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int f = blockIdx.x / CS;
    const int cw = (cols + CS - 1) / CS, c0 = rank * cw;
    const int nown = cols - c0 < cw ? (cols - c0 > 0 ? cols - c0 : 0) : cw;
    extern __shared__ __align__(16) unsigned char rqc_raw[];
    T *colbuf = reinterpret_cast<T *>(rqc_raw);   // cw x rows: this CTA's columns
    T *xs = colbuf + (size_t)cw * rows;           // 2 x rows: the reflector, by step parity
    __shared__ T red[RQR_THREADS / 32];
    __shared__ T s_tau[2];
    __shared__ T s_scale;
    A += (size_t)f * rows * cols;
    tau += (size_t)f * cols;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = RQR_THREADS / 32;
    for (int e = tid; e < nown * rows; e += RQR_THREADS) colbuf[e] = A[(size_t)c0 * rows + e];
    __syncthreads();
    const int steps = cols < rows ? cols : rows;
    for (int j = 0; j < steps; ++j) {
        const int oj = j / cw, par = j & 1, len = rows - j;
        T *xb = xs + (size_t)par * rows;
        if (rank == oj) {
            T *x = colbuf + (size_t)(j - c0) * rows + j;
            T sg = 0;
            for (int i = 1 + tid; i < len; i += RQR_THREADS) sg = fma(x[i], x[i], sg);
            sg = warp_sum(sg);
            if (lane == 0) red[wid] = sg;
            __syncthreads();
            if (tid == 0) {
                T sigma = 0;
                for (int w = 0; w < nw; ++w) sigma += red[w];
                const T alpha = x[0];
                if (sigma == 0) {
                    s_tau[par] = 0;
                    s_scale = 0;
                } else {
                    const T nrm = sqrt(alpha * alpha + sigma);
                    const T beta = alpha >= 0 ? -nrm : nrm;
                    s_tau[par] = (beta - alpha) / beta;
                    s_scale = T(1) / (alpha - beta);
                    x[0] = beta;
                }
                tau[j] = s_tau[par];
            }
            __syncthreads();
            if (s_tau[par] != 0) {
                const T sc = s_scale;
                for (int i = 1 + tid; i < len; i += RQR_THREADS) {
                    const T v = x[i] * sc;
                    x[i] = v;
                    xb[j + i] = v;
                }
            }
        }
        cluster.sync();
        const T tv = *cluster.map_shared_rank(&s_tau[par], oj);
        if (tv != 0) {
            if (rank != oj) {
                const T *ox = cluster.map_shared_rank(xb, oj);
                for (int i = j + 1 + tid; i < rows; i += RQR_THREADS) xb[i] = ox[i];
            }
            __syncthreads();
            const T *x = xb + j;   // x[0] = 1 implicitly
            for (int cl = wid; cl < nown; cl += nw) {
                if (c0 + cl <= j) continue;
                T *col = colbuf + (size_t)cl * rows + j;
                T w = lane == 0 ? col[0] : T(0);
                for (int i = 1 + lane; i < len; i += 32) w = fma(x[i], col[i], w);
                w = warp_sum(w) * tv;
                if (lane == 0) col[0] -= w;
                for (int i = 1 + lane; i < len; i += 32) col[i] = fma(-x[i], w, col[i]);
            }
        }
        __syncthreads();
    }
    cluster.sync();   // no CTA leaves while another may read its reflector or tau
    for (int e = tid; e < nown * rows; e += RQR_THREADS) A[(size_t)c0 * rows + e] = colbuf[e];
}

template <class T, int CS>
static bool rqr_cluster_launch(ia_context *ctx, int rows, int cols, T *Y, T *tau, int batch, bool one_wave, int &st)
{
    const int cw = (cols + CS - 1) / CS;
    const size_t smem = sizeof(T) * ((size_t)cw * rows + 2 * (size_t)rows);
    if (cw < 1 || smem > 200 * 1024 || (one_wave && CS * batch > ctx->sm_count)) return false;
    st = IA_OK;
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024)
        e = cudaFuncSetAttribute(rqr_cluster_kernel<T, CS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) {
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3((unsigned)(CS * batch));
        lc.blockDim = dim3(RQR_THREADS);
        lc.dynamicSmemBytes = smem;
        lc.stream = ctx->stream;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = CS;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        lc.attrs = at;
        lc.numAttrs = 1;
        e = cudaLaunchKernelEx(&lc, rqr_cluster_kernel<T, CS>, rows, cols, Y, tau);
    }
    if (e != cudaSuccess) st = cuda_status(e);
    return true;
}

// The same explicit factor over column groups: CTA (g, f) forms columns
// [FQ_COLS g, FQ_COLS (g + 1)) of bin f's Q, a warp per column held in shared
// memory; each reflector j (from the group's last column down to 0) is staged
// in shared memory once and applied by every warp whose column c >= j.  The
// operations per column are rform_q_kernel's, in the same order (bitwise the
// same Q); a bin's columns spread over cols / FQ_COLS CTAs instead of one,
// and a reflector is read from L2 once per CTA instead of once per warp.
constexpr int FQ_COLS = 16;

template <class T>
__global__ void __launch_bounds__(32 * FQ_COLS) rform_q_group_kernel(int rows, int cols, const T *__restrict__ Y,
                                                                     const T *__restrict__ tau, T *__restrict__ Q)
{
    extern __shared__ __align__(16) unsigned char fq_raw[];
    T *qs = reinterpret_cast<T *>(fq_raw);   // FQ_COLS x rows: the group's columns
    T *vs = qs + (size_t)FQ_COLS * rows;     // rows: the current reflector
    const int f = blockIdx.y, c0 = blockIdx.x * FQ_COLS;
    Y += (size_t)f * rows * cols;
    tau += (size_t)f * cols;
    Q += (size_t)f * rows * cols;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int c = c0 + wid;
    T *q = qs + (size_t)wid * rows;
    for (int i = lane; i < rows; i += 32) q[i] = i == c ? T(1) : T(0);
    const int ctop = (c0 + FQ_COLS < cols ? c0 + FQ_COLS : cols) - 1;
    for (int j = ctop < rows - 1 ? ctop : rows - 1; j >= 0; --j) {
        __syncthreads();   // every warp is done with the previous reflector
        for (int i = j + 1 + (int)threadIdx.x; i < rows; i += blockDim.x) vs[i] = Y[i + (size_t)j * rows];
        __syncthreads();
        const T t = tau[j];
        if (t == 0 || c >= cols || j > c) continue;   // H_j leaves e_c alone for j > c
        T acc = lane == 0 ? q[j] : T(0);
        for (int i = j + 1 + lane; i < rows; i += 32) acc = fma(vs[i], q[i], acc);
        acc = warp_sum(acc) * t;
        if (lane == 0) q[j] -= acc;
        for (int i = j + 1 + lane; i < rows; i += 32) q[i] = fma(-vs[i], acc, q[i]);
    }
    __syncwarp();
    if (c < cols)
        for (int i = lane; i < rows; i += 32) Q[i + (size_t)c * rows] = q[i];
}

// Q = orth(Y): QR of Y in place, then the explicit thin factor into Q
template <class T>
static int orthonormalise(ia_context *ctx, int rows, int cols, T *Y, T *tau, T *Q, int batch)
{
    // the QR: over a cluster of 8, 4 or 2 CTAs per bin -- the largest whose
    // clusters fit on the SMs in one wave, else the smallest whose column
    // share fits shared memory, in several waves (with the columns in shared
    // memory a cluster step is far faster than the one-CTA kernel's from L2:
    // 0.12 against 4.1 ms per 16-bin launch at 1284 x 128) -- else one CTA
    // per bin
    int st = IA_OK;
    if (!(rqr_cluster_launch<T, 8>(ctx, rows, cols, Y, tau, batch, true, st) ||
          rqr_cluster_launch<T, 4>(ctx, rows, cols, Y, tau, batch, true, st) ||
          rqr_cluster_launch<T, 2>(ctx, rows, cols, Y, tau, batch, true, st) ||
          rqr_cluster_launch<T, 2>(ctx, rows, cols, Y, tau, batch, false, st) ||
          rqr_cluster_launch<T, 4>(ctx, rows, cols, Y, tau, batch, false, st) ||
          rqr_cluster_launch<T, 8>(ctx, rows, cols, Y, tau, batch, false, st)))
        rqr_kernel<T><<<batch, RQR_THREADS, 0, ctx->stream>>>(rows, cols, Y, tau);
    if (st) return st;
    IA_LAUNCH_CHECK(ctx);
    const size_t fsm = sizeof(T) * (size_t)(FQ_COLS + 1) * rows;
    if (fsm <= 200 * 1024) {
        if (fsm > 48 * 1024)
            IA_CUDA_TRY(cudaFuncSetAttribute(rform_q_group_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)fsm));
        dim3 g((cols + FQ_COLS - 1) / FQ_COLS, batch);
        rform_q_group_kernel<T><<<g, 32 * FQ_COLS, fsm, ctx->stream>>>(rows, cols, Y, tau, Q);
    } else {
        rform_q_kernel<T><<<batch, 512, 0, ctx->stream>>>(rows, cols, Y, tau, Q);
    }
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// --------------------------------------------------------------------------
// small helpers
// --------------------------------------------------------------------------
// deterministic start block, entries uniform in [-1, 1) from an integer hash
// of (row, column) (a 32-bit avalanche mix: xorshift-multiply rounds)
__device__ __forceinline__ unsigned mix32(unsigned h)
{
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    h *= 0x846ca68bu;
    h ^= h >> 16;
    return h;
}

template <class T>
__global__ void start_block_kernel(int rows, int cols, T *Q, int batch)
{
    const size_t per = (size_t)rows * cols;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < per * batch; e += (size_t)gridDim.x * blockDim.x) {
        const unsigned h = mix32((unsigned)(e % per) * 2654435761u + 0x9e3779b9u);
        Q[e] = (T)((double)h * (2.0 / 4294967296.0) - 1.0);
    }
}

template <class TI, class TO>
__global__ void convert_kernel(size_t count, const TI *__restrict__ in, TO *__restrict__ out)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        out[e] = (TO)in[e];
}

template <class TI, class TO>
static int convert(ia_context *ctx, size_t count, const TI *in, TO *out)
{
    const size_t want = (count + 255) / 256, cap = (size_t)ctx->sm_count * 16;
    const int blocks = (int)(want < cap ? want : cap);
    if (blocks <= 0) return IA_OK;
    convert_kernel<TI, TO><<<blocks, 256, 0, ctx->stream>>>(count, in, out);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// Bc = (B + B^T) / 2 as complex, b x b per matrix
__global__ void sym_complex_kernel(int b, const double *__restrict__ B, double2 *__restrict__ Bc, int batch)
{
    const size_t per = (size_t)b * b;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < per * batch; e += (size_t)gridDim.x * blockDim.x) {
        const size_t f = e / per, o = e % per;
        const int i = (int)(o % b), j = (int)(o / b);
        const double *Bf = B + f * per;
        Bc[e] = make_double2(0.5 * (Bf[i + (size_t)j * b] + Bf[j + (size_t)i * b]), 0.0);
    }
}

// Ritz values lambda_j = w_j^T B w_j and real Ritz coefficient vectors
// W (b x nm) from the right singular vectors of the symmetric B (real
// matrices keep Jacobi rotations real).  One CTA per matrix, warp per column.
// X <- I for every bin (b x b complex)
__global__ void eye_c_kernel(int b, double2 *__restrict__ X, int batch)
{
    const size_t per = (size_t)b * b;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < per * batch; e += (size_t)gridDim.x * blockDim.x) {
        const size_t o = e % per;
        X[e] = make_double2((o % b) == (o / b) ? 1.0 : 0.0, 0.0);
    }
}

// Two-sided Jacobi eigensolver of the real symmetric b x b Rayleigh-Ritz
// matrix B (symmetrised), one CTA per bin: herm_jacobi_kernel's sweeps
// (every pair checked at once, only rounds holding a pair above tol = 2 N eps
// max|S_ii| run, pairs with both diagonal entries below the floor N eps
// max|S_ii| skipped, Rutishauser's stable rotation, a round's rotations
// applied to columns then rows over the whole CTA) in real arithmetic, with S
// in shared memory and the eigenvectors accumulated into X (global) from the
// identity; LAM <- diag(S), unsorted.
constexpr int RJ_THREADS = 512;

// round-robin (circle) ordering: pair k of round `round` over N2 (even) slots
__device__ __forceinline__ void rr_pair_r(int N2, int round, int k, int &i, int &j)
{
    if (k == 0) {
        i = round;
        j = N2 - 1;
    } else {
        i = round + k;
        if (i >= N2 - 1) i -= N2 - 1;
        j = round - k + N2 - 1;
        if (j >= N2 - 1) j -= N2 - 1;
    }
    if (i > j) {
        const int t = i;
        i = j;
        j = t;
    }
}

__global__ void __launch_bounds__(RJ_THREADS) rsym_jacobi_kernel(int N, const double *__restrict__ B,
                                                                 double *__restrict__ X, double *__restrict__ LAM,
                                                                 int max_sweeps, int *__restrict__ info)
{
    extern __shared__ __align__(16) double rj_sm[];
    const int N2 = N + (N & 1), P = N2 / 2;
    double *S = rj_sm;                                   // N x N
    double *cs = S + (size_t)N * N;                      // P
    double *sp = cs + P;                                 // P
    double *dg = sp + P;                                 // N: diag(S) at the sweep's start
    int *pi = reinterpret_cast<int *>(dg + N);           // P
    int *pj = pi + P;                                    // P
    int *rflag = pj + P;                                 // N2 - 1
    __shared__ double red[RJ_THREADS / 32];
    __shared__ int s_rot, s_nact;
    const int f = blockIdx.x;
    B += (size_t)f * N * N;
    X += (size_t)f * N * N;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    for (int e = tid; e < N * N; e += blockDim.x) {
        const int i = e % N, j = e / N;
        S[e] = 0.5 * (B[e] + B[j + (size_t)i * N]);
        X[e] = i == j ? 1.0 : 0.0;
    }
    __syncthreads();
    double lm = 0.0;
    for (int i = tid; i < N; i += blockDim.x) lm = fmax(lm, fabs(S[i + (size_t)i * N]));
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
    const double tol = 2.0 * (double)N * 2.220446049250313e-16 * red[0], floor2 = 0.5 * tol;
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        for (int r = tid; r < N2 - 1; r += blockDim.x) rflag[r] = 0;
        for (int i = tid; i < N; i += blockDim.x) dg[i] = S[i + (size_t)i * N];
        if (tid == 0) {
            s_rot = 0;
            s_nact = 0;
        }
        __syncthreads();
        for (int e = tid; e < (N2 - 1) * P; e += blockDim.x) {
            const int round = e / P, k = e - round * P;
            int i, j;
            rr_pair_r(N2, round, k, i, j);
            if (j >= N || (dg[i] < floor2 && dg[j] < floor2)) continue;
            if (fabs(S[i + (size_t)j * N]) > tol) rflag[round] = 1;
        }
        __syncthreads();
        for (int round = 0; round < N2 - 1; ++round) {
            if (!rflag[round]) continue;
            int mine = 0;
            for (int k = tid; k < P; k += blockDim.x) {
                int i, j;
                rr_pair_r(N2, round, k, i, j);
                if (j >= N) continue;
                const double g0 = S[i + (size_t)j * N], g = fabs(g0);
                if (!(g > tol)) continue;
                const double a = S[i + (size_t)i * N], b = S[j + (size_t)j * N];
                if (a < floor2 && b < floor2) continue;
                const double zeta = (b - a) / (2.0 * g);
                const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / sqrt(1.0 + t * t);
                const int slot = atomicAdd(&s_nact, 1);
                cs[slot] = c;
                sp[slot] = t * c * g0 / g;
                pi[slot] = i;
                pj[slot] = j;
                ++mine;
            }
            if (mine) atomicAdd(&s_rot, mine);
            if (!__syncthreads_or(mine)) continue;
            const int nact = s_nact;
            // columns of S and X: [u v] <- [u v] G
            for (int e = tid; e < nact * 2 * N; e += blockDim.x) {
                const int q = e / (2 * N), rem = e - q * 2 * N, mat = rem / N, r = rem - mat * N;
                const int i = pi[q], j = pj[q];
                const double c = cs[q], w = sp[q];
                double *M = mat == 0 ? S : X;
                double *ci = M + (size_t)i * N, *cj = M + (size_t)j * N;
                const double u = ci[r], v = cj[r];
                ci[r] = c * u - w * v;
                cj[r] = c * v + w * u;
            }
            __syncthreads();
            if (tid == 0) s_nact = 0;
            // rows of S: [u; v] <- G^T [u; v]
            for (int e = tid; e < nact * N; e += blockDim.x) {
                const int q = e / N, col = e - q * N;
                const int i = pi[q], j = pj[q];
                const double c = cs[q], w = sp[q];
                double *a = S + i + (size_t)col * N, *b = S + j + (size_t)col * N;
                const double u = *a, v = *b;
                *a = c * u - w * v;
                *b = c * v + w * u;
            }
            __syncthreads();
        }
        const int total = s_rot;
        __syncthreads();
        if (total == 0) break;
    }
    if (tid == 0 && sweep >= max_sweeps && info) atomicOr(&info[f], IA_INFO_NOCONV);
    for (int i = tid; i < N; i += blockDim.x) LAM[(size_t)f * N + i] = S[i + (size_t)i * N];
}

static size_t rsym_jacobi_smem(int N)
{
    const int N2 = N + (N & 1), P = N2 / 2;
    return sizeof(double) * ((size_t)N * N + 2 * (size_t)P + N) + sizeof(int) * (2 * (size_t)P + N2);
}

// V (complex, zero imaginary parts) <- the columns of the real X ordered by
// decreasing eigenvalue lam (ties by index), one CTA per bin
__global__ void sort_eig_real_kernel(int b, const double *__restrict__ lam, const double *__restrict__ X,
                                     double2 *__restrict__ V)
{
    extern __shared__ int ser_rank[];
    const int f = blockIdx.x;
    lam += (size_t)f * b;
    X += (size_t)f * b * b;
    V += (size_t)f * b * b;
    for (int i = threadIdx.x; i < b; i += blockDim.x) {
        const double li = lam[i];
        int rk = 0;
        for (int j = 0; j < b; ++j) {
            const double lj = lam[j];
            if (lj > li || (lj == li && j < i)) ++rk;
        }
        ser_rank[i] = rk;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
        const int i = e / b, r = e - i * b;
        V[r + (size_t)ser_rank[i] * b] = make_double2(X[e], 0.0);
    }
}

// V <- the columns of X ordered by decreasing eigenvalue lam (ties by index),
// one CTA per bin
__global__ void sort_eig_kernel(int b, const double *__restrict__ lam, const double2 *__restrict__ X,
                                double2 *__restrict__ V)
{
    extern __shared__ int se_rank[];
    const int f = blockIdx.x;
    lam += (size_t)f * b;
    X += (size_t)f * b * b;
    V += (size_t)f * b * b;
    for (int i = threadIdx.x; i < b; i += blockDim.x) {
        const double li = lam[i];
        int rk = 0;
        for (int j = 0; j < b; ++j) {
            const double lj = lam[j];
            if (lj > li || (lj == li && j < i)) ++rk;
        }
        se_rank[i] = rk;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
        const int i = e / b, r = e - i * b;
        V[r + (size_t)se_rank[i] * b] = X[e];
    }
}

__global__ void ritz_kernel(int b, int nm, const double *__restrict__ B, const double2 *__restrict__ V,
                            double *__restrict__ lambda, double *__restrict__ W)
{
    const int f = blockIdx.x;
    B += (size_t)f * b * b;
    V += (size_t)f * b * b;
    W += (size_t)f * b * nm;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = wid; j < nm; j += nw) {
        const double2 *v = V + (size_t)j * b;
        double acc = 0.0;
        for (int r = lane; r < b; r += 32) {
            double br = 0.0;
            for (int c = 0; c < b; ++c) br = fma(B[r + (size_t)c * b], v[c].x, br);
            acc = fma(v[r].x, br, acc);
            W[r + (size_t)j * b] = v[r].x;
        }
        acc = warp_sum(acc);
        if (lane == 0) lambda[(size_t)f * nm + j] = acc;
    }
}

// sign convention: the first component whose magnitude is within 1e-6 of the
// largest is made positive (symmetric geometries give modes with components
// of equal magnitude and opposite sign; the 1e-6 band keeps the choice off
// rounding noise).  Non-finite values flag IA_INFO_NONFINITE.
__global__ void mode_sign_kernel(int n, int nm, double *__restrict__ X, const double *__restrict__ lambda,
                                 int *__restrict__ info)
{
    const int f = blockIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    bool bad = false;
    for (int j = wid; j < nm; j += nw) {
        double *x = X + ((size_t)f * nm + j) * n;
        double best = 0.0;
        for (int i = lane; i < n; i += 32) {
            const double a = fabs(x[i]);
            if (!(a == a) || isinf(a)) bad = true;
            best = fmax(best, a);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, o));
        const double thr = best * (1.0 - 1e-6);
        int bi = n;
        for (int i = lane; i < n; i += 32)
            if (fabs(x[i]) >= thr) { bi = i; break; }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) bi = min(bi, __shfl_xor_sync(0xffffffffu, bi, o));
        const bool flip = bi < n && x[bi] < 0.0;
        __syncwarp();
        if (flip)
            for (int i = lane; i < n; i += 32) x[i] = -x[i];
        const double l = lambda[(size_t)f * nm + j];
        if (!(l == l) || isinf(l)) bad = true;
    }
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0 && info && bad) info[f] |= IA_INFO_NONFINITE;
}

size_t radiation_modes_ws_bytes(int n, int F, int nm, const ia_config *cfg, bool gram)
{
    const size_t b = (size_t)min(n, nm + max(0, cfg->mode_oversample));
    const size_t nb = (size_t)n * b * F, bb = b * b * F;
    size_t s = 4 * ws_round(8 * nb) + ws_round(8 * b * F) + ws_round(8 * bb) + 4 * ws_round(16 * bb) +
               ws_round(8 * b * F) + ws_round(8 * b * (size_t)nm * F);
    if (cfg->precision == IA_PREC_MIXED)
        s += ws_round(4 * (size_t)n * n * F) + 3 * ws_round(4 * nb) + ws_round(4 * b * F);
    (void)gram;
    return s + 4096;
}

// gram: the operator is R R^T (R general, n x n): its eigenpairs are the left
// singular vectors and the squared singular values of R
int radiation_modes_batched(ia_context *ctx, int n, int F, const double *R, int nm, const ia_config *cfg,
                            double *lambda, double *modes, int *info, WsCursor &cur, bool gram)
{
    const int b = min(n, nm + max(0, cfg->mode_oversample));
    const bool mixed = cfg->precision == IA_PREC_MIXED;
    const long long nn = (long long)n * n, nb = (long long)n * b, bb = (long long)b * b;
    double *Q = cur.take<double>(nb * F);
    double *Y = cur.take<double>(nb * F);
    double *Y2 = cur.take<double>(nb * F);
    double *Tg = cur.take<double>(nb * F);
    // Yo = op Qi at FP64 accuracy, op = R or R R^T
    auto apply64 = [&](const double *Qi, double *Yo) -> int {
        if (!gram) return prod64(ctx, mixed, OP_N, n, b, n, R, n, nn, Qi, n, nb, Yo, n, nb, F);
        int s2 = prod64(ctx, mixed, OP_T, n, b, n, R, n, nn, Qi, n, nb, Tg, n, nb, F);
        return s2 ? s2 : prod64(ctx, mixed, OP_N, n, b, n, R, n, nn, Tg, n, nb, Yo, n, nb, F);
    };
    double *tau = cur.take<double>((size_t)b * F);
    double *B = cur.take<double>(bb * F);
    double2 *Bc = cur.take<double2>(bb * F);
    double2 *Vc = cur.take<double2>(bb * F);
    double2 *Ysvd = cur.take<double2>(bb * F);
    double2 *Vacc = cur.take<double2>(bb * F);
    double *s = cur.take<double>((size_t)b * F);
    double *Wr = cur.take<double>((size_t)b * nm * F);
    int st;
    const int blocks = ctx->sm_count * 8;
    int steps64 = max(0, cfg->mode_iters);
    if (mixed) {
        float *R32 = cur.take<float>(nn * F);
        float *Q32 = cur.take<float>(nb * F);
        float *Y32 = cur.take<float>(nb * F);
        float *tau32 = cur.take<float>((size_t)b * F);
        float *T32 = cur.take<float>(nb * F);
        if ((st = convert(ctx, (size_t)nn * F, R, R32))) return st;
        start_block_kernel<float><<<blocks, 256, 0, ctx->stream>>>(n, b, Q32, F);
        IA_LAUNCH_CHECK(ctx);
        for (int t = 0; t < cfg->mode_iters; ++t) {
            const float *src = Q32;
            if (gram) {
                if ((st = rgemm_batched<float>(ctx, OP_T, n, b, n, 1.f, R32, n, nn, Q32, n, nb, 0.f, T32, n, nb, F)))
                    return st;
                src = T32;
            }
            if ((st = rgemm_batched<float>(ctx, OP_N, n, b, n, 1.f, R32, n, nn, src, n, nb, 0.f, Y32, n, nb, F)))
                return st;
            if ((st = orthonormalise<float>(ctx, n, b, Y32, tau32, Q32, F))) return st;
        }
        if ((st = convert(ctx, (size_t)nb * F, Q32, Q))) return st;
        steps64 = max(1, cfg->refine_steps);
    } else {
        start_block_kernel<double><<<blocks, 256, 0, ctx->stream>>>(n, b, Q, F);
        IA_LAUNCH_CHECK(ctx);
    }
    for (int t = 0; t < steps64; ++t) {
        if ((st = apply64(Q, Y))) return st;
        if ((st = orthonormalise<double>(ctx, n, b, Y, tau, Q, F))) return st;
    }
    // Rayleigh-Ritz: B = Q^T op Q, eigenpairs of B, modes = Q W
    if ((st = apply64(Q, Y2))) return st;
    if ((st = prod64(ctx, mixed, OP_T, b, b, n, Q, n, nb, Y2, n, nb, B, b, bb, F))) return st;
    // eigenpairs of the symmetric (positive semidefinite) B by the two-sided
    // FP64 Jacobi, eigenvectors accumulated from the identity, then ordered by
    // decreasing eigenvalue (was: a one-sided complex Jacobi SVD with a
    // rotation accumulator, 28.8 of 55.8 ms for the 16-bin BEM modes): in real
    // arithmetic with B in shared memory when it fits, else the complex
    // Hermitian kernel on a copy
    const size_t rjs = rsym_jacobi_smem(b);
    if (rjs <= 200 * 1024) {
        double *Xr = reinterpret_cast<double *>(Ysvd);
        if (rjs > 48 * 1024)
            IA_CUDA_TRY(cudaFuncSetAttribute(rsym_jacobi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rjs));
        rsym_jacobi_kernel<<<F, RJ_THREADS, rjs, ctx->stream>>>(b, B, Xr, s, 16, info);
        IA_LAUNCH_CHECK(ctx);
        sort_eig_real_kernel<<<F, 256, sizeof(int) * (size_t)b, ctx->stream>>>(b, s, Xr, Vc);
        IA_LAUNCH_CHECK(ctx);
    } else {
        sym_complex_kernel<<<blocks, 256, 0, ctx->stream>>>(b, B, Bc, F);
        IA_LAUNCH_CHECK(ctx);
        eye_c_kernel<<<blocks, 256, 0, ctx->stream>>>(b, Ysvd, F);
        IA_LAUNCH_CHECK(ctx);
        if ((st = herm_jacobi_batched(ctx, b, Bc, Ysvd, s, 16, F, info))) return st;
        sort_eig_kernel<<<F, 256, sizeof(int) * (size_t)b, ctx->stream>>>(b, s, Ysvd, Vc);
        IA_LAUNCH_CHECK(ctx);
    }
    (void)Vacc;
    ritz_kernel<<<F, 256, 0, ctx->stream>>>(b, nm, B, Vc, lambda, Wr);
    IA_LAUNCH_CHECK(ctx);
    if ((st = prod64(ctx, mixed, OP_N, n, nm, b, Q, n, nb, Wr, b, (long long)b * nm, modes, n, (long long)n * nm, F)))
        return st;
    mode_sign_kernel<<<F, 256, 0, ctx->stream>>>(n, nm, modes, lambda, info);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// --------------------------------------------------------------------------
// Sound power W = 1/2 Re(v^H R v) = 1/2 (a^T R a + b^T R b) for v = a + i b and
// symmetric R.  Stage 1: CTA per (64-column block, frequency), thread per row,
// partial sums per right-hand side; stage 2 adds the column blocks in a fixed
// order (deterministic).
// --------------------------------------------------------------------------
constexpr int SP_COLS = 64;
constexpr int SP_RHS = 8;

__global__ void __launch_bounds__(256) sound_power_partial_kernel(int n, const double *__restrict__ R, int nrhs,
                                                                   int r0, int nr, const double2 *__restrict__ v,
                                                                   double *__restrict__ part)
{
    __shared__ double2 sv[SP_RHS][SP_COLS];
    __shared__ double red[SP_RHS][8];
    const int f = blockIdx.y, jb = blockIdx.x, j0 = jb * SP_COLS;
    const size_t nn = (size_t)n * n;
    R += f * nn;
    v += (size_t)f * n * nrhs;
    for (int e = threadIdx.x; e < SP_RHS * SP_COLS; e += blockDim.x) {
        const int r = e / SP_COLS, jl = e % SP_COLS, j = j0 + jl;
        sv[r][jl] = (r < nr && j < n) ? v[j + (size_t)(r0 + r) * n] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    const int jn = min(SP_COLS, n - j0);
    double acc[SP_RHS];
#pragma unroll
    for (int r = 0; r < SP_RHS; ++r) acc[r] = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double2 t[SP_RHS];
#pragma unroll
        for (int r = 0; r < SP_RHS; ++r) t[r] = make_double2(0.0, 0.0);
        for (int jl = 0; jl < jn; ++jl) {
            const double rij = R[i + (size_t)(j0 + jl) * n];
#pragma unroll
            for (int r = 0; r < SP_RHS; ++r) {
                t[r].x = fma(rij, sv[r][jl].x, t[r].x);
                t[r].y = fma(rij, sv[r][jl].y, t[r].y);
            }
        }
#pragma unroll
        for (int r = 0; r < SP_RHS; ++r) {
            if (r >= nr) break;
            const double2 vi = v[i + (size_t)(r0 + r) * n];
            acc[r] = fma(vi.x, t[r].x, fma(vi.y, t[r].y, acc[r]));
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int r = 0; r < SP_RHS; ++r) {
        const double w = warp_sum(acc[r]);
        if (lane == 0) red[r][wid] = w;
    }
    __syncthreads();
    if (threadIdx.x < nr) {
        double w = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) w += red[threadIdx.x][k];
        part[((size_t)f * gridDim.x + jb) * SP_RHS + threadIdx.x] = w;
    }
}

__global__ void sound_power_sum_kernel(int F, int nblk, int nrhs, int r0, int nr, const double *__restrict__ part,
                                       double *__restrict__ W)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= F * nr) return;
    const int f = e / nr, r = e % nr;
    double w = 0.0;
    for (int k = 0; k < nblk; ++k) w += part[((size_t)f * nblk + k) * SP_RHS + r];
    W[(size_t)f * nrhs + r0 + r] = 0.5 * w;
}

int sound_power_batched(ia_context *ctx, int n, int F, const double *R, int nrhs, const double2 *v, double *W,
                        WsCursor &cur)
{
    const int nblk = (n + SP_COLS - 1) / SP_COLS;
    double *part = cur.take<double>((size_t)F * nblk * SP_RHS);
    for (int r0 = 0; r0 < nrhs; r0 += SP_RHS) {
        const int nr = min(SP_RHS, nrhs - r0);
        sound_power_partial_kernel<<<dim3(nblk, F), 256, 0, ctx->stream>>>(n, R, nrhs, r0, nr, v, part);
        IA_LAUNCH_CHECK(ctx);
        sound_power_sum_kernel<<<(F * nr + 255) / 256, 256, 0, ctx->stream>>>(F, nblk, nrhs, r0, nr, part, W);
        IA_LAUNCH_CHECK(ctx);
    }
    return IA_OK;
}

size_t sound_power_ws_bytes(int n, int F) { return ws_round(8 * (size_t)F * ((n + SP_COLS - 1) / SP_COLS) * SP_RHS) + 256; }

}  // namespace ia
