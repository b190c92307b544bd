// Double-float complex GEMM: C = alpha op(A) op(B) + beta C for FP64
// operands, with every product and sum carried as an unevaluated pair of FP32
// values (hi + lo, ~48-bit significand).  GB300 issues FP32 at ~64x its FP64
// rate, so this runs several times faster than an FP64 GEMM while keeping the
// residuals, transfer products and eigen-refinement products of the mixed
// path at FP64-level accuracy (about 1e-13 relative over K = 642 sums).
//
// Products use the error-free transformation p + e = x_hi y_hi (fmaf), plus
// the cross terms x_hi y_lo + x_lo y_hi; sums use TwoSum on the high word with
// the low word accumulated and renormalised after each K tile (Dekker 1971;
// Hida, Li, Bailey 2001).  Tiles of 64 x 64, 32 x 32 or 64 x 32 outputs (the
// autotuner picks per shape; all sum k in the same order), K tile 8, 256
// threads, operands split to (hi, lo) on the way into shared memory.
// op(A), op(B) in {N, C} (C = conjugate transpose).
#include <type_traits>
#include "ia_common.cuh"
#include "ia_internal.h"
#include "tune.h"

namespace ia {

constexpr int DF_K = 8;

struct df2 {   // complex double-float accumulator
    float rh, rl, ih, il;
};

__device__ __forceinline__ float4 split_c(double2 v, bool conj)
{
    if (conj) v.y = -v.y;
    float rh = __double2float_rn(v.x), ih = __double2float_rn(v.y);
    float rl = __double2float_rn(v.x - (double)rh), il = __double2float_rn(v.y - (double)ih);
    return make_float4(rh, ih, rl, il);
}

// an operand element as (re hi, im hi, re lo, im lo): split from FP64 on the
// way in, or already split (float4 operands, no FP64 instructions)
__device__ __forceinline__ float4 ld_df(const double2 *P, size_t i, bool conj) { return split_c(P[i], conj); }
__device__ __forceinline__ float4 ld_df(const float4 *P, size_t i, bool conj)
{
    float4 v = P[i];
    if (conj) {
        v.y = -v.y;
        v.w = -v.w;
    }
    return v;
}

// (ah, al) += (xh + xl)(yh + yl), low word renormalised later
__device__ __forceinline__ void df_mac(float &ah, float &al, float xh, float xl, float yh, float yl)
{
    float p = xh * yh;
    float e = fmaf(xh, yh, -p);
    e = fmaf(xh, yl, e);
    e = fmaf(xl, yh, e);
    float s = ah + p;
    float v = s - ah;
    float err = (ah - (s - v)) + (p - v);
    ah = s;
    al += err + e;
}

__device__ __forceinline__ void df_norm(float &ah, float &al)
{
    float s = ah + al;
    al = al - (s - ah);
    ah = s;
}

template <int BM, int BN, int TM, int TN, class TA, class TB>
__global__ void __launch_bounds__(256) dfgemm_kernel(int opa, int opb, int M, int N, int K, double alpha,
                                                     const TA *__restrict__ A, int lda, long long sA,
                                                     const TB *__restrict__ B, int ldb, long long sB,
                                                     double beta, double2 *__restrict__ C, int ldc, long long sC)
{
    constexpr int NTX = BN / TN, NTY = BM / TM;
    static_assert(NTX * NTY == 256, "256 threads per tile");
    __shared__ float4 As[DF_K][BM];
    __shared__ float4 Bs[DF_K][BN];
    const int f = blockIdx.z;
    A += f * sA;
    B += f * sB;
    C += f * sC;
    const int tx = threadIdx.x % NTX, ty = threadIdx.x / NTX;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    df2 acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = df2{0.f, 0.f, 0.f, 0.f};
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k0 = 0; k0 < K; k0 += DF_K) {
#pragma unroll
        for (int e = threadIdx.x; e < DF_K * BM; e += 256) {
            int r, kk;
            if (opa == OP_N) { r = e % BM; kk = e / BM; }
            else { kk = e % DF_K; r = e / DF_K; }
            int gr = m0 + r, gk = k0 + kk;
            float4 v = z4;
            if (gr < M && gk < K)
                v = opa == OP_N ? ld_df(A, gr + (size_t)gk * lda, false) : ld_df(A, gk + (size_t)gr * lda, true);
            As[kk][r] = v;
        }
#pragma unroll
        for (int e = threadIdx.x; e < DF_K * BN; e += 256) {
            int kk, c;
            if (opb == OP_N) { kk = e % DF_K; c = e / DF_K; }
            else { c = e % BN; kk = e / BN; }
            int gk = k0 + kk, gc = n0 + c;
            float4 v = z4;
            if (gk < K && gc < N)
                v = opb == OP_N ? ld_df(B, gk + (size_t)gc * ldb, false) : ld_df(B, gc + (size_t)gk * ldb, true);
            Bs[kk][c] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < DF_K; ++kk) {
            float4 a[TM], b[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + NTY * i];
#pragma unroll
            for (int j = 0; j < TN; ++j) b[j] = Bs[kk][tx + NTX * j];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) {
                    // a = (x: re_h, y: im_h, z: re_l, w: im_l)
                    df2 &c = acc[i][j];
                    df_mac(c.rh, c.rl, a[i].x, a[i].z, b[j].x, b[j].z);
                    df_mac(c.rh, c.rl, -a[i].y, -a[i].w, b[j].y, b[j].w);
                    df_mac(c.ih, c.il, a[i].x, a[i].z, b[j].y, b[j].w);
                    df_mac(c.ih, c.il, a[i].y, a[i].w, b[j].x, b[j].z);
                }
        }
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j) {
                df_norm(acc[i][j].rh, acc[i][j].rl);
                df_norm(acc[i][j].ih, acc[i][j].il);
            }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        int r = m0 + ty + NTY * i;
        if (r >= M) continue;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            int c = n0 + tx + NTX * j;
            if (c >= N) continue;
            double2 v = make_double2(alpha * ((double)acc[i][j].rh + (double)acc[i][j].rl),
                                     alpha * ((double)acc[i][j].ih + (double)acc[i][j].il));
            double2 *p = C + r + (size_t)c * ldc;
            if (beta != 0.0) {
                double2 o = *p;
                v.x = fma(beta, o.x, v.x);
                v.y = fma(beta, o.y, v.y);
            }
            *p = v;
        }
    }
}

template <int BM, int BN, int TM, int TN, class TA, class TB>
static int dfgemm_launch(ia_context *ctx, Op opa, Op opb, int M, int N, int K, double alpha, const TA *A, int lda,
                         long long sA, const TB *B, int ldb, long long sB, double beta, double2 *C, int ldc,
                         long long sC, int batch)
{
    dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, batch);
    dfgemm_kernel<BM, BN, TM, TN, TA, TB>
        <<<grid, 256, 0, ctx->stream>>>(opa, opb, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// tile variants: 64x64 (4x4 per thread), 32x32 (2x2), 64x32 (4x2)
template <class TA, class TB>
static int dfgemm_any(ia_context *ctx, Op opa, Op opb, int M, int N, int K, double alpha, const TA *A, int lda,
                      long long sA, const TB *B, int ldb, long long sB, double beta, double2 *C, int ldc, long long sC,
                      int batch)
{
    if (M <= 0 || N <= 0 || batch <= 0) return IA_OK;
    if ((opa != OP_N && opa != OP_C) || (opb != OP_N && opb != OP_C)) return IA_ERR_ARG;
    auto launch = [&](int v, double2 *Cout) -> int {
        switch (v) {
        case 1: return dfgemm_launch<32, 32, 2, 2>(ctx, opa, opb, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, Cout,
                                                   ldc, sC, batch);
        case 2: return dfgemm_launch<64, 32, 4, 2>(ctx, opa, opb, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, Cout,
                                                   ldc, sC, batch);
        default: return dfgemm_launch<64, 64, 4, 4>(ctx, opa, opb, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta,
                                                    Cout, ldc, sC, batch);
        }
    };
    TuneKey key{};
    key.kernel = std::is_same<TA, float4>::value ? TK_DFGEMM4 : TK_DFGEMM;
    key.v[0] = opa;
    key.v[1] = opb;
    key.v[2] = M;
    key.v[3] = N;
    key.v[4] = K;
    key.v[5] = batch;
    const size_t cbytes = sizeof(double2) * ((size_t)(batch - 1) * sC + (size_t)ldc * (N - 1) + M);
    TuneScratch scratch{ctx};
    const int v = tune_select(ctx, key, 3, [&](int vv) -> int {
        if (!scratch.p) {
            int st = scratch.init(C, cbytes);
            if (st) return st;
        }
        return launch(vv, (double2 *)scratch.p);
    });
    return launch(v, C);
}

int dfgemm_batched(ia_context *ctx, Op opa, Op opb, int M, int N, int K, double alpha, const double2 *A, int lda,
                   long long sA, const double2 *B, int ldb, long long sB, double beta, double2 *C, int ldc,
                   long long sC, int batch)
{
    return dfgemm_any<double2, double2>(ctx, opa, opb, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC,
                                        batch);
}

int dfgemm4_batched(ia_context *ctx, Op opa, Op opb, int M, int N, int K, double alpha, const float4 *A, int lda,
                    long long sA, const float4 *B, int ldb, long long sB, double beta, double2 *C, int ldc,
                    long long sC, int batch)
{
    return dfgemm_any<float4, float4>(ctx, opa, opb, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch);
}

// out[e] = (re hi, im hi, re lo, im lo) of in[e]
__global__ void split_df_kernel(size_t count, const double2 *__restrict__ in, float4 *__restrict__ out)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x)
        out[e] = split_c(in[e], false);
}

// out[e] = the high (FP32) parts of in[e]
__global__ void df_hi_kernel(size_t count, const float4 *__restrict__ in, float2 *__restrict__ out)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        const float4 v = in[e];
        out[e] = make_float2(v.x, v.y);
    }
}

static int grid_for(ia_context *ctx, size_t count)
{
    const size_t want = (count + 255) / 256, cap = (size_t)ctx->sm_count * 16;
    return (int)(want < cap ? want : cap);
}

int split_df_batched(ia_context *ctx, size_t count, const double2 *in, float4 *out)
{
    if (!count) return IA_OK;
    split_df_kernel<<<grid_for(ctx, count), 256, 0, ctx->stream>>>(count, in, out);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

int df_hi_batched(ia_context *ctx, size_t count, const float4 *in, float2 *out)
{
    if (!count) return IA_OK;
    df_hi_kernel<<<grid_for(ctx, count), 256, 0, ctx->stream>>>(count, in, out);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

}  // namespace ia
