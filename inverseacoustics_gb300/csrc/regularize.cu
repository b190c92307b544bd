// Fused filter-factor / GCV / back-projection kernels, FP64.
//
// regularize_kernel, one CTA per (frequency, right-hand side), from explicit
// SVD factors:
//   beta = U^H b                                    (tsvd.cuh:151, gcvG.m:25)
//   delta0 = ||b||^2 - ||beta||^2 if m > p          (gcvG.m:26, :32-35)
//   lambda by GCV (gcv.cuh), TSVD truncation or a fixed lambda
//   x = V (phi .* beta): Tikhonov phi = s/(s^2+lambda^2) (tikhonovG.m:30) or
//                        TSVD phi = 1/s on the first k (tsvdG.m:21-23; betak,
//                        tsvd.cuh:1-8)
// gcv_beta_kernel does the same from beta already projected (the pipeline
// carries U^H b through the Jacobi rotations) and writes z = phi .* beta.
#include "gcv.cuh"
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

constexpr int REG_THREADS = 256;

__global__ void __launch_bounds__(REG_THREADS) regularize_kernel(int m, int n, int p, const double2 *U,
                                                                   const double *S, const double2 *V, int nrhs,
                                                                   const double2 *B, ia_config cfg, double2 *X,
                                                                   double *LAM)
{
    extern __shared__ double sm[];
    double *s = sm;                                      // p
    double *b2 = s + p;                                  // p
    double2 *z = reinterpret_cast<double2 *>(b2 + p);    // p
    double *gval = reinterpret_cast<double *>(z + p);    // gcv_points
    __shared__ double red[REG_THREADS / 32];
    __shared__ double s_d0;
    const int f = blockIdx.x, r = blockIdx.y;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    U += (size_t)f * m * p;
    V += (size_t)f * n * p;
    S += (size_t)f * p;
    const double2 *b = B + ((size_t)f * nrhs + r) * m;
    double2 *x = X + ((size_t)f * nrhs + r) * n;

    for (int j = threadIdx.x; j < p; j += blockDim.x) s[j] = S[j];
    for (int j = wid; j < p; j += nw) {
        double2 acc = make_double2(0.0, 0.0);
        for (int i = lane; i < m; i += 32) zcfma(acc, U[i + (size_t)j * m], b[i]);
        acc = warp_sum2(acc);
        if (lane == 0) {
            z[j] = acc;
            b2[j] = zabs2(acc);
        }
    }
    double nb = 0.0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) nb += zabs2(b[i]);
    nb = warp_sum(nb);
    if (lane == 0) red[wid] = nb;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tb = 0.0, tbeta = 0.0;
        for (int w = 0; w < nw; ++w) tb += red[w];
        for (int j = 0; j < p; ++j) tbeta += b2[j];
        double d0 = tb - tbeta;
        s_d0 = (m > p && d0 > 0.0) ? d0 : 0.0;
    }
    __syncthreads();
    const double lam = choose_lambda(s, b2, p, s_d0, (double)(m - p), cfg, gval);
    for (int j = threadIdx.x; j < p; j += blockDim.x) z[j] = zscale(z[j], filter_phi(cfg.method, j, s[j], lam, cfg.tsvd_k));
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double2 acc = make_double2(0.0, 0.0);
        for (int j = 0; j < p; ++j) zfma(acc, V[i + (size_t)j * n], z[j]);
        x[i] = acc;
    }
    if (LAM && threadIdx.x == 0) LAM[(size_t)f * nrhs + r] = (cfg.method == IA_METHOD_TSVD) ? 0.0 : lam;
}

int regularize_batched(ia_context *ctx, int m, int n, int p, int batch, const double2 *U, const double *s,
                       const double2 *V, int nrhs, const double2 *b, const ia_config *cfg, double2 *x,
                       double *lambda)
{
    if (int st = check_method(*cfg, p)) return st;
    size_t smem = sizeof(double) * (size_t)p * 2 + sizeof(double2) * (size_t)p + sizeof(double) * (size_t)cfg->gcv_points;
    if (smem > 200 * 1024) return IA_ERR_TOO_LARGE;
    IA_CUDA_TRY(cudaFuncSetAttribute(regularize_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    dim3 g(batch, nrhs);
    regularize_kernel<<<g, REG_THREADS, smem, ctx->stream>>>(m, n, p, U, s, V, nrhs, b, *cfg, x, lambda);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// From beta (F x nrhs x p, sorted like s) to z = phi .* beta (same layout).
__global__ void __launch_bounds__(REG_THREADS) gcv_beta_kernel(int m, int p, const double *S, int nrhs,
                                                                 const double2 *BETA, const double *BNORM2,
                                                                 ia_config cfg, double2 *Z, double *LAM)
{
    extern __shared__ double sm[];
    double *s = sm;
    double *b2 = s + p;
    double *gval = b2 + p;
    __shared__ double s_d0;
    const int f = blockIdx.x, r = blockIdx.y;
    S += (size_t)f * p;
    const double2 *beta = BETA + ((size_t)f * nrhs + r) * p;
    double2 *z = Z + ((size_t)f * nrhs + r) * p;
    for (int j = threadIdx.x; j < p; j += blockDim.x) {
        s[j] = S[j];
        b2[j] = zabs2(beta[j]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double d0 = 0.0;
        if (BNORM2 && m > p) {
            double tbeta = 0.0;
            for (int j = 0; j < p; ++j) tbeta += b2[j];
            d0 = BNORM2[(size_t)f * nrhs + r] - tbeta;
            if (!(d0 > 0.0)) d0 = 0.0;
        }
        s_d0 = d0;
    }
    __syncthreads();
    const double lam = choose_lambda(s, b2, p, s_d0, (double)(m - p), cfg, gval);
    for (int j = threadIdx.x; j < p; j += blockDim.x) z[j] = zscale(beta[j], filter_phi(cfg.method, j, s[j], lam, cfg.tsvd_k));
    if (LAM && threadIdx.x == 0) LAM[(size_t)f * nrhs + r] = (cfg.method == IA_METHOD_TSVD) ? 0.0 : lam;
}

int gcv_beta_batched(ia_context *ctx, int m, int p, int batch, const double *s, int nrhs, const double2 *beta,
                     const double *bnorm2, const ia_config *cfg, double2 *z, double *lambda)
{
    if (int st = check_method(*cfg, p)) return st;
    size_t smem = sizeof(double) * ((size_t)p * 2 + (size_t)cfg->gcv_points);
    if (smem > 200 * 1024) return IA_ERR_TOO_LARGE;
    IA_CUDA_TRY(cudaFuncSetAttribute(gcv_beta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    dim3 g(batch, nrhs);
    gcv_beta_kernel<<<g, REG_THREADS, smem, ctx->stream>>>(m, p, s, nrhs, beta, bnorm2, *cfg, z, lambda);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

}  // namespace ia
