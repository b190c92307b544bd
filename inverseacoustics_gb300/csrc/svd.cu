// Batched one-sided (Hestenes) Jacobi SVD in FP64, one CTA per frequency.
//
// Replaces cusolverDnZgesvd in csvd() (CUDA/tsvd.cuh:39,93) and the MATLAB
// svd() behind csvdG.m:17-24.  The columns of Y (M x N, M >= N) are
// orthogonalised pairwise with complex plane rotations; a round-robin
// (circle-method) ordering makes the N/2 pairs of a round disjoint, so each
// warp rotates one pair with no synchronisation inside a round.  Column dot
// products are warp-shuffle reductions in a fixed order, so repeated runs
// give identical results.  A pair is rotated while
// |y_i^H y_j| > sqrt(Mdot) eps ||y_i|| ||y_j||; the sweep loop ends after a
// sweep without rotations or at the sweep cap (IA_INFO_NOCONV).
//
// Only the first Mdot rows enter the dot products; rows Mdot..M-1 are rotated
// along (the pipeline keeps conj(b)^T there, so U^H b falls out of the
// rotations without forming U).
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

constexpr int SVD_MAX_WARPS = 16;

__device__ __forceinline__ void rr_pair(int N2, int round, int k, int &i, int &j)
{
    if (k == 0) {
        i = round;
        j = N2 - 1;
    } else {
        i = (round + k) % (N2 - 1);
        j = (round - k + N2 - 1) % (N2 - 1);
    }
    if (i > j) { int t = i; i = j; j = t; }
}

// Rotation that zeroes y_i^H y_j for column norms a, b and product g.
__device__ __forceinline__ bool jacobi_rotation(double a, double b, double2 g, double tol, double &c, double2 &sp)
{
    double gm = sqrt(g.x * g.x + g.y * g.y);
    if (!(gm > tol * sqrt(a) * sqrt(b)) || gm == 0.0) return false;
    double zeta = (b - a) / (2.0 * gm);
    double t;
    if (fabs(zeta) > 1e150) t = 0.5 / zeta;
    else t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
    c = 1.0 / sqrt(1.0 + t * t);
    double s = t * c;
    sp = make_double2(s * g.x / gm, s * g.y / gm);   // s' = s e^{i arg gamma}
    return true;
}

// KPL > 0: rows cached in registers (M <= 32*KPL); KPL == 0: streamed.
template <int KPL>
__global__ void __launch_bounds__(SVD_MAX_WARPS * 32) jacobi_kernel(int M, int Mdot, int N, double2 *Y, long long sY,
                                                                      double2 *V, long long sV, int max_sweeps,
                                                                      double tol, int *info)
{
    __shared__ int s_rot;
    const int f = blockIdx.x;
    Y += f * sY;
    if (V) V += f * sV;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int N2 = N + (N & 1);
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        if (threadIdx.x == 0) s_rot = 0;
        __syncthreads();
        int rot_local = 0;
        for (int round = 0; round < N2 - 1; ++round) {
            for (int k = wid; k < N2 / 2; k += nw) {
                int i, j;
                rr_pair(N2, round, k, i, j);
                if (j >= N) continue;
                double2 *yi = Y + (size_t)i * M, *yj = Y + (size_t)j * M;
                double a = 0.0, b = 0.0, c;
                double2 g = make_double2(0.0, 0.0), sp;
                if (KPL > 0) {
                    double2 ui[KPL > 0 ? KPL : 1], vj[KPL > 0 ? KPL : 1];
#pragma unroll
                    for (int t = 0; t < KPL; ++t) {
                        int r = lane + 32 * t;
                        ui[t] = r < M ? yi[r] : make_double2(0.0, 0.0);
                        vj[t] = r < M ? yj[r] : make_double2(0.0, 0.0);
                        if (r < Mdot) {
                            a = fma(ui[t].x, ui[t].x, fma(ui[t].y, ui[t].y, a));
                            b = fma(vj[t].x, vj[t].x, fma(vj[t].y, vj[t].y, b));
                            zcfma(g, ui[t], vj[t]);
                        }
                    }
                    a = warp_sum(a);
                    b = warp_sum(b);
                    g = warp_sum2(g);
                    if (!jacobi_rotation(a, b, g, tol, c, sp)) continue;
                    const double2 spc = zconj(sp);
#pragma unroll
                    for (int t = 0; t < KPL; ++t) {
                        int r = lane + 32 * t;
                        if (r < M) {
                            double2 nu = zscale(ui[t], c), nv = zscale(vj[t], c);
                            zfms(nu, spc, vj[t]);
                            zfma(nv, sp, ui[t]);
                            yi[r] = nu;
                            yj[r] = nv;
                        }
                    }
                } else {
                    for (int r = lane; r < Mdot; r += 32) {
                        double2 u = yi[r], v = yj[r];
                        a = fma(u.x, u.x, fma(u.y, u.y, a));
                        b = fma(v.x, v.x, fma(v.y, v.y, b));
                        zcfma(g, u, v);
                    }
                    a = warp_sum(a);
                    b = warp_sum(b);
                    g = warp_sum2(g);
                    if (!jacobi_rotation(a, b, g, tol, c, sp)) continue;
                    const double2 spc = zconj(sp);
                    for (int r = lane; r < M; r += 32) {
                        double2 u = yi[r], v = yj[r];
                        double2 nu = zscale(u, c), nv = zscale(v, c);
                        zfms(nu, spc, v);
                        zfma(nv, sp, u);
                        yi[r] = nu;
                        yj[r] = nv;
                    }
                }
                if (V) {
                    const double2 spc = zconj(sp);
                    double2 *vi = V + (size_t)i * N, *vjp = V + (size_t)j * N;
                    for (int r = lane; r < N; r += 32) {
                        double2 u = vi[r], v = vjp[r];
                        double2 nu = zscale(u, c), nv = zscale(v, c);
                        zfms(nu, spc, v);
                        zfma(nv, sp, u);
                        vi[r] = nu;
                        vjp[r] = nv;
                    }
                }
                rot_local++;
            }
            __syncthreads();
        }
        if (lane == 0 && rot_local) atomicAdd(&s_rot, rot_local);
        __syncthreads();
        int total = s_rot;
        __syncthreads();
        if (total == 0) break;
    }
    if (threadIdx.x == 0 && sweep >= max_sweeps && info) atomicOr(&info[f], IA_INFO_NOCONV);
}

__global__ void identity_kernel(int N, double2 *V, long long sV)
{
    const int f = blockIdx.y;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N * N; e += gridDim.x * blockDim.x) {
        int r = e % N, c = e / N;
        V[f * sV + e] = make_double2(r == c ? 1.0 : 0.0, 0.0);
    }
}

int jacobi_rows_batched(ia_context *ctx, int M, int Mdot, int N, double2 *Y, double2 *V, int batch, int max_sweeps,
                        int *info)
{
    if (V) {
        dim3 g((N * N + 255) / 256 < 256 ? (N * N + 255) / 256 : 256, batch);
        identity_kernel<<<g, 256, 0, ctx->stream>>>(N, V, (long long)N * N);
        IA_LAUNCH_CHECK(ctx);
    }
    int nw = (N + 1) / 2;
    if (nw > SVD_MAX_WARPS) nw = SVD_MAX_WARPS;
    if (nw < 1) nw = 1;
    const double tol = sqrt((double)Mdot) * 2.220446049250313e-16;
    const long long sY = (long long)M * N, sV = (long long)N * N;
    if (M <= 128)
        jacobi_kernel<4><<<batch, nw * 32, 0, ctx->stream>>>(M, Mdot, N, Y, sY, V, sV, max_sweeps, tol, info);
    else if (M <= 256)
        jacobi_kernel<8><<<batch, nw * 32, 0, ctx->stream>>>(M, Mdot, N, Y, sY, V, sV, max_sweeps, tol, info);
    else
        jacobi_kernel<0><<<batch, nw * 32, 0, ctx->stream>>>(M, Mdot, N, Y, sY, V, sV, max_sweeps, tol, info);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

int jacobi_svd_batched(ia_context *ctx, int M, int N, double2 *Y, double2 *V, int batch, int max_sweeps, int *info)
{
    return jacobi_rows_batched(ctx, M, M, N, Y, V, batch, max_sweeps, info);
}

// sigma_j = ||y_j||, descending order (ties by index), U = Y/sigma, V permuted.
__global__ void svd_finalize_kernel(int M, int N, const double2 *Y, const double2 *V, double *s, double2 *Uy,
                                    double2 *Vs, int *info)
{
    extern __shared__ double sm[];
    double *sig = sm;                              // N
    int *rank = reinterpret_cast<int *>(sm + N);   // N
    const int f = blockIdx.x;
    Y += (size_t)f * M * N;
    if (V) V += (size_t)f * N * N;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = wid; j < N; j += nw) {
        double a = 0.0;
        for (int r = lane; r < M; r += 32) {
            double2 u = Y[r + (size_t)j * M];
            a = fma(u.x, u.x, fma(u.y, u.y, a));
        }
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
        if (s) s[(size_t)f * N + rk] = sj;
        if (info && (!(sj == sj) || isinf(sj))) atomicOr(&info[f], IA_INFO_NONFINITE);
    }
    __syncthreads();
    if (Uy) {
        for (int j = wid; j < N; j += nw) {
            double inv = sig[j] > 0.0 ? 1.0 / sig[j] : 0.0;
            double2 *dst = Uy + (size_t)f * M * N + (size_t)rank[j] * M;
            for (int r = lane; r < M; r += 32) dst[r] = zscale(Y[r + (size_t)j * M], inv);
        }
    }
    if (Vs && V) {
        for (int j = wid; j < N; j += nw) {
            double2 *dst = Vs + (size_t)f * N * N + (size_t)rank[j] * N;
            for (int r = lane; r < N; r += 32) dst[r] = V[r + (size_t)j * N];
        }
    }
}

int svd_finalize_batched(ia_context *ctx, int M, int N, const double2 *Y, const double2 *V, double *s, double2 *Uy,
                         double2 *Vs, int batch, int *info)
{
    size_t smem = (size_t)N * (sizeof(double) + sizeof(int));
    svd_finalize_kernel<<<batch, 256, smem, ctx->stream>>>(M, N, Y, V, s, Uy, Vs, info);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

size_t svd_workspace_bytes(int m, int n, int batch)
{
    int M = m >= n ? m : n, N = m >= n ? n : m;
    return ws_round(sizeof(double2) * (size_t)M * N * batch) + ws_round(sizeof(double2) * (size_t)N * N * batch) +
           512;
}

int svd_batched(ia_context *ctx, int m, int n, const double2 *A, bool transposed_input, double2 *U, double *s,
                double2 *V, int batch, int max_sweeps, int *info, double2 *Y, double2 *Vacc)
{
    const bool tall = m >= n;
    const int M = tall ? m : n, N = tall ? n : m;
    int st = IA_OK;
    const long long sA = (long long)m * n;
    if (tall) {
        // Y = A (m x n)
        if (!transposed_input) st = zcopy2d_batched(ctx, m, n, A, m, sA, Y, M, (long long)M * N, false, batch);
        else st = ztranspose_batched(ctx, n, m, A, n, sA, Y, M, (long long)M * N, false, batch);
    } else {
        // Y = A^H (n x m)
        if (!transposed_input) st = ztranspose_batched(ctx, m, n, A, m, sA, Y, M, (long long)M * N, true, batch);
        else st = zcopy2d_batched(ctx, n, m, A, n, sA, Y, M, (long long)M * N, true, batch);
    }
    if (st) return st;
    st = jacobi_svd_batched(ctx, M, N, Y, Vacc, batch, max_sweeps, info);
    if (st) return st;
    // tall:  A = Uy S Vacc^H        -> U = Uy,   V = Vacc
    // wide:  A^H = Uy S Vacc^H      -> U = Vacc, V = Uy
    if (tall) return svd_finalize_batched(ctx, M, N, Y, Vacc, s, U, V, batch, info);
    return svd_finalize_batched(ctx, M, N, Y, Vacc, s, V, U, batch, info);
}

}  // namespace ia
