// Differentiable ESM array design: the Tikhonov reconstruction error of known
// source fields and its gradient by a hand-written adjoint.
//
//   s_j  = u_j (1 - d / |u_j|)          equivalent sources, retreat d
//   G_ij = exp(i k r_ij) / (4 pi r_ij)   microphone i, source j (esmV.m:29-30)
//   p    = G q + noise
//   q^   = G^H (G G^H + lambda^2 I)^-1 p = V diag(s/(s^2+lambda^2)) U^H p
//                                          (tikhonovG.m:26-30, data-space form)
//   L    = mean over frequencies f and fields r of ||q^ - q|| / ||q||
//
// Adjoint, per frequency, with K = G G^H + lambda^2 I, y = K^-1 p, e = q^ - q,
// g = e / (||e|| ||q|| F R), z = K^-1 G g, w = g - G^H z:
//   dL = Re sum_ij A_ij dG_ij - 2 lambda^2 Re(z^H y) dlog(lambda)
//   A_ij = sum_r conj(y_ir) w_jr - conj(z_ir) e_jr      (the p = G q path included)
//   dG_ij = G_ij (i k - 1/r_ij) (m_i - s_j) . (dm_i - ds_j) / r_ij,  ds_j = -u_j/|u_j| dd
//
// The reference has no such path.  With l <= m microphones the data-space
// form needs only K (l x l) and its LU per frequency, so nothing of size
// m x m or an SVD is kept for the backward pass.
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

// sources and unit directions from the surface points and the retreat
__global__ void design_sources_kernel(int m, const double *__restrict__ surf, const double *__restrict__ retreat,
                                      double *__restrict__ src, double *__restrict__ unit)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const double x = surf[j], y = surf[j + m], z = surf[j + 2 * m];
    const double rn = sqrt(x * x + y * y + z * z);
    const double sc = 1.0 - retreat[0] / rn;
    src[j] = x * sc;
    src[j + m] = y * sc;
    src[j + 2 * m] = z * sc;
    unit[j] = x / rn;
    unit[j + m] = y / rn;
    unit[j + 2 * m] = z / rn;
}

// K_f += lambda_f^2 I
__global__ void diag_shift_kernel(int l, int F, const double *__restrict__ loglam, double2 *__restrict__ K)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= l * F) return;
    const int f = e / l, i = e % l;
    const double lam = exp(loglam[f]);
    K[(size_t)f * l * l + i + (size_t)i * l].x += lam * lam;
}

// per (f, r): e = q^ - q, err = ||e|| / ||q||, g = e / (||e|| ||q|| F R)
__global__ void design_seed_kernel(int m, int F, int R, const double2 *__restrict__ Qh, const double2 *__restrict__ Q,
                                   double2 *__restrict__ E, double2 *__restrict__ Gb, double *__restrict__ err,
                                   int *__restrict__ info)
{
    __shared__ double red[2][32];
    const int f = blockIdx.y, r = blockIdx.x;
    const size_t o = ((size_t)f * R + r) * m;
    double se = 0.0, sq = 0.0;
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
        const double2 a = Qh[o + j], b = Q[o + j];
        const double2 d = make_double2(a.x - b.x, a.y - b.y);
        E[o + j] = d;
        se += d.x * d.x + d.y * d.y;
        sq += b.x * b.x + b.y * b.y;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    se = warp_sum(se);
    sq = warp_sum(sq);
    if (lane == 0) { red[0][wid] = se; red[1][wid] = sq; }
    __syncthreads();
    if (threadIdx.x == 0) {
        se = 0.0;
        sq = 0.0;
        for (int w = 0; w < nw; ++w) { se += red[0][w]; sq += red[1][w]; }
        red[0][0] = sqrt(se);
        red[1][0] = sqrt(sq);
        const double v = red[0][0] / red[1][0];
        err[(size_t)f * R + r] = v;
        if (!(v == v) || isinf(v)) atomicOr(&info[f], IA_INFO_NONFINITE);
    }
    __syncthreads();
    const double den = red[0][0] * red[1][0] * (double)F * (double)R;
    const double sc = den > 0.0 ? 1.0 / den : 0.0;       // ||e|| = 0: the norm has no gradient; take 0
    for (int j = threadIdx.x; j < m; j += blockDim.x) Gb[o + j] = zscale(E[o + j], sc);
}

// dL/dlog(lambda_f) = -2 lambda_f^2 Re sum_r z_r^H y_r
__global__ void design_loglam_kernel(int l, int R, const double *__restrict__ loglam, const double2 *__restrict__ Z,
                                     const double2 *__restrict__ Y, double *__restrict__ gl)
{
    __shared__ double red[32];
    const int f = blockIdx.x;
    const size_t o = (size_t)f * l * R;
    double s = 0.0;
    for (int e = threadIdx.x; e < l * R; e += blockDim.x) s += Z[o + e].x * Y[o + e].x + Z[o + e].y * Y[o + e].y;
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        const double lam = exp(loglam[f]);
        gl[f] = -2.0 * lam * lam * t;
    }
}

// Geometry adjoint.  CTA per (microphone i, frequency f), threads over sources
// j: A_ij from the R fields, c_ij = Re(A_ij G_ij (i k - 1/r)) / r, partial
// sums of c_ij (m_i - s_j) (microphone gradient) and c_ij (m_i - s_j) . u_j
// (retreat gradient) into part[f][i][0..3].
constexpr int DG_THREADS = 128;
constexpr int DG_MAXR = 32;

__global__ void __launch_bounds__(DG_THREADS) design_geometry_kernel(
    int l, int m, int R, const double *__restrict__ mics, const double *__restrict__ src,
    const double *__restrict__ unit, const double *__restrict__ kv, const double2 *__restrict__ G,
    const double2 *__restrict__ Y, const double2 *__restrict__ Z, const double2 *__restrict__ W,
    const double2 *__restrict__ E, double *__restrict__ part)
{
    __shared__ double2 sy[DG_MAXR], sz[DG_MAXR];
    __shared__ double red[4][DG_THREADS / 32];
    const int i = blockIdx.x, f = blockIdx.y;
    const double k = kv[f];
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        const double2 yv = Y[((size_t)f * R + r) * l + i], zv = Z[((size_t)f * R + r) * l + i];
        sy[r] = make_double2(yv.x, -yv.y);                 // conj(y_ir)
        sz[r] = make_double2(zv.x, -zv.y);                 // conj(z_ir)
    }
    __syncthreads();
    const double mx = mics[i], my = mics[i + l], mz = mics[i + 2 * l];
    const double2 *Gf = G + (size_t)f * l * m;
    const size_t ob = (size_t)f * R * m;
    double ax = 0.0, ay = 0.0, az = 0.0, ad = 0.0;
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
        double2 A = make_double2(0.0, 0.0);
        for (int r = 0; r < R; ++r) {
            const double2 w = W[ob + (size_t)r * m + j], e = E[ob + (size_t)r * m + j];
            zfma(A, sy[r], w);
            zfms(A, sz[r], e);
        }
        const double dx = mx - src[j], dy = my - src[j + m], dz = mz - src[j + 2 * m];
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double inv = 1.0 / sqrt(r2);
        const double2 g = Gf[i + (size_t)j * l];
        // Re(A g (i k - 1/r)) / r
        const double2 ag = zmul(A, g);
        const double c = (-ag.y * k - ag.x * inv) * inv;
        ax = fma(c, dx, ax);
        ay = fma(c, dy, ay);
        az = fma(c, dz, az);
        ad = fma(c, dx * unit[j] + dy * unit[j + m] + dz * unit[j + 2 * m], ad);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    ax = warp_sum(ax);
    ay = warp_sum(ay);
    az = warp_sum(az);
    ad = warp_sum(ad);
    if (lane == 0) { red[0][wid] = ax; red[1][wid] = ay; red[2][wid] = az; red[3][wid] = ad; }
    __syncthreads();
    if (threadIdx.x < 4) {
        double s = 0.0;
        for (int w = 0; w < DG_THREADS / 32; ++w) s += red[threadIdx.x][w];
        part[((size_t)f * l + i) * 4 + threadIdx.x] = s;
    }
}

// sums over frequencies (and microphones for the retreat) in a fixed order
__global__ void design_reduce_kernel(int l, int F, const double *__restrict__ part, double *__restrict__ gm,
                                     double *__restrict__ gd)
{
    __shared__ double red[32];
    double sd = 0.0;
    for (int i = threadIdx.x; i < l; i += blockDim.x) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for (int f = 0; f < F; ++f) {
            const double *p = part + ((size_t)f * l + i) * 4;
            s0 += p[0];
            s1 += p[1];
            s2 += p[2];
            sd += p[3];
        }
        gm[i] = s0;
        gm[i + l] = s1;
        gm[i + 2 * l] = s2;
    }
    sd = warp_sum(sd);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sd;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        gd[0] = t;
    }
}

size_t esm_design_ws_bytes(int l, int m, int F, int R)
{
    const size_t L = l, M = m, FF = F, RR = R;
    return 2 * ws_round(24 * M) + ws_round(16 * FF * L * M) + ws_round(16 * FF * L * L) + ws_round(4 * FF * L) +
           3 * ws_round(16 * FF * L * RR) + 4 * ws_round(16 * FF * M * RR) + ws_round(32 * FF * L) + 4096;
}

int esm_design_batched(ia_context *ctx, int l, int m, int F, int R, const double *mics, const double *surf,
                       const double *retreat, const double *k, const double *loglam, const double2 *q,
                       const double2 *noise, double *err, double *gm, double *gd, double *gl, int *info,
                       WsCursor &cur)
{
    if (R > DG_MAXR) return IA_ERR_ARG;
    const long long lm = (long long)l * m, ll = (long long)l * l, lR = (long long)l * R, mR = (long long)m * R;
    double *src = cur.take<double>(3 * (size_t)m);
    double *unit = cur.take<double>(3 * (size_t)m);
    double2 *G = cur.take<double2>((size_t)lm * F);
    double2 *K = cur.take<double2>((size_t)ll * F);
    int *ipiv = cur.take<int>((size_t)l * F);
    double2 *Y = cur.take<double2>((size_t)lR * F);
    double2 *Z = cur.take<double2>((size_t)lR * F);
    double2 *P = cur.take<double2>((size_t)lR * F);
    double2 *Qh = cur.take<double2>((size_t)mR * F);
    double2 *E = cur.take<double2>((size_t)mR * F);
    double2 *Gb = cur.take<double2>((size_t)mR * F);
    double2 *W = cur.take<double2>((size_t)mR * F);
    double *part = cur.take<double>((size_t)F * l * 4);
    const double2 one = make_double2(1.0, 0.0), zero = make_double2(0.0, 0.0), mone = make_double2(-1.0, 0.0);
    int st;
    design_sources_kernel<<<(m + 127) / 128, 128, 0, ctx->stream>>>(m, surf, retreat, src, unit);
    IA_LAUNCH_CHECK(ctx);
    if ((st = monopole_batched(ctx, l, m, F, mics, src, k, G))) return st;
    // p = G q (+ noise)
    if (noise) IA_CUDA_TRY(cudaMemcpyAsync(P, noise, sizeof(double2) * lR * F, cudaMemcpyDeviceToDevice, ctx->stream));
    if ((st = zgemm_batched(ctx, OP_N, OP_N, l, R, m, one, G, l, lm, q, m, mR, noise ? one : zero, P, l, lR, F)))
        return st;
    // K = G G^H + lambda^2 I, LU
    if ((st = zgemm_batched(ctx, OP_N, OP_C, l, l, m, one, G, l, lm, G, l, lm, zero, K, l, ll, F))) return st;
    diag_shift_kernel<<<(l * F + 255) / 256, 256, 0, ctx->stream>>>(l, F, loglam, K);
    IA_LAUNCH_CHECK(ctx);
    if ((st = zgetrf_batched(ctx, l, K, l, ll, ipiv, info, F))) return st;
    // y = K^-1 p, q^ = G^H y
    IA_CUDA_TRY(cudaMemcpyAsync(Y, P, sizeof(double2) * lR * F, cudaMemcpyDeviceToDevice, ctx->stream));
    if ((st = zgetrs_batched(ctx, l, R, K, l, ll, ipiv, Y, l, lR, F))) return st;
    if ((st = zgemm_batched(ctx, OP_C, OP_N, m, R, l, one, G, l, lm, Y, l, lR, zero, Qh, m, mR, F))) return st;
    design_seed_kernel<<<dim3(R, F), 256, 0, ctx->stream>>>(m, F, R, Qh, q, E, Gb, err, info);
    IA_LAUNCH_CHECK(ctx);
    if (!gm) return IA_OK;
    // z = K^-1 G g, w = g - G^H z
    if ((st = zgemm_batched(ctx, OP_N, OP_N, l, R, m, one, G, l, lm, Gb, m, mR, zero, Z, l, lR, F))) return st;
    if ((st = zgetrs_batched(ctx, l, R, K, l, ll, ipiv, Z, l, lR, F))) return st;
    IA_CUDA_TRY(cudaMemcpyAsync(W, Gb, sizeof(double2) * mR * F, cudaMemcpyDeviceToDevice, ctx->stream));
    if ((st = zgemm_batched(ctx, OP_C, OP_N, m, R, l, mone, G, l, lm, Z, l, lR, one, W, m, mR, F))) return st;
    design_loglam_kernel<<<F, 256, 0, ctx->stream>>>(l, R, loglam, Z, Y, gl);
    IA_LAUNCH_CHECK(ctx);
    design_geometry_kernel<<<dim3(l, F), DG_THREADS, 0, ctx->stream>>>(l, m, R, mics, src, unit, k, G, Y, Z, W, E,
                                                                        part);
    IA_LAUNCH_CHECK(ctx);
    design_reduce_kernel<<<1, 256, 0, ctx->stream>>>(l, F, part, gm, gd);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

}  // namespace ia
