// BEM radiation modes: the reference's own radiation-mode path, invr()
// (CUDA/invr.cuh:457-909), specified by MATLAB/invrS.m:18-170 and
// invrV.m:65-119, batched over frequencies:
//
//   A, B, A_hs, B_hs   the IBEM collocation rows (ibem_assemble.cu), with
//                       n_ch CHIEF rows below the m surface rows
//   Z = A \ B           surface velocity -> surface pressure (invrS.m:159);
//                       LU when square, Householder least squares with CHIEF
//                       rows (invr.cuh:860-863 zgels)
//   G                   surface mass matrix, G_ab = sum_e |n_e| sum_q w_q N_a N_b
//                       over the regular rule (invrS.m:65, invr.cuh:605-624)
//   modes               real variant: U_r, s_r of the resistance R = Re(G Z)
//                       (invrS.m:160-161); complex variant: of G Z itself
//                       (invr.cuh:868-889 zgesvd)
//   H_r = (A_hs Z - B_hs) U_r, P_r = Z U_r   modal transfer and surface
//                       pressures (invrS.m:165-169; invr.cuh:900-907)
//
// invr.cuh:904,907 take n_am as the inner dimension of the output products
// (so only n_am = m gives H U and Z U); here every product has the sizes
// invrS.m gives.  Real variant: left singular vectors by subspace iteration on
// R R^T (radiation.cu).  Complex variant: one-sided Jacobi SVD of G Z (svd.cu),
// each column's phase fixed so that its first component within 1e-6 of the
// largest magnitude is real and positive.
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

// thread per node row, incident elements in adjacency order (deterministic)
__global__ void mass_matrix_kernel(int m, const int *__restrict__ gptr, const int *__restrict__ gidx,
                                   const int *__restrict__ adj_ptr, const int *__restrict__ adj,
                                   const int *__restrict__ evert, const double *__restrict__ egeo,
                                   const double *__restrict__ rule, int nq, double *__restrict__ gval)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int r0 = gptr[i], r1 = gptr[i + 1];
    for (int t = r0; t < r1; ++t) gval[t] = 0.0;
    for (int a = adj_ptr[i]; a < adj_ptr[i + 1]; ++a) {
        const int code = adj[a], e = code >> 2, sa = code & 3;
        const double an = egeo[(size_t)e * 16 + 12];
        const int4 vv = reinterpret_cast<const int4 *>(evert)[e];
        for (int sb = 0; sb < 3; ++sb) {
            double acc = 0.0;
            for (int q = 0; q < nq; ++q) {
                const double x1 = rule[q], x2 = rule[q + nq], w = rule[q + 2 * nq];
                const double na = sa == 0 ? x1 : (sa == 1 ? x2 : 1.0 - x1 - x2);
                const double nb = sb == 0 ? x1 : (sb == 1 ? x2 : 1.0 - x1 - x2);
                acc = fma(w * na, nb, acc);
            }
            const int j = sb == 0 ? vv.x : (sb == 1 ? vv.y : vv.z);
            for (int t = r0; t < r1; ++t)
                if (gidx[t] == j) {
                    gval[t] = fma(an, acc, gval[t]);
                    break;
                }
        }
    }
}

// out_f = G Z_f (complex) or Re(G Z_f), column-major m x m; Z_f with leading
// dimension ldz; grid (row blocks, column, frequency)
template <bool CPLX>
__global__ void gz_kernel(int m, const int *__restrict__ gptr, const int *__restrict__ gidx,
                          const double *__restrict__ gval, const double2 *__restrict__ Z, int ldz, long long sZ,
                          void *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, f = blockIdx.z;
    if (i >= m) return;
    const double2 *z = Z + (size_t)f * sZ + (size_t)j * ldz;
    double re = 0.0, im = 0.0;
    for (int t = gptr[i]; t < gptr[i + 1]; ++t) {
        const double g = gval[t];
        const double2 v = z[gidx[t]];
        re = fma(g, v.x, re);
        if (CPLX) im = fma(g, v.y, im);
    }
    const size_t o = (size_t)f * m * m + (size_t)j * m + i;
    if (CPLX) static_cast<double2 *>(out)[o] = make_double2(re, im);
    else static_cast<double *>(out)[o] = re;
}

// real variant: s = sqrt(max(lambda, 0)); Uc = U as complex
__global__ void modes_finish_kernel(size_t nsv, const double *__restrict__ lam, double *__restrict__ s, size_t nu,
                                    const double *__restrict__ U, double2 *__restrict__ Uc)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < nu; e += stride) {
        Uc[e] = make_double2(U[e], 0.0);
        if (e < nsv) s[e] = sqrt(fmax(lam[e], 0.0));
    }
}

// complex variant: the leading nm columns of each m x m U (and the leading nm
// singular values), each column multiplied by the unit phase that makes its
// first component within 1e-6 of the largest magnitude real and positive.
// Block per frequency, warp per column.
__global__ void modes_phase_kernel(int m, int nm, const double2 *__restrict__ U, const double *__restrict__ sfull,
                                   double2 *__restrict__ Uc, double *__restrict__ sr)
{
    const int f = blockIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = wid; j < nm; j += nw) {
        const double2 *u = U + ((size_t)f * m + j) * m;
        double best = 0.0;
        for (int i = lane; i < m; i += 32) best = fmax(best, hypot(u[i].x, u[i].y));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(0xffffffffu, best, o));
        const double thr = best * (1.0 - 1e-6);
        int bi = m;
        for (int i = lane; i < m; i += 32)
            if (hypot(u[i].x, u[i].y) >= thr) { bi = i; break; }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) bi = min(bi, __shfl_xor_sync(0xffffffffu, bi, o));
        double2 ph = make_double2(1.0, 0.0);
        if (bi < m) {
            const double2 p = u[bi];
            const double a = hypot(p.x, p.y);
            if (a > 0.0) ph = make_double2(p.x / a, -p.y / a);
        }
        double2 *dst = Uc + ((size_t)f * nm + j) * m;
        for (int i = lane; i < m; i += 32) dst[i] = zmul(u[i], ph);
        if (lane == 0) sr[(size_t)f * nm + j] = sfull[(size_t)f * m + j];
    }
}

// out = hi + lo of double-float complex pairs
__global__ void df_join_kernel(size_t count, const float4 *__restrict__ in, double2 *__restrict__ out)
{
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < count; e += (size_t)gridDim.x * blockDim.x) {
        const float4 v = in[e];
        out[e] = make_double2((double)v.x + (double)v.z, (double)v.y + (double)v.w);
    }
}

static bool bem_mixed_solve(const ia_config *cfg, int n_ch) { return cfg->precision == IA_PREC_MIXED && n_ch == 0; }

size_t bem_modes_ws_bytes(const ia_mesh *mesh, int l, int n_ch, int F, int nm, const ia_config *cfg, bool cplx)
{
    const size_t M = mesh->m, MT = M + n_ch, L = l, FF = F;
    size_t b = 4 * ws_round(16 * MT * M * FF) + 4 * ws_round(16 * M * L * FF) + ws_round(4 * M * FF) +
               ws_round(8 * (size_t)mesh->gnnz) + ws_round(16 * M * nm * FF);
    if (cplx) b += ws_round(16 * M * M * FF) + ws_round(8 * M * FF);
    else b += ws_round(8 * M * M * FF) + ws_round(8 * nm * FF) + radiation_modes_ws_bytes(mesh->m, F, nm, cfg, true);
    if (bem_mixed_solve(cfg, n_ch)) b += 2 * ws_round(8 * M * M * FF) + ws_round(16 * M * M * FF);
    return b + 4096;
}

// Mixed Z = A^-1 B and H = A_hs Z - B_hs: A and B arrive as double-float row
// blocks (A^T, B^T as float4); FP32 LU of A and FP32 solves for Z, refined
// with double-float residuals B - A Z (max(1, refine_steps) times); H by the
// double-float GEMM.  On exit Z (FP64, m x m) is in At's storage.
static int bem_mixed_z(ia_context *ctx, const ia_mesh *mesh, int l, const double *mics, int F, const double *k,
                       const ia_config *cfg, double2 *At, double2 *Bt, double2 *A, double2 *B, double2 *Ahs_t,
                       double2 *Bhs_t, double2 *Ahs, double2 *H, int *ipiv, int *info, WsCursor &cur)
{
    const int m = mesh->m;
    const long long mm = (long long)m * m, ml = (long long)m * l;
    int st;
    if ((st = ibem_rows(ctx, mesh, l, mics, 0, nullptr, F, k, cfg->c, cfg->rho, At, Bt, Ahs_t, Bhs_t, true, true)))
        return st;
    // A, B column-major as float4 pairs (16-byte moves through the double2 view)
    if ((st = ztranspose_batched(ctx, m, m, At, m, mm, A, m, mm, false, F))) return st;
    if ((st = ztranspose_batched(ctx, m, m, Bt, m, mm, B, m, mm, false, F))) return st;
    if ((st = ztranspose_batched(ctx, m, l, Ahs_t, m, ml, Ahs, l, ml, false, F))) return st;
    if ((st = ztranspose_batched(ctx, m, l, Bhs_t, m, ml, H, l, ml, false, F))) return st;
    float4 *A4 = reinterpret_cast<float4 *>(A), *B4 = reinterpret_cast<float4 *>(B);
    float2 *A32 = cur.take<float2>((size_t)mm * F);
    float2 *Z32 = cur.take<float2>((size_t)mm * F);
    float4 *Z4 = cur.take<float4>((size_t)mm * F);
    double2 *Z = At, *R = Bt;
    if ((st = df_hi_batched(ctx, (size_t)mm * F, A4, A32))) return st;
    if ((st = getrf_batched<float2>(ctx, m, A32, m, mm, ipiv, info, F))) return st;
    if ((st = df_hi_batched(ctx, (size_t)mm * F, B4, Z32))) return st;
    if ((st = getrs_batched<float2>(ctx, m, m, A32, m, mm, ipiv, Z32, m, mm, F))) return st;
    if ((st = copy2d_batched<float2, double2>(ctx, m, m, Z32, m, mm, Z, m, mm, false, F))) return st;
    const int steps = cfg->refine_steps > 1 ? cfg->refine_steps : 1;
    const size_t n4 = (size_t)mm * F;
    for (int it = 0; it < steps; ++it) {
        df_join_kernel<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(n4, B4, R);
        IA_LAUNCH_CHECK(ctx);
        if ((st = split_df_batched(ctx, n4, Z, Z4))) return st;
        if ((st = dfgemm4_batched(ctx, OP_N, OP_N, m, m, m, -1.0, A4, m, mm, Z4, m, mm, 1.0, R, m, mm, F))) return st;
        if ((st = copy2d_batched<double2, float2>(ctx, m, m, R, m, mm, Z32, m, mm, false, F))) return st;
        if ((st = getrs_batched<float2>(ctx, m, m, A32, m, mm, ipiv, Z32, m, mm, F))) return st;
        if ((st = add2d_batched<float2>(ctx, m, m, Z32, m, mm, Z, m, mm, F))) return st;
    }
    // H = A_hs Z - B_hs (A_hs split into A_hs^T's storage)
    float4 *Ahs4 = reinterpret_cast<float4 *>(Ahs_t);
    if ((st = split_df_batched(ctx, n4, Z, Z4))) return st;
    if ((st = split_df_batched(ctx, (size_t)ml * F, Ahs, Ahs4))) return st;
    return dfgemm4_batched(ctx, OP_N, OP_N, l, m, m, 1.0, Ahs4, l, ml, Z4, m, mm, -1.0, H, l, ml, F);
}

int bem_modes_batched(ia_context *ctx, const ia_mesh *mesh, int l, const double *mics, int n_ch, const double *cp,
                      int F, const double *k, int nm, const ia_config *cfg, bool cplx, void *Ur, double *sr,
                      double2 *Hr, double2 *Pr, int *info, WsCursor &cur)
{
    const int m = mesh->m, mt = m + n_ch;
    int st;
    const long long mm = (long long)m * m, tm = (long long)mt * m, ml = (long long)m * l;
    double2 *At = cur.take<double2>(tm * F), *Bt = cur.take<double2>(tm * F);
    double2 *A = cur.take<double2>(tm * F), *B = cur.take<double2>(tm * F);
    double2 *Ahs_t = cur.take<double2>(ml * F), *Bhs_t = cur.take<double2>(ml * F);
    double2 *Ahs = cur.take<double2>(ml * F), *H = cur.take<double2>(ml * F);
    int *ipiv = cur.take<int>((size_t)m * F);
    double *gval = cur.take<double>((size_t)mesh->gnnz);
    double2 *Uc = cplx ? static_cast<double2 *>(Ur) : cur.take<double2>((size_t)m * nm * F);
    const double2 one = make_double2(1.0, 0.0), mone = make_double2(-1.0, 0.0), zero = make_double2(0.0, 0.0);
    const bool mixed_z = bem_mixed_solve(cfg, n_ch);
    double2 *Z = At;
    if (mixed_z) {
        if ((st = bem_mixed_z(ctx, mesh, l, mics, F, k, cfg, At, Bt, A, B, Ahs_t, Bhs_t, Ahs, H, ipiv, info, cur)))
            return st;
    } else {
        // collocation rows, then A, B (mt x m), A_hs, B_hs (l x m) column-major
        if ((st = ibem_rows(ctx, mesh, l, mics, n_ch, cp, F, k, cfg->c, cfg->rho, At, Bt, Ahs_t, Bhs_t,
                            cfg->precision == IA_PREC_MIXED)))
            return st;
        if ((st = ztranspose_batched(ctx, m, mt, At, m, tm, A, mt, tm, false, F))) return st;
        if ((st = ztranspose_batched(ctx, m, mt, Bt, m, tm, B, mt, tm, false, F))) return st;
        if ((st = ztranspose_batched(ctx, m, l, Ahs_t, m, ml, Ahs, l, ml, false, F))) return st;
        if ((st = ztranspose_batched(ctx, m, l, Bhs_t, m, ml, H, l, ml, false, F))) return st;
        // Z = A \ B (B's storage, leading dimension mt)
        if (n_ch == 0) {
            if ((st = zgetrf_batched(ctx, m, A, mt, tm, ipiv, info, F))) return st;
            if ((st = zgetrs_batched(ctx, m, m, A, mt, tm, ipiv, B, mt, tm, F))) return st;
        } else {
            if ((st = zgeqrs_batched(ctx, mt, m, A, mt, tm, m, B, mt, tm, F))) return st;
            if ((st = zbacksolve_upper_batched(ctx, m, m, A, mt, tm, B, mt, tm, F))) return st;
        }
        // compact Z (ld mt -> m) into At's storage
        if ((st = zcopy2d_batched(ctx, m, m, B, mt, tm, Z, m, mm, false, F))) return st;
        // H = A_hs Z - B_hs
        if ((st = zgemm_batched(ctx, OP_N, OP_N, l, m, m, one, Ahs, l, ml, Z, m, mm, mone, H, l, ml, F))) return st;
    }
    mass_matrix_kernel<<<(m + 127) / 128, 128, 0, ctx->stream>>>(m, mesh->d_gptr, mesh->d_gidx, mesh->d_adj_ptr,
                                                                  mesh->d_adj, mesh->d_evert, mesh->d_egeo,
                                                                  mesh->d_reg, mesh->nq, gval);
    IA_LAUNCH_CHECK(ctx);
    const dim3 gz_grid((m + 127) / 128, m, F);
    if (cplx) {
        // SVD of G Z: columns of Y orthogonalised in place, U = Y / sigma
        double2 *Y = cur.take<double2>(mm * F);
        double *sfull = cur.take<double>((size_t)m * F);
        double2 *Ufull = Bt;
        gz_kernel<true><<<gz_grid, 128, 0, ctx->stream>>>(m, mesh->d_gptr, mesh->d_gidx, gval, Z, m, mm, Y);
        IA_LAUNCH_CHECK(ctx);
        if ((st = jacobi_svd_batched(ctx, m, m, Y, nullptr, F, cfg->svd_max_sweeps, info))) return st;
        if ((st = svd_finalize_batched(ctx, m, m, Y, nullptr, sfull, Ufull, nullptr, F, info))) return st;
        modes_phase_kernel<<<F, 256, 0, ctx->stream>>>(m, nm, Ufull, sfull, Uc, sr);
        IA_LAUNCH_CHECK(ctx);
    } else {
        // left singular vectors of R = Re(G Z): eigenvectors of R R^T
        double *R = cur.take<double>(mm * F);
        double *lam = cur.take<double>((size_t)nm * F);
        double *Urr = static_cast<double *>(Ur);
        gz_kernel<false><<<gz_grid, 128, 0, ctx->stream>>>(m, mesh->d_gptr, mesh->d_gidx, gval, Z, m, mm, R);
        IA_LAUNCH_CHECK(ctx);
        if ((st = radiation_modes_batched(ctx, m, F, R, nm, cfg, lam, Urr, info, cur, true))) return st;
        const size_t nu = (size_t)m * nm * F;
        modes_finish_kernel<<<ctx->sm_count * 4, 256, 0, ctx->stream>>>((size_t)nm * F, lam, sr, nu, Urr, Uc);
        IA_LAUNCH_CHECK(ctx);
    }
    // H_r = H U_r, P_r = Z U_r (double-float products on the mixed path)
    const long long mn = (long long)m * nm;
    if (mixed_z) {
        if ((st = dfgemm_batched(ctx, OP_N, OP_N, l, nm, m, 1.0, H, l, ml, Uc, m, mn, 0.0, Hr, l, (long long)l * nm,
                                 F)))
            return st;
        if (Pr) st = dfgemm_batched(ctx, OP_N, OP_N, m, nm, m, 1.0, Z, m, mm, Uc, m, mn, 0.0, Pr, m, mn, F);
        return st;
    }
    if ((st = zgemm_batched(ctx, OP_N, OP_N, l, nm, m, one, H, l, ml, Uc, m, mn, zero, Hr, l, (long long)l * nm, F)))
        return st;
    if (Pr) st = zgemm_batched(ctx, OP_N, OP_N, m, nm, m, one, Z, m, mm, Uc, m, mn, zero, Pr, m, mn, F);
    return st;
}

}  // namespace ia
