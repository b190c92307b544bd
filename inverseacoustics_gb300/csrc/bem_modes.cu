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
// R R^T (radiation.cu).  Complex variant: subspace iteration on the real
// representation of (G Z)(G Z)^H (radiation.cu again) and one complex vector
// per doubled eigenvalue while the subspace is at most half the space, else
// the one-sided Jacobi SVD of G Z (svd.cu).  Each complex column's phase is
// fixed so that its first component within 1e-6 of the largest magnitude is
// real and positive.
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

// unit phase that makes a column's first component within 1e-6 of the largest
// magnitude real and positive (warp-cooperative; every lane gets the phase)
__device__ double2 column_phase(int m, const double2 *u, int lane)
{
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
    return ph;
}

// complex variant (FP64): the leading nm columns of each m x m U and the
// leading nm singular values, each column multiplied by its unit phase.
// Block per frequency, warp per column.
__global__ void modes_phase_kernel(int m, int nm, const double2 *__restrict__ U, const double *__restrict__ sfull,
                                   double2 *__restrict__ Uc, double *__restrict__ sr)
{
    const int f = blockIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = wid; j < nm; j += nw) {
        const double2 *u = U + ((size_t)f * m + j) * m;
        const double2 ph = column_phase(m, u, lane);
        double2 *dst = Uc + ((size_t)f * nm + j) * m;
        for (int i = lane; i < m; i += 32) dst[i] = zmul(u[i], ph);
        if (lane == 0) sr[(size_t)f * nm + j] = sfull[(size_t)f * m + j];
    }
}

// complex variant (mixed): the real representation Yr = [[Re Y, -Im Y],
// [Im Y, Re Y]] (2m x 2m, column-major) of Y = G Z.  Yr Yr^T represents
// Y Y^H: every eigenvalue of Y Y^H appears twice, with the eigenvectors
// [Re u; Im u] and [-Im u; Re u] (the images of u and i u).
__global__ void real_rep_kernel(int m, const double2 *__restrict__ Y, double *__restrict__ Yr, int batch)
{
    const size_t n = 2 * (size_t)m, per = n * n;
    const size_t total = per * batch, stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += stride) {
        const size_t f = e / per, o = e % per;
        const int r = (int)(o % n), c = (int)(o / n);
        const int i = r < m ? r : r - m, j = c < m ? c : c - m;
        const double2 y = Y[f * (size_t)m * m + i + (size_t)j * m];
        Yr[e] = (r < m) == (c < m) ? y.x : (r < m ? -y.y : y.y);
    }
}

// Complex modes from the nc leading real Ritz vectors V (2m x nc, Ritz values
// lam descending) of the real representation.  A candidate v gives the complex
// vector w = v(0:m) + i v(m:2m).  Ritz values within 1e-12 lam_1 of a
// cluster's first one form the cluster: its r real vectors span (the image
// of) r/2 complex dimensions, each eigenvalue's pair [Re u; Im u],
// [-Im u; Re u] giving u and i u.  Per cluster, up to ceil(r/2) times: the
// free candidate with the largest squared residual against the accepted modes
// (ties to the lower index; none above 0.1 ends the cluster) is
// orthogonalised (two classical Gram-Schmidt passes), normalised and accepted
// with s = sqrt(max(lam, 0)).  Picking the largest residual keeps a cluster's
// last complex direction reachable however the Ritz vectors split it (a
// first-come rule with a threshold can spend it on earlier rejects).  Accepted
// columns get the unit phase of the FP64 variant; fewer than nm accepted flags
// IA_INFO_NOCONV (the rest zero).  Block per frequency.
constexpr int PICK_THREADS = 256;

__global__ void __launch_bounds__(PICK_THREADS) modes_pick_kernel(int m, int nm, int nc,
                                                                  const double *__restrict__ V,
                                                                  const double *__restrict__ lam,
                                                                  double2 *__restrict__ Uc, double *__restrict__ sr,
                                                                  int *__restrict__ info)
{
    extern __shared__ __align__(16) double2 pk_w[];              // m: candidate
    double2 *dots = pk_w + m;                                     // nm
    double *res = reinterpret_cast<double *>(dots + nm);          // nc
    int *taken = reinterpret_cast<int *>(res + nc);               // nc
    __shared__ double red[PICK_THREADS / 32];
    __shared__ int s_pick;
    const int f = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    const size_t n2 = 2 * (size_t)m;
    V += (size_t)f * n2 * nc;
    lam += (size_t)f * nc;
    Uc += (size_t)f * nm * m;
    sr += (size_t)f * nm;
    for (int c = tid; c < nc; c += blockDim.x) taken[c] = 0;
    const double ctol = 1e-12 * fmax(lam[0], 0.0);
    __syncthreads();
    int acc = 0, c0 = 0;
    while (c0 < nc && acc < nm) {
        int c1 = c0 + 1;
        while (c1 < nc && lam[c0] - lam[c1] <= ctol) ++c1;
        const int q = (c1 - c0 + 1) / 2;
        for (int t = 0; t < q && acc < nm; ++t) {
            for (int c = c0 + wid; c < c1; c += nw) {
                if (taken[c]) {
                    if (lane == 0) res[c] = -1.0;
                    continue;
                }
                const double *v = V + (size_t)c * n2;
                double nr = 0.0;
                for (int i = lane; i < m; i += 32) nr = fma(v[i], v[i], fma(v[m + i], v[m + i], nr));
                nr = warp_sum(nr);
                double pr = 0.0;
                for (int k = 0; k < acc; ++k) {
                    const double2 *u = Uc + (size_t)k * m;
                    double2 d = make_double2(0.0, 0.0);
                    for (int i = lane; i < m; i += 32) zcfma(d, u[i], make_double2(v[i], v[m + i]));
                    d = warp_sum2(d);
                    pr += zabs2(d);
                }
                if (lane == 0) res[c] = nr - pr;
            }
            __syncthreads();
            if (tid == 0) {
                int best = -1;
                double bv = 0.1;
                for (int c = c0; c < c1; ++c)
                    if (res[c] > bv) {
                        bv = res[c];
                        best = c;
                    }
                s_pick = best;
            }
            __syncthreads();
            const int pick = s_pick;
            if (pick < 0) break;
            const double *v = V + (size_t)pick * n2;
            for (int i = tid; i < m; i += blockDim.x) pk_w[i] = make_double2(v[i], v[m + i]);
            __syncthreads();
            for (int pass = 0; pass < 2; ++pass) {
                for (int k = wid; k < acc; k += nw) {
                    const double2 *u = Uc + (size_t)k * m;
                    double2 d = make_double2(0.0, 0.0);
                    for (int i = lane; i < m; i += 32) zcfma(d, u[i], pk_w[i]);     // u^H w
                    d = warp_sum2(d);
                    if (lane == 0) dots[k] = d;
                }
                __syncthreads();
                for (int i = tid; i < m; i += blockDim.x) {
                    double2 w = pk_w[i];
                    for (int k = 0; k < acc; ++k) zfms(w, dots[k], Uc[(size_t)k * m + i]);
                    pk_w[i] = w;
                }
                __syncthreads();
            }
            double nr = 0.0;
            for (int i = tid; i < m; i += blockDim.x) nr += zabs2(pk_w[i]);
            nr = warp_sum(nr);
            if (lane == 0) red[wid] = nr;
            __syncthreads();
            double tot = 0.0;
            for (int w = 0; w < nw; ++w) tot += red[w];
            const double sc = 1.0 / sqrt(tot);
            for (int i = tid; i < m; i += blockDim.x) Uc[(size_t)acc * m + i] = zscale(pk_w[i], sc);
            if (tid == 0) {
                sr[acc] = sqrt(fmax(lam[pick], 0.0));
                taken[pick] = 1;
            }
            ++acc;
            __syncthreads();
        }
        c0 = c1;
    }
    for (int k = acc; k < nm; ++k) {
        for (int i = tid; i < m; i += blockDim.x) Uc[(size_t)k * m + i] = make_double2(0.0, 0.0);
        if (tid == 0) sr[k] = 0.0;
    }
    if (tid == 0 && acc < nm && info) atomicOr(&info[f], IA_INFO_NOCONV);
    __syncthreads();
    for (int k = wid; k < acc; k += nw) {
        double2 *u = Uc + (size_t)k * m;
        const double2 ph = column_phase(m, u, lane);
        __syncwarp();
        for (int i = lane; i < m; i += 32) u[i] = zmul(u[i], ph);
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

// Subspace of the complex variant, on the real representation (every
// eigenvalue doubled): 2 (nm + max(nm, mode_oversample)) real vectors, all
// returned as Ritz vectors (a cluster of equal eigenvalues that straddles the
// 2 nm-th one needs candidates beyond it).  Mixed: 2 mode_iters FP32 and
// 4 max(1, refine_steps) double-float iterations; FP64: as many FP64 ones.
// The spectrum of G Z is dense (singular values of a 642-node sphere fall
// only to 0.15 s_1 by the 32nd), so the real variant's settings would stop
// near 1e-7 s_1; these reach ~1e-15 s_1 and residuals ~1e-11 lambda_1 there.
struct ComplexModeSub {
    ia_config cfg;
    int nr;   // real Ritz vectors
};

static ComplexModeSub complex_mode_sub(const ia_config *cfg, int m, int nm)
{
    ComplexModeSub c{*cfg, 0};
    const int p = cfg->mode_oversample > nm ? cfg->mode_oversample : nm;
    const int refine = 4 * (cfg->refine_steps > 1 ? cfg->refine_steps : 1);
    c.nr = nm + p < m ? 2 * (nm + p) : 2 * m;
    c.cfg.mode_oversample = 0;
    if (cfg->precision == IA_PREC_MIXED) {
        c.cfg.mode_iters = 2 * cfg->mode_iters;
        c.cfg.refine_steps = refine;
    } else {
        c.cfg.mode_iters = 2 * cfg->mode_iters + refine;
    }
    return c;
}

// The subspace pays while it is at most half the space (2 (nm + p) <= m);
// beyond that (invr with n_am near m) the complex variant takes the FP64
// one-sided Jacobi SVD of the whole G Z.
static bool complex_mode_subspace(const ia_config *cfg, int m, int nm)
{
    const int p = cfg->mode_oversample > nm ? cfg->mode_oversample : nm;
    return 2 * (long long)(nm + p) <= m;
}

// slices of the mixed Z solve's tensor-core products (0: double-float GEMMs)
static int bem_slices(const ia_config *cfg)
{
    if (cfg->gemm_slices < TC_SLICES_MIN) return 0;
    return cfg->gemm_slices < TC_SLICES_MAX ? cfg->gemm_slices + 1 : TC_SLICES_MAX;
}

size_t bem_modes_ws_bytes(const ia_mesh *mesh, int l, int n_ch, int F, int nm, const ia_config *cfg, bool cplx)
{
    const size_t M = mesh->m, MT = M + n_ch, L = l, FF = F;
    size_t b = 4 * ws_round(16 * MT * M * FF) + 4 * ws_round(16 * M * L * FF) + ws_round(4 * M * FF) +
               ws_round(8 * (size_t)mesh->gnnz) + ws_round(16 * M * nm * FF);
    if (cplx) {
        b += ws_round(16 * M * M * FF) + ws_round(8 * M * FF);
        if (complex_mode_subspace(cfg, mesh->m, nm)) {
            const ComplexModeSub c = complex_mode_sub(cfg, mesh->m, nm);
            const size_t NR = c.nr;
            b += ws_round(32 * M * M * FF) + ws_round(16 * M * NR * FF) + ws_round(8 * NR * FF) +
                 radiation_modes_ws_bytes(2 * mesh->m, F, c.nr, &c.cfg, true);
        }
    } else b += ws_round(8 * M * M * FF) + ws_round(8 * nm * FF) + radiation_modes_ws_bytes(mesh->m, F, nm, cfg, true);
    if (cfg->precision == IA_PREC_MIXED) b += ws_round(ibem_geom_bytes(mesh, (int)(MT + L)));   // assembly geometry
    if (bem_mixed_solve(cfg, n_ch)) {
        b += 2 * ws_round(8 * M * M * FF) + ws_round(16 * M * M * FF);
        if (tc_products_ok(bem_slices(cfg), mesh->m))
            b += tc_planes_bytes(mesh->m > l ? mesh->m : l, mesh->m, bem_slices(cfg), false, F) +
                 tc_planes_bytes(mesh->m, mesh->m, bem_slices(cfg), true, F) + 1024;
    }
    return b + 4096;
}

// Mixed Z = A^-1 B and H = A_hs Z - B_hs: A and B arrive as double-float row
// blocks (A^T, B^T as float4); FP32 LU of A and FP32 solves for Z, refined
// with FP64-level residuals B - A Z (max(1, refine_steps) times); H =
// A_hs Z - B_hs.  Both FP64-level products run on the tensor cores (BF16
// slices, one more than cfg->gemm_slices: Z's error reaches the modes through
// A's conditioning, which low kR makes large; A sliced once) or, with
// gemm_slices 0, as double-float CUDA-core GEMMs.  On exit Z (FP64, m x m) is
// in At's storage.
static int bem_mixed_z(ia_context *ctx, const ia_mesh *mesh, int l, const double *mics, int F, const double *k,
                       const ia_config *cfg, double2 *At, double2 *Bt, double2 *A, double2 *B, double2 *Ahs_t,
                       double2 *Bhs_t, double2 *Ahs, double2 *H, int *ipiv, int *info, WsCursor &cur)
{
    const int m = mesh->m;
    const long long mm = (long long)m * m, ml = (long long)m * l;
    int st;
    const size_t gbytes = ibem_geom_bytes(mesh, m + l);
    float2 *G = gbytes ? cur.take<float2>(gbytes / sizeof(float2)) : nullptr;
    if (cur.off > cur.cap) return IA_ERR_ALLOC;
    if ((st = ibem_rows(ctx, mesh, l, mics, 0, nullptr, F, k, cfg->c, cfg->rho, At, Bt, Ahs_t, Bhs_t, true, true, G)))
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
    const int S = bem_slices(cfg);
    const bool tcg = tc_products_ok(S, m);
    TcPlanes Pa{}, Pz{};
    WsCursor ca{nullptr, 0, 0}, cz{nullptr, 0, 0};
    if (tcg) {
        // A's planes once (rows of A, then of A_hs in the same region), Z's per product
        const size_t ba = tc_planes_bytes(m > l ? m : l, m, S, false, F), bz = tc_planes_bytes(m, m, S, true, F);
        ca = WsCursor{(char *)cur.take<unsigned char>(ba), 0, ba};
        cz = WsCursor{(char *)cur.take<unsigned char>(bz), 0, bz};
        if (cur.off > cur.cap) return IA_ERR_ALLOC;
        if ((st = tc_slice(ctx, false, OP_N, A4, m, mm, m, m, S, F, Pa, ca))) return st;
    }
    for (int it = 0; it < steps; ++it) {
        df_join_kernel<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(n4, B4, R);
        IA_LAUNCH_CHECK(ctx);
        if (tcg) {
            cz.off = 0;
            if ((st = tc_slice(ctx, true, OP_N, Z, m, mm, m, m, S, F, Pz, cz))) return st;
            if ((st = tc_gemm(ctx, Pa, Pz, m, m, -1.0, 1.0, R, m, mm, F, info))) return st;
        } else {
            if ((st = split_df_batched(ctx, n4, Z, Z4))) return st;
            if ((st = dfgemm4_batched(ctx, OP_N, OP_N, m, m, m, -1.0, A4, m, mm, Z4, m, mm, 1.0, R, m, mm, F)))
                return st;
        }
        if ((st = copy2d_batched<double2, float2>(ctx, m, m, R, m, mm, Z32, m, mm, false, F))) return st;
        if ((st = getrs_batched<float2>(ctx, m, m, A32, m, mm, ipiv, Z32, m, mm, F))) return st;
        if ((st = add2d_batched<float2>(ctx, m, m, Z32, m, mm, Z, m, mm, F))) return st;
    }
    // H = A_hs Z - B_hs
    if (tcg) {
        ca.off = 0;
        cz.off = 0;
        if ((st = tc_slice(ctx, false, OP_N, Ahs, l, ml, l, m, S, F, Pa, ca))) return st;
        if ((st = tc_slice(ctx, true, OP_N, Z, m, mm, m, m, S, F, Pz, cz))) return st;
        return tc_gemm(ctx, Pa, Pz, l, m, 1.0, -1.0, H, l, ml, F, info);
    }
    // (A_hs split into A_hs^T's storage)
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
        const bool df = cfg->precision == IA_PREC_MIXED;
        const size_t gbytes = df ? ibem_geom_bytes(mesh, mt + l) : 0;
        float2 *G = gbytes ? cur.take<float2>(gbytes / sizeof(float2)) : nullptr;
        if (cur.off > cur.cap) return IA_ERR_ALLOC;
        if ((st = ibem_rows(ctx, mesh, l, mics, n_ch, cp, F, k, cfg->c, cfg->rho, At, Bt, Ahs_t, Bhs_t, df, false, G)))
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
        double2 *Y = cur.take<double2>(mm * F);
        double *sfull = cur.take<double>((size_t)m * F);
        gz_kernel<true><<<gz_grid, 128, 0, ctx->stream>>>(m, mesh->d_gptr, mesh->d_gidx, gval, Z, m, mm, Y);
        IA_LAUNCH_CHECK(ctx);
        if (complex_mode_subspace(cfg, m, nm)) {
            // subspace iteration on the real representation (radiation.cu),
            // then one complex vector per doubled eigenvalue
            const ComplexModeSub c = complex_mode_sub(cfg, m, nm);
            const int n2 = 2 * m;
            double *Yr = cur.take<double>((size_t)n2 * n2 * F);
            double *V2 = cur.take<double>((size_t)n2 * c.nr * F);
            double *lam2 = cur.take<double>((size_t)c.nr * F);
            real_rep_kernel<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(m, Y, Yr, F);
            IA_LAUNCH_CHECK(ctx);
            if ((st = radiation_modes_batched(ctx, n2, F, Yr, c.nr, &c.cfg, lam2, V2, info, cur, true))) return st;
            const size_t smem = sizeof(double2) * ((size_t)m + nm) + (sizeof(double) + sizeof(int)) * (size_t)c.nr;
            if (smem > 227 * 1024) return IA_ERR_TOO_LARGE;
            if (smem > 48 * 1024)
                IA_CUDA_TRY(cudaFuncSetAttribute(modes_pick_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)smem));
            modes_pick_kernel<<<F, PICK_THREADS, smem, ctx->stream>>>(m, nm, c.nr, V2, lam2, Uc, sr, info);
        } else {
            // FP64 SVD of Y: columns orthogonalised in place, U = Y / sigma
            double2 *Ufull = Bt;
            if ((st = jacobi_svd_batched(ctx, m, m, Y, nullptr, F, cfg->svd_max_sweeps, info))) return st;
            if ((st = svd_finalize_batched(ctx, m, m, Y, nullptr, sfull, Ufull, nullptr, F, info))) return st;
            modes_phase_kernel<<<F, 256, 0, ctx->stream>>>(m, nm, Ufull, sfull, Uc, sr);
        }
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
