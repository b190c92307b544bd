// IBEM collocation rows, FP64, gather form, frequency-blocked.
//
// Follows the reference's CPU ibem() assembly (CUDA/ibem.cuh:486-738; GPU
// kernels :1-261), the OpenBEM collocation scheme on linear triangles:
//   x_q = xi1 v0 + xi2 v1 + (1-xi1-xi2) v2, n = (v0 - v2) x (v1 - v2)
//   g = exp(ikr)/r, ft = n.(x_q - x_o)/r^2
//   B[o, v] += w N_v |n| g / 4pi,  A[o, v] += w N_v ft (ikr - 1) g / 4pi
//   C[o] += w (-ft/r) / 4pi over every element; A[o,o] -= 1 + C[o]
//   elements incident to a surface node use that vertex's singular-rule page
//   field and CHIEF rows use the regular rule and no C term
//   B scaled by i rho c k
//
// Layout of the work: one CTA owns one row (collocation point) for a block of
// FB consecutive frequencies and keeps those FB rows of A and B in shared
// memory.  Its threads walk the elements colour by colour: elements of one
// colour share no vertex, so the three column updates of all threads never
// collide and need no atomics; colours are separated by __syncthreads().  The
// per-(element, quadrature point) geometry -- x_q, w N_v / 4pi,
// w N_v |n| / 4pi -- is precomputed at mesh creation.  Within a block,
// exp(i k_f r) advances by one complex multiply per frequency when the k_f are
// evenly spaced (exp(i k_{f+1} r) = exp(i k_f r) exp(i dk r)), and is
// evaluated directly otherwise.  For a surface row, the elements incident to
// the node use the singular rule: each warp takes one of them, lanes stride
// the rule's points, shuffles reduce in a fixed order.  Rows are written once,
// coalesced, row-major (the transpose of the reference's column-major
// ass/bss/ahs/bhs, CUDA/ibem.cuh:481-482, :621-622).  Results are
// deterministic.
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

constexpr int IBEM_FB = 4;          // frequencies per CTA
constexpr int IBEM_THREADS = 128;   // 4 warps
constexpr int IBEM_MAX_NQ = 64;

// per-frequency phase factors of one block
struct FreqBlock {
    double k[IBEM_FB];
    double dk;
    int nf;
    bool uniform;
};

// Regular-rule integral of one element against x_o for the block's
// frequencies.  qd: precomputed (x, y, z, wa0..2, wb0..2) for each point,
// structure of arrays with stride n (elements) and 9 * n per point.
__device__ __forceinline__ void regular_element(const double *__restrict__ qd, int n, int e, int nq, double nx,
                                                double ny, double nz, double xo, double yo, double zo,
                                                const FreqBlock &fb, double2 (&a)[IBEM_FB][3],
                                                double2 (&b)[IBEM_FB][3], double &ct)
{
    for (int q = 0; q < nq; ++q) {
        const double *p = qd + (size_t)q * 9 * n + e;
        const double dx = p[0] - xo, dy = p[(size_t)n] - yo, dz = p[2 * (size_t)n] - zo;
        const double wa[3] = {p[3 * (size_t)n], p[4 * (size_t)n], p[5 * (size_t)n]};
        const double wb[3] = {p[6 * (size_t)n], p[7 * (size_t)n], p[8 * (size_t)n]};
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double invr = rsqrt(r2);
        const double r = r2 * invr;
        const double ft = (nx * dx + ny * dy + nz * dz) * (invr * invr);
        ct = fma(-(wa[0] + wa[1] + wa[2]) * ft, invr, ct);
        double2 ph, step = make_double2(1.0, 0.0);
        {
            double s, c;
            sincos(fb.k[0] * r, &s, &c);
            ph = make_double2(c, s);
            if (fb.uniform && fb.nf > 1) {
                sincos(fb.dk * r, &s, &c);
                step = make_double2(c, s);
            }
        }
#pragma unroll
        for (int f = 0; f < IBEM_FB; ++f) {
            if (f >= fb.nf) break;
            if (f > 0) {
                if (fb.uniform) ph = zmul(ph, step);
                else {
                    double s, c;
                    sincos(fb.k[f] * r, &s, &c);
                    ph = make_double2(c, s);
                }
            }
            const double gr = ph.x * invr, gi = ph.y * invr;
            const double kr = fb.k[f] * r;
            const double tr = -gr - kr * gi, ti = kr * gr - gi;   // (ikr - 1) g
#pragma unroll
            for (int v = 0; v < 3; ++v) {
                const double sa = wa[v] * ft;
                a[f][v].x = fma(sa, tr, a[f][v].x);
                a[f][v].y = fma(sa, ti, a[f][v].y);
                b[f][v].x = fma(wb[v], gr, b[f][v].x);
                b[f][v].y = fma(wb[v], gi, b[f][v].y);
            }
        }
    }
}

// Singular-rule integral of one element (raw geometry eg, rule SoA) against
// x_o, lanes striding the points; reduced over the warp on return.
__device__ __forceinline__ void singular_element(const double *__restrict__ eg, const double *__restrict__ rule, int nq,
                                                 double xo, double yo, double zo, const FreqBlock &fb, int lane,
                                                 double2 (&a)[IBEM_FB][3], double2 (&b)[IBEM_FB][3], double &ct)
{
    const double v0x = eg[0], v0y = eg[1], v0z = eg[2];
    const double v1x = eg[3], v1y = eg[4], v1z = eg[5];
    const double v2x = eg[6], v2y = eg[7], v2z = eg[8];
    const double nx = eg[9], ny = eg[10], nz = eg[11], an = eg[12];
    for (int q = lane; q < nq; q += 32) {
        const double x1 = rule[q], x2 = rule[q + nq], w = rule[q + 2 * nq] * IA_INV4PI;
        const double x3 = 1.0 - x1 - x2;
        const double dx = x1 * v0x + x2 * v1x + x3 * v2x - xo;
        const double dy = x1 * v0y + x2 * v1y + x3 * v2y - yo;
        const double dz = x1 * v0z + x2 * v1z + x3 * v2z - zo;
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double invr = rsqrt(r2);
        const double r = r2 * invr;
        const double ft = (nx * dx + ny * dy + nz * dz) * (invr * invr);
        ct = fma(-w * ft, invr, ct);
        const double N[3] = {x1, x2, x3};
#pragma unroll
        for (int f = 0; f < IBEM_FB; ++f) {
            if (f >= fb.nf) break;
            double s, c;
            sincos(fb.k[f] * r, &s, &c);
            const double gr = c * invr, gi = s * invr;
            const double kr = fb.k[f] * r;
            const double tr = -gr - kr * gi, ti = kr * gr - gi;
#pragma unroll
            for (int v = 0; v < 3; ++v) {
                const double sa = w * N[v] * ft, sb = w * N[v] * an;
                a[f][v].x = fma(sa, tr, a[f][v].x);
                a[f][v].y = fma(sa, ti, a[f][v].y);
                b[f][v].x = fma(sb, gr, b[f][v].x);
                b[f][v].y = fma(sb, gi, b[f][v].y);
            }
        }
    }
}

__global__ void __launch_bounds__(IBEM_THREADS) ibem_rows_kernel(
    int m, int n, int l, int n_ch, int ncolors, int F, const double *__restrict__ nodes, const double *__restrict__ egeo,
    const double *__restrict__ qdat, const int *__restrict__ evert, const int *__restrict__ color_ptr,
    const int *__restrict__ adj_ptr, const int *__restrict__ adj, int nq, const double *__restrict__ sing, int nqs,
    const double *__restrict__ mics, const double *__restrict__ cp, const double *__restrict__ kv, double c,
    double rho, double2 *__restrict__ At, double2 *__restrict__ Bt, double2 *__restrict__ Ahs_t,
    double2 *__restrict__ Bhs_t)
{
    extern __shared__ double2 rowbuf[];   // IBEM_FB x (A row, B row), m each
    __shared__ double ct_red[IBEM_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int row = blockIdx.x;
    const int f0 = blockIdx.y * IBEM_FB;
    const int mt = m + n_ch;
    FreqBlock fb;
    fb.nf = F - f0 < IBEM_FB ? F - f0 : IBEM_FB;
#pragma unroll
    for (int f = 0; f < IBEM_FB; ++f) fb.k[f] = kv[f0 + (f < fb.nf ? f : fb.nf - 1)];
    fb.dk = fb.nf > 1 ? fb.k[1] - fb.k[0] : 0.0;
    fb.uniform = true;
#pragma unroll
    for (int f = 2; f < IBEM_FB; ++f)
        if (f < fb.nf && fabs(fb.k[f] - (fb.k[0] + f * fb.dk)) > 1e-12 * fabs(fb.k[f])) fb.uniform = false;
    for (int j = tid; j < 2 * IBEM_FB * m; j += blockDim.x) rowbuf[j] = make_double2(0.0, 0.0);
    double xo, yo, zo;
    int self = -1;
    if (row < m) {
        xo = nodes[row]; yo = nodes[row + m]; zo = nodes[row + 2 * m];
        self = row;
    } else if (row < mt) {
        int i = row - m;
        xo = cp[i]; yo = cp[i + n_ch]; zo = cp[i + 2 * n_ch];
    } else {
        int i = row - mt;
        xo = mics[i]; yo = mics[i + l]; zo = mics[i + 2 * l];
    }
    __syncthreads();
    double ct = 0.0;
    const double *nrm = egeo;   // normals at egeo[(9 + d) + 16 e]
    for (int cidx = 0; cidx < ncolors; ++cidx) {
        const int e0 = color_ptr[cidx], e1 = color_ptr[cidx + 1];
        for (int e = e0 + tid; e < e1; e += blockDim.x) {
            const int4 vv = reinterpret_cast<const int4 *>(evert)[e];
            if (vv.x == self || vv.y == self || vv.z == self) continue;
            double2 a[IBEM_FB][3], b[IBEM_FB][3];
#pragma unroll
            for (int f = 0; f < IBEM_FB; ++f)
#pragma unroll
                for (int v = 0; v < 3; ++v) { a[f][v] = make_double2(0.0, 0.0); b[f][v] = make_double2(0.0, 0.0); }
            const double *g = nrm + (size_t)e * 16;
            regular_element(qdat, n, e, nq, g[9], g[10], g[11], xo, yo, zo, fb, a, b, ct);
            const int cols[3] = {vv.x, vv.y, vv.z};
#pragma unroll
            for (int f = 0; f < IBEM_FB; ++f) {
                if (f >= fb.nf) break;
                double2 *Ar = rowbuf + (size_t)f * 2 * m, *Br = Ar + m;
#pragma unroll
                for (int v = 0; v < 3; ++v) {
                    Ar[cols[v]] = zadd(Ar[cols[v]], a[f][v]);
                    Br[cols[v]] = zadd(Br[cols[v]], b[f][v]);
                }
            }
        }
        __syncthreads();
    }
    // singular elements of a surface row: one warp per incident element
    if (self >= 0) {
        const int a0 = adj_ptr[self], a1 = adj_ptr[self + 1];
        for (int base = a0; base < a1; base += IBEM_THREADS / 32) {
            const int ai = base + wid;
            double2 a[IBEM_FB][3], b[IBEM_FB][3];
#pragma unroll
            for (int f = 0; f < IBEM_FB; ++f)
#pragma unroll
                for (int v = 0; v < 3; ++v) { a[f][v] = make_double2(0.0, 0.0); b[f][v] = make_double2(0.0, 0.0); }
            int e = -1, slot = 0;
            if (ai < a1) {
                const int code = adj[ai];
                e = code >> 2;
                slot = code & 3;
                singular_element(egeo + (size_t)e * 16, sing + (size_t)3 * nqs * slot, nqs, xo, yo, zo, fb, lane, a,
                                 b, ct);
            }
            // warps take turns so two incident elements never update a column together
            for (int w = 0; w < IBEM_THREADS / 32; ++w) {
                if (w == wid && e >= 0) {
#pragma unroll
                    for (int f = 0; f < IBEM_FB; ++f)
#pragma unroll
                        for (int v = 0; v < 3; ++v) {
                            a[f][v] = warp_sum2(a[f][v]);
                            b[f][v] = warp_sum2(b[f][v]);
                        }
                    if (lane == 0) {
                        const int4 vv = reinterpret_cast<const int4 *>(evert)[e];
                        const int cols[3] = {vv.x, vv.y, vv.z};
#pragma unroll
                        for (int f = 0; f < IBEM_FB; ++f) {
                            if (f >= fb.nf) break;
                            double2 *Ar = rowbuf + (size_t)f * 2 * m, *Br = Ar + m;
#pragma unroll
                            for (int v = 0; v < 3; ++v) {
                                Ar[cols[v]] = zadd(Ar[cols[v]], a[f][v]);
                                Br[cols[v]] = zadd(Br[cols[v]], b[f][v]);
                            }
                        }
                    }
                }
                __syncthreads();
            }
        }
        // C term: every element's contribution, reduced in a fixed order
        double cs = warp_sum(ct);
        if (lane == 0) ct_red[wid] = cs;
        __syncthreads();
        if (tid == 0) {
            double tot = 0.0;
            for (int w = 0; w < IBEM_THREADS / 32; ++w) tot += ct_red[w];
            for (int f = 0; f < fb.nf; ++f) rowbuf[(size_t)f * 2 * m + self].x -= 1.0 + tot;
        }
        __syncthreads();
    }
    // scale B by i rho c k and write the rows
    for (int f = 0; f < fb.nf; ++f) {
        const int fg = f0 + f;
        const double s = rho * c * fb.k[f];
        const double2 *Ar = rowbuf + (size_t)f * 2 * m, *Br = Ar + m;
        double2 *arow, *brow;
        if (row < mt) {
            arow = At ? At + ((size_t)fg * mt + row) * m : nullptr;
            brow = Bt ? Bt + ((size_t)fg * mt + row) * m : nullptr;
        } else {
            arow = Ahs_t ? Ahs_t + ((size_t)fg * l + (row - mt)) * m : nullptr;
            brow = Bhs_t ? Bhs_t + ((size_t)fg * l + (row - mt)) * m : nullptr;
        }
        for (int j = tid; j < m; j += blockDim.x) {
            if (arow) arow[j] = Ar[j];
            const double2 bv = Br[j];
            if (brow) brow[j] = make_double2(-s * bv.y, s * bv.x);
        }
    }
}

int ibem_rows(ia_context *ctx, const ia_mesh *mesh, int l, const double *mics, int n_ch, const double *cp, int F,
              const double *k, double c, double rho, double2 *At, double2 *Bt, double2 *Ahs_t, double2 *Bhs_t)
{
    if (mesh->nq > IBEM_MAX_NQ) return IA_ERR_RULE;
    const int m = mesh->m;
    const int rows = m + n_ch + l;
    const size_t smem = sizeof(double2) * 2 * (size_t)m * IBEM_FB;
    if (smem > 220 * 1024) return IA_ERR_TOO_LARGE;
    IA_CUDA_TRY(cudaFuncSetAttribute(ibem_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    dim3 g(rows, (F + IBEM_FB - 1) / IBEM_FB);
    ibem_rows_kernel<<<g, IBEM_THREADS, smem, ctx->stream>>>(
        m, mesh->n, l, n_ch, mesh->ncolors, F, mesh->d_nodes, mesh->d_egeo, mesh->d_qdat, mesh->d_evert,
        mesh->d_color_ptr, mesh->d_adj_ptr, mesh->d_adj, mesh->nq, mesh->d_sing, mesh->nqs, mics, cp, k, c, rho, At,
        Bt, Ahs_t, Bhs_t);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

}  // namespace ia
