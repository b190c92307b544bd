// IBEM collocation rows, gather form, frequency-blocked.
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
// w N_v |n| / 4pi -- is precomputed at mesh creation; the double-float
// kernel also reads the per-(row, element, point) r, 1/r and n.(x_q - x_o)/r^2
// from a table computed once per call (ibem_geom_kernel), where the caller
// gives it workspace for one.  Within a block,
// exp(i k_f r) advances by one complex multiply per frequency when the k_f are
// evenly spaced (exp(i k_{f+1} r) = exp(i k_f r) exp(i dk r)), and is
// evaluated directly otherwise.  For a surface row, the elements incident to
// the node use the singular rule: each warp takes one of them, lanes stride
// the rule's points, shuffles reduce in a fixed order.  Rows are written once,
// coalesced, row-major (the transpose of the reference's column-major
// ass/bss/ahs/bhs, CUDA/ibem.cuh:481-482, :621-622).  Results are
// deterministic.
//
// The regular-element arithmetic is generic in its real type R: double for
// the FP64 path, double-float (dfl, df32.cuh) for the mixed path, which moves
// the dominant work from GB300's FP64 pipe to its FP32 pipe at ~1e-14
// relative accuracy.  The singular elements stay FP64 in both.
#include <cstdlib>
#include <type_traits>
#include "df32.cuh"
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

// Frequencies per CTA.  FP64: 4, so the geometry and the singular-element
// work of the slow FP64 pipe serve four frequencies.  Double-float: 1 -- the
// accumulators of a block dominate the registers (244 at 4, 146 at 2, 96 at
// 1) and the row buffers the shared memory, so one frequency per CTA runs 5
// CTAs per SM instead of 2, which outweighed recomputing the geometry per
// frequency (measured per 64-bin launch: 13.1 ms at 4, 11.7 at 2, 11.0 at 1;
// with the table-driven sin/cos the whole 64-bin pass still ran 28.2 ms at 2
// against 27.9 at 1).  With the geometry table the frequencies of a row share
// the geometry through L2 instead, and the kernel runs 7 CTAs per SM (72
// registers, the sin/cos table read through L1): 10.3 -> 7.3 ms per 64-bin
// assembly.  The launch bounds keep the inline double-float kernel at 5 CTAs
// per SM (96 registers) and the FP64 kernel at 3 (168).
constexpr int IBEM_FB_MAX = 4;
template <class R> struct AsmBlock { static constexpr int FB = 4; };
template <> struct AsmBlock<dfl> { static constexpr int FB = 1; };
constexpr int IBEM_THREADS = IA_ASM_THREADS;   // 4 warps; mesh colours are balanced to this
constexpr int IBEM_MAX_NQ = 64;

// ---- the real-type policy -------------------------------------------------
__device__ __forceinline__ double r_from(double x) { return x; }
__device__ __forceinline__ double r_to_double(double x) { return x; }
__device__ __forceinline__ double r_add(double a, double b) { return a + b; }
__device__ __forceinline__ double r_sub(double a, double b) { return a - b; }
__device__ __forceinline__ double r_mul(double a, double b) { return a * b; }
__device__ __forceinline__ void r_mac(double &acc, double a, double b) { acc = fma(a, b, acc); }
__device__ __forceinline__ double r_norm(double a) { return a; }
__device__ __forceinline__ double r_rsqrt(double a) { return rsqrt(a); }
__device__ __forceinline__ double r_zero(double) { return 0.0; }
__device__ __forceinline__ void r_sincos(double theta, const float4 *, const DfTrigRed &, const DfTrigCoef &, double &s,
                                         double &c)
{
    sincos(theta, &s, &c);
}

__device__ __forceinline__ dfl r_from(dfl x) { return x; }
__device__ __forceinline__ double r_to_double(dfl x) { return df_to_double(x); }
__device__ __forceinline__ dfl r_add(dfl a, dfl b) { return df_add(a, b); }
__device__ __forceinline__ dfl r_sub(dfl a, dfl b) { return df_sub(a, b); }
__device__ __forceinline__ dfl r_mul(dfl a, dfl b) { return df_mul(a, b); }
__device__ __forceinline__ void r_mac(dfl &acc, dfl a, dfl b) { df_mac(acc, a, b); }
__device__ __forceinline__ dfl r_norm(dfl a) { return df_norm(a); }
__device__ __forceinline__ dfl r_rsqrt(dfl a) { return df_rsqrt(a); }
__device__ __forceinline__ dfl r_zero(dfl) { return dfl{0.0f, 0.0f}; }
__device__ __forceinline__ void r_sincos(dfl theta, const float4 *tab, const DfTrigRed &P, const DfTrigCoef &C, dfl &s,
                                         dfl &c)
{
    df_sincos_tab(theta, tab, P, C, s, c);
}

template <class R> __device__ __forceinline__ R r_of_double(double x);
template <> __device__ __forceinline__ double r_of_double<double>(double x) { return x; }
template <> __device__ __forceinline__ dfl r_of_double<dfl>(double x) { return df_from_double(x); }

template <class R>
struct cx {
    R re, im;
};

template <class R> __device__ __forceinline__ cx<R> cx_zero() { return cx<R>{r_zero(R()), r_zero(R())}; }
template <class R> __device__ __forceinline__ cx<R> cx_add(cx<R> a, cx<R> b) { return cx<R>{r_add(a.re, b.re), r_add(a.im, b.im)}; }
template <class R> __device__ __forceinline__ cx<R> cx_mul(cx<R> a, cx<R> b)
{
    return cx<R>{r_sub(r_mul(a.re, b.re), r_mul(a.im, b.im)), r_add(r_mul(a.re, b.im), r_mul(a.im, b.re))};
}
template <class R> __device__ __forceinline__ cx<R> cx_norm(cx<R> a) { return cx<R>{r_norm(a.re), r_norm(a.im)}; }

// per-frequency phase factors of one block
struct FreqBlock {
    double k[IBEM_FB_MAX];
    double dk;
    int nf;
    bool uniform;
};

// Frequency-independent geometry of one quadrature point p (x, y, z at
// stride n) against x_o: r, 1/r and ft = n.(x_q - x_o) / r^2.
template <class R>
__device__ __forceinline__ void point_geometry(const R *__restrict__ p, int n, R nx, R ny, R nz, R xo, R yo, R zo,
                                               R &r, R &invr, R &ft)
{
    const R dx = r_sub(p[0], xo), dy = r_sub(p[(size_t)n], yo), dz = r_sub(p[2 * (size_t)n], zo);
    const R r2 = r_add(r_add(r_mul(dx, dx), r_mul(dy, dy)), r_mul(dz, dz));
    invr = r_rsqrt(r2);
    r = r_mul(r2, invr);
    const R nd = r_add(r_add(r_mul(nx, dx), r_mul(ny, dy)), r_mul(nz, dz));
    ft = r_mul(nd, r_mul(invr, invr));
}

// Regular-rule integral of one element against x_o for the block's
// frequencies.  qd: precomputed (x, y, z, wa0..2, wb0..2) for each point,
// structure of arrays with stride n (elements) and 9 * n per point.  GT: the
// point geometry (r, 1/r, ft) is read from this row's geometry table gq
// (ibem_geom_kernel; planes of stride n, 3 n per point) instead of computed.
template <class R, int FB, bool CT, bool GT>
__device__ __forceinline__ void regular_element(const R *__restrict__ qd, int n, int e, int nq, R nx, R ny, R nz,
                                                R xo, R yo, R zo, const float2 *__restrict__ gq,
                                                const FreqBlock &fb, const R (&kf)[FB], R dkf,
                                                const float4 *tab, const DfTrigRed &P, const DfTrigCoef &C,
                                                const R *cw, cx<R> (&a)[FB][3], cx<R> (&b)[FB][3], R &ct)
{
    for (int q = 0; q < nq; ++q) {
        const R *p = qd + (size_t)q * 9 * n + e;
        const R wa[3] = {p[3 * (size_t)n], p[4 * (size_t)n], p[5 * (size_t)n]};
        const R wb[3] = {p[6 * (size_t)n], p[7 * (size_t)n], p[8 * (size_t)n]};
        R r, invr, ft;
        if constexpr (GT) {
            const float2 *g = gq + (size_t)q * 3 * n;
            const float2 g0 = g[0], g1 = g[(size_t)n], g2 = g[2 * (size_t)n];
            r = R{g0.x, g0.y};
            invr = R{g1.x, g1.y};
            ft = R{g2.x, g2.y};
        } else {
            point_geometry(p, n, nx, ny, nz, xo, yo, zo, r, invr, ft);
        }
        if (CT) r_mac(ct, r_mul(cw[q], ft), r_sub(r_zero(R()), invr));   // C term: w_q / 4pi (-ft / r)
        cx<R> ph, step;
        r_sincos(r_mul(kf[0], r), tab, P, C, ph.im, ph.re);
        if (fb.uniform && fb.nf > 1) r_sincos(r_mul(dkf, r), tab, P, C, step.im, step.re);
        R sa[3];
#pragma unroll
        for (int v = 0; v < 3; ++v) sa[v] = r_mul(wa[v], ft);
#pragma unroll
        for (int f = 0; f < FB; ++f) {
            if (f >= fb.nf) break;
            if (f > 0) {
                if (fb.uniform) ph = cx_mul(ph, step);
                else r_sincos(r_mul(kf[f], r), tab, P, C, ph.im, ph.re);
            }
            const R gr = r_mul(ph.re, invr), gi = r_mul(ph.im, invr);
            const R kr = r_mul(kf[f], r);
            const R tr = r_sub(r_sub(r_zero(R()), gr), r_mul(kr, gi));   // (ikr - 1) g
            const R ti = r_sub(r_mul(kr, gr), gi);
#pragma unroll
            for (int v = 0; v < 3; ++v) {
                r_mac(a[f][v].re, sa[v], tr);
                r_mac(a[f][v].im, sa[v], ti);
                r_mac(b[f][v].re, wb[v], gr);
                r_mac(b[f][v].im, wb[v], gi);
            }
        }
    }
}

// Singular-rule integral of one element (raw geometry eg, rule SoA) against
// x_o, FP64; the caller reduces over the warp.  With nq <= 16 the lanes split
// as (point, half of the frequency block): each lane evaluates half the
// frequencies, so all 32 lanes work; otherwise lanes stride the points.
template <int FB>
__device__ __forceinline__ void singular_element(const double *__restrict__ eg, const double *__restrict__ rule, int nq,
                                                 double xo, double yo, double zo, const FreqBlock &fb, int lane,
                                                 double2 (&a)[FB][3], double2 (&b)[FB][3], double &ct)
{
    const double v0x = eg[0], v0y = eg[1], v0z = eg[2];
    const double v1x = eg[3], v1y = eg[4], v1z = eg[5];
    const double v2x = eg[6], v2y = eg[7], v2z = eg[8];
    const double nx = eg[9], ny = eg[10], nz = eg[11], an = eg[12];
    const bool halves = nq <= 16 && FB >= 2;
    const int q0 = halves ? (lane & 15) : lane, qstep = halves ? 16 : 32;
    const int fh = halves ? (lane >> 4) * (FB / 2) : 0, fcount = halves ? FB / 2 : FB;
    for (int q = q0; q < nq; q += qstep) {
        const double x1 = rule[q], x2 = rule[q + nq], w = rule[q + 2 * nq] * IA_INV4PI;
        const double x3 = 1.0 - x1 - x2;
        const double dx = x1 * v0x + x2 * v1x + x3 * v2x - xo;
        const double dy = x1 * v0y + x2 * v1y + x3 * v2y - yo;
        const double dz = x1 * v0z + x2 * v1z + x3 * v2z - zo;
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double invr = rsqrt(r2);
        const double r = r2 * invr;
        const double ft = (nx * dx + ny * dy + nz * dz) * (invr * invr);
        if (fh == 0) ct = fma(-w * ft, invr, ct);
        const double N[3] = {x1, x2, x3};
#pragma unroll
        for (int f = 0; f < FB; ++f) {
            if (f >= fb.nf) break;
            if (f < fh || f >= fh + fcount) continue;
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

__device__ __forceinline__ void write_split_rows(int m, int tid, const cx<double> *, const cx<double> *, double,
                                                 float4 *, float4 *)
{
}

__device__ __forceinline__ void write_split_rows(int m, int tid, const cx<dfl> *Ar, const cx<dfl> *Br, double s,
                                                 float4 *arow, float4 *brow)
{
    const dfl sd = df_from_double(s);
    for (int j = tid; j < m; j += IBEM_THREADS) {
        if (arow) {
            const dfl re = df_norm(Ar[j].re), im = df_norm(Ar[j].im);
            arow[j] = make_float4(re.hi, im.hi, re.lo, im.lo);
        }
        if (brow) {
            const dfl re = df_neg(df_mul(sd, Br[j].im)), im = df_mul(sd, Br[j].re);   // i s B
            brow[j] = make_float4(re.hi, im.hi, re.lo, im.lo);
        }
    }
}

template <class R, bool GT>
__global__ void __launch_bounds__(IBEM_THREADS, GT ? 7 : std::is_same<R, dfl>::value ? 5 : 3) ibem_rows_kernel(
    int m, int n, int l, int n_ch, int ncolors, int F, const double *__restrict__ nodes, const double *__restrict__ egeo,
    const R *__restrict__ qdat, const R *__restrict__ qnrm, const int *__restrict__ evert,
    const int *__restrict__ color_ptr, const int *__restrict__ adj_ptr, const int *__restrict__ adj, int nq,
    const double *__restrict__ reg,
    const double *__restrict__ sing, int nqs, const double *__restrict__ mics, const double *__restrict__ cp,
    const double *__restrict__ kv, double c, double rho, DfTrigCoef C, DfTrigRed P, const float4 *__restrict__ dftab,
    int split_ab, const double *__restrict__ creg, const float2 *__restrict__ gtab, double2 *__restrict__ At,
    double2 *__restrict__ Bt, double2 *__restrict__ Ahs_t, double2 *__restrict__ Bhs_t)
{
    constexpr int FB = AsmBlock<R>::FB;
    extern __shared__ __align__(16) unsigned char ibem_smem[];
    cx<R> *rowbuf = reinterpret_cast<cx<R> *>(ibem_smem);   // FB x (A row, B row), m each
    constexpr bool DF = std::is_same<R, dfl>::value;
    // sin/cos table: staged in shared memory, except in the table-reading
    // kernel, which reads it through L1 (its 16 KB make room for a seventh
    // CTA per SM)
    float4 *tab_s = DF && !GT ? reinterpret_cast<float4 *>(rowbuf + 2 * FB * (size_t)m) : nullptr;
    const float4 *tab = DF ? (GT ? dftab : tab_s) : nullptr;
    __shared__ double ct_red[IBEM_THREADS / 32];
    __shared__ R cw[IBEM_MAX_NQ];   // regular-rule weights w_q / 4pi (the C term)
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    // with the geometry table the frequency blocks of one row are consecutive
    // CTAs (one 1-D grid), so they read the row's table from L2 together
    const int nfb = (F + FB - 1) / FB;
    const int row = GT ? (int)(blockIdx.x / nfb) : (int)blockIdx.x;
    const int f0 = (GT ? (int)(blockIdx.x % nfb) : (int)blockIdx.y) * FB;
    const int mt = m + n_ch;
    FreqBlock fb;
    fb.nf = F - f0 < FB ? F - f0 : FB;
#pragma unroll
    for (int f = 0; f < FB; ++f) fb.k[f] = kv[f0 + (f < fb.nf ? f : fb.nf - 1)];
    fb.dk = fb.nf > 1 ? fb.k[1] - fb.k[0] : 0.0;
    fb.uniform = true;
#pragma unroll
    for (int f = 2; f < FB; ++f)
        if (f < fb.nf && fabs(fb.k[f] - (fb.k[0] + f * fb.dk)) > 1e-12 * fabs(fb.k[f])) fb.uniform = false;
    R kf[FB];
#pragma unroll
    for (int f = 0; f < FB; ++f) kf[f] = r_of_double<R>(fb.k[f]);
    const R dkf = r_of_double<R>(fb.dk);
    for (int j = tid; j < 2 * FB * m; j += blockDim.x) rowbuf[j] = cx_zero<R>();
    if (tab_s)
        for (int j = tid; j < DF_TRIG_TABLE; j += blockDim.x) tab_s[j] = dftab[j];
    for (int q = tid; q < nq; q += blockDim.x) cw[q] = r_of_double<R>(reg[q + 2 * nq] * IA_INV4PI);
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
    const R xr = r_of_double<R>(xo), yr = r_of_double<R>(yo), zr = r_of_double<R>(zo);
    __syncthreads();
    R ctr = r_zero(R());
    for (int cidx = 0; cidx < ncolors; ++cidx) {
        const int e0 = color_ptr[cidx], e1 = color_ptr[cidx + 1];
        for (int e = e0 + tid; e < e1; e += blockDim.x) {
            const int4 vv = reinterpret_cast<const int4 *>(evert)[e];
            if (vv.x == self || vv.y == self || vv.z == self) continue;
            cx<R> a[FB][3], b[FB][3];
#pragma unroll
            for (int f = 0; f < FB; ++f)
#pragma unroll
                for (int v = 0; v < 3; ++v) { a[f][v] = cx_zero<R>(); b[f][v] = cx_zero<R>(); }
            const float2 *gq = GT ? gtab + (size_t)row * nq * 3 * n + e : nullptr;
            regular_element<R, FB, !DF, GT>(qdat, n, e, nq, qnrm[e], qnrm[e + n], qnrm[e + 2 * (size_t)n], xr, yr,
                                            zr, gq, fb, kf, dkf, tab, P, C, cw, a, b, ctr);
            if (!DF) ctr = r_norm(ctr);
            const int cols[3] = {vv.x, vv.y, vv.z};
#pragma unroll
            for (int f = 0; f < FB; ++f) {
                if (f >= fb.nf) break;
                cx<R> *Ar = rowbuf + (size_t)f * 2 * m, *Br = Ar + m;
#pragma unroll
                for (int v = 0; v < 3; ++v) {
                    Ar[cols[v]] = cx_add(Ar[cols[v]], cx_norm(a[f][v]));
                    Br[cols[v]] = cx_add(Br[cols[v]], cx_norm(b[f][v]));
                }
            }
        }
        __syncthreads();
    }
    double ct = r_to_double(ctr);
    // singular elements of a surface row: one warp per incident element
    if (self >= 0) {
        const int a0 = adj_ptr[self], a1 = adj_ptr[self + 1];
        for (int base = a0; base < a1; base += IBEM_THREADS / 32) {
            const int ai = base + wid;
            double2 a[FB][3], b[FB][3];
#pragma unroll
            for (int f = 0; f < FB; ++f)
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
                    for (int f = 0; f < FB; ++f)
#pragma unroll
                        for (int v = 0; v < 3; ++v) {
                            a[f][v] = warp_sum2(a[f][v]);
                            b[f][v] = warp_sum2(b[f][v]);
                        }
                    if (lane == 0) {
                        const int4 vv = reinterpret_cast<const int4 *>(evert)[e];
                        const int cols[3] = {vv.x, vv.y, vv.z};
#pragma unroll
                        for (int f = 0; f < FB; ++f) {
                            if (f >= fb.nf) break;
                            cx<R> *Ar = rowbuf + (size_t)f * 2 * m, *Br = Ar + m;
#pragma unroll
                            for (int v = 0; v < 3; ++v) {
                                Ar[cols[v]] = cx_add(Ar[cols[v]], cx<R>{r_of_double<R>(a[f][v].x), r_of_double<R>(a[f][v].y)});
                                Br[cols[v]] = cx_add(Br[cols[v]], cx<R>{r_of_double<R>(b[f][v].x), r_of_double<R>(b[f][v].y)});
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
            // the regular elements' part: evaluated above (FP64 kernel) or
            // once per mesh (creg, double-float kernel)
            double tot = DF ? creg[self] : 0.0;
            for (int w = 0; w < IBEM_THREADS / 32; ++w) tot += ct_red[w];
            const R diag = r_of_double<R>(-(1.0 + tot));
            for (int f = 0; f < fb.nf; ++f) {
                cx<R> &d = rowbuf[(size_t)f * 2 * m + self];
                d.re = r_add(d.re, diag);
            }
        }
        __syncthreads();
    }
    // scale B by i rho c k and write the rows (FP64)
    for (int f = 0; f < fb.nf; ++f) {
        const int fg = f0 + f;
        const double s = rho * c * fb.k[f];
        const cx<R> *Ar = rowbuf + (size_t)f * 2 * m, *Br = Ar + m;
        double2 *arow, *brow;
        // the row's offset in its output (F x mt x m surface rows or F x l x m field rows)
        [[maybe_unused]] const long long roff =
            row < mt ? ((long long)fg * mt + row) * m : ((long long)fg * l + (row - mt)) * m;
        [[maybe_unused]] const long long rext = row < mt ? (long long)F * mt * m : (long long)F * l * m;
        if (!IA_IDX_OK(roff + m - 1, rext)) continue;
        if (row < mt) {
            arow = At ? At + ((size_t)fg * mt + row) * m : nullptr;
            brow = Bt ? Bt + ((size_t)fg * mt + row) * m : nullptr;
        } else {
            arow = Ahs_t ? Ahs_t + ((size_t)fg * l + (row - mt)) * m : nullptr;
            brow = Bhs_t ? Bhs_t + ((size_t)fg * l + (row - mt)) * m : nullptr;
        }
        if (DF && split_ab && row < mt) {
            // A and B rows of the surface system as (re hi, im hi, re lo, im lo)
            // pairs for the double-float GEMMs (the normalised pair equals the
            // split of the FP64 value)
            write_split_rows(m, tid, Ar, Br, s, reinterpret_cast<float4 *>(arow), reinterpret_cast<float4 *>(brow));
            continue;
        }
        for (int j = tid; j < m; j += blockDim.x) {
            if (arow) arow[j] = make_double2(r_to_double(Ar[j].re), r_to_double(Ar[j].im));
            const double br = r_to_double(Br[j].re), bi = r_to_double(Br[j].im);
            if (brow) brow[j] = make_double2(-s * bi, s * br);
        }
    }
}

// The regular elements' C term per surface node, FP64: the frequency-
// independent part of the collocation diagonal, sum over the elements not
// incident to the node and the regular rule's points of w_q / 4pi (-(n.d) / r^3)
// (the same terms the FP64 assembly kernel sums per row).  The double-float
// assembly reads it rather than evaluating it for every (row, frequency).
__global__ void __launch_bounds__(IBEM_THREADS) creg_kernel(int m, int n, int nq, const double *__restrict__ nodes,
                                                            const double *__restrict__ qdat,
                                                            const double *__restrict__ qnrm,
                                                            const int *__restrict__ evert,
                                                            const double *__restrict__ reg, double *__restrict__ creg)
{
    __shared__ double red[IBEM_THREADS / 32];
    const int row = blockIdx.x, tid = threadIdx.x;
    const double xo = nodes[row], yo = nodes[row + m], zo = nodes[row + 2 * (size_t)m];
    double ct = 0.0;
    for (int e = tid; e < n; e += IBEM_THREADS) {
        const int4 vv = reinterpret_cast<const int4 *>(evert)[e];
        if (vv.x == row || vv.y == row || vv.z == row) continue;
        const double nx = qnrm[e], ny = qnrm[e + n], nz = qnrm[e + 2 * (size_t)n];
        for (int q = 0; q < nq; ++q) {
            const double *p = qdat + (size_t)q * 9 * n + e;
            const double dx = p[0] - xo, dy = p[(size_t)n] - yo, dz = p[2 * (size_t)n] - zo;
            const double r2 = dx * dx + dy * dy + dz * dz;
            const double invr = rsqrt(r2);
            const double ft = (nx * dx + ny * dy + nz * dz) * (invr * invr);
            ct = fma(reg[q + 2 * nq] * IA_INV4PI * ft, -invr, ct);
        }
    }
    ct = warp_sum(ct);
    if ((tid & 31) == 0) red[tid >> 5] = ct;
    __syncthreads();
    if (tid == 0 && IA_IDX_OK(row, m)) {
        double tot = 0.0;
        for (int w = 0; w < IBEM_THREADS / 32; ++w) tot += red[w];
        creg[row] = tot;
    }
}

int mesh_creg(ia_context *ctx, ia_mesh *mesh)
{
    if (mesh->nq > IBEM_MAX_NQ) return IA_ERR_RULE;
    creg_kernel<<<mesh->m, IBEM_THREADS, 0, ctx->stream>>>(mesh->m, mesh->n, mesh->nq, mesh->d_nodes, mesh->d_qdat,
                                                         mesh->d_qnrm, mesh->d_evert, mesh->d_reg, mesh->d_creg);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// Geometry table of the double-float assembly: for every row (collocation or
// field point), regular-rule point q and element e, the frequency-independent
// r, 1/r and ft (point_geometry, the same arithmetic the rows kernel does
// inline), stored as (hi, lo) pairs at G[((row nq + q) 3 + c) n + e] so a
// warp's threads (consecutive elements) load each value coalesced.  The rows
// kernel then spends its issue slots on the per-frequency work only.  One
// thread per (row, element).
__global__ void __launch_bounds__(128) ibem_geom_kernel(int m, int n, int l, int n_ch, int nq, int nblk,
                                                        const double *__restrict__ nodes, const double *__restrict__ cp,
                                                        const double *__restrict__ mics, const dfl *__restrict__ qdat,
                                                        const dfl *__restrict__ qnrm, float2 *__restrict__ G)
{
    const int row = (int)(blockIdx.x / nblk);
    const int e = (int)(blockIdx.x % nblk) * 128 + (int)threadIdx.x;
    const int mt = m + n_ch;
    if (e >= n || row >= mt + l) return;
    double xo, yo, zo;
    if (row < m) {
        xo = nodes[row]; yo = nodes[row + m]; zo = nodes[row + 2 * m];
    } else if (row < mt) {
        const int i = row - m;
        xo = cp[i]; yo = cp[i + n_ch]; zo = cp[i + 2 * n_ch];
    } else {
        const int i = row - mt;
        xo = mics[i]; yo = mics[i + l]; zo = mics[i + 2 * l];
    }
    const dfl xr = df_from_double(xo), yr = df_from_double(yo), zr = df_from_double(zo);
    const dfl nx = qnrm[e], ny = qnrm[e + n], nz = qnrm[e + 2 * (size_t)n];
    [[maybe_unused]] const long long gext = (long long)(mt + l) * nq * 3 * n;
    for (int q = 0; q < nq; ++q) {
        dfl r, invr, ft;
        point_geometry(qdat + (size_t)q * 9 * n + e, n, nx, ny, nz, xr, yr, zr, r, invr, ft);
        const long long o = ((long long)row * nq + q) * 3 * n + e;
        if (!IA_IDX_OK(o + 2 * (long long)n, gext)) continue;
        G[o] = make_float2(r.hi, r.lo);
        G[o + n] = make_float2(invr.hi, invr.lo);
        G[o + 2 * (size_t)n] = make_float2(ft.hi, ft.lo);
    }
}

// Largest geometry table the double-float assembly uses (per call, in the
// caller's workspace); above it the rows kernel computes the geometry inline.
// IA_ASM_GEOM_TABLE=0 selects the inline form at every size.
constexpr size_t IBEM_GEOM_MAX_BYTES = size_t(1) << 30;

size_t ibem_geom_bytes(const ia_mesh *mesh, int rows)
{
    const char *e = getenv("IA_ASM_GEOM_TABLE");
    if (e && e[0] == '0') return 0;
    const size_t b = sizeof(float2) * 3 * (size_t)rows * mesh->nq * mesh->n;
    return b <= IBEM_GEOM_MAX_BYTES ? b : 0;
}

int ibem_rows(ia_context *ctx, const ia_mesh *mesh, int l, const double *mics, int n_ch, const double *cp, int F,
              const double *k, double c, double rho, double2 *At, double2 *Bt, double2 *Ahs_t, double2 *Bhs_t,
              bool df32, bool split_ab, float2 *gtab, bool build_gtab)
{
    if (mesh->nq > IBEM_MAX_NQ) return IA_ERR_RULE;
    const int m = mesh->m;
    const int rows = m + n_ch + l;
    const int FB = df32 ? AsmBlock<dfl>::FB : AsmBlock<double>::FB;
    // the table-reading kernel reads the sin/cos table through L1
    const size_t smem = sizeof(double2) * 2 * (size_t)m * FB + (df32 && !gtab ? DF_TRIG_TABLE * sizeof(float4) : 0);
    if (smem > 220 * 1024) return IA_ERR_TOO_LARGE;
    static const DfTrigCoef coef = df_trig_coefficients();
    static const DfTrigRed red = df_trig_reduction_constants();
    const int nfb = (F + FB - 1) / FB;
    dim3 g(rows, nfb);
    if (df32 && gtab) {
        // the geometry table (ibem_geom_bytes(mesh, rows) bytes), then the rows
        // kernel reading it, the frequency blocks of a row in consecutive CTAs
        const int nblk = (mesh->n + 127) / 128;
        if (build_gtab) {
            ibem_geom_kernel<<<(unsigned)rows * nblk, 128, 0, ctx->stream>>>(
                m, mesh->n, l, n_ch, mesh->nq, nblk, mesh->d_nodes, cp, mics, (const dfl *)mesh->d_qdat_f,
                (const dfl *)mesh->d_qnrm_f, gtab);
            IA_LAUNCH_CHECK(ctx);
        }
        IA_CUDA_TRY(cudaFuncSetAttribute(ibem_rows_kernel<dfl, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         220 * 1024));
        ibem_rows_kernel<dfl, true><<<(unsigned)rows * nfb, IBEM_THREADS, smem, ctx->stream>>>(
            m, mesh->n, l, n_ch, mesh->ncolors, F, mesh->d_nodes, mesh->d_egeo, (const dfl *)mesh->d_qdat_f,
            (const dfl *)mesh->d_qnrm_f, mesh->d_evert, mesh->d_color_ptr, mesh->d_adj_ptr, mesh->d_adj, mesh->nq,
            mesh->d_reg, mesh->d_sing, mesh->nqs, mics, cp, k, c, rho, coef, red, mesh->d_dftab, split_ab ? 1 : 0,
            mesh->d_creg, gtab, At, Bt, Ahs_t, Bhs_t);
    } else if (df32) {
        IA_CUDA_TRY(cudaFuncSetAttribute(ibem_rows_kernel<dfl, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         220 * 1024));
        ibem_rows_kernel<dfl, false><<<g, IBEM_THREADS, smem, ctx->stream>>>(
            m, mesh->n, l, n_ch, mesh->ncolors, F, mesh->d_nodes, mesh->d_egeo, (const dfl *)mesh->d_qdat_f,
            (const dfl *)mesh->d_qnrm_f, mesh->d_evert, mesh->d_color_ptr, mesh->d_adj_ptr, mesh->d_adj, mesh->nq,
            mesh->d_reg, mesh->d_sing, mesh->nqs, mics, cp, k, c, rho, coef, red, mesh->d_dftab, split_ab ? 1 : 0,
            mesh->d_creg, nullptr, At, Bt, Ahs_t, Bhs_t);
    } else {
        IA_CUDA_TRY(cudaFuncSetAttribute(ibem_rows_kernel<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         220 * 1024));
        ibem_rows_kernel<double, false><<<g, IBEM_THREADS, smem, ctx->stream>>>(
            m, mesh->n, l, n_ch, mesh->ncolors, F, mesh->d_nodes, mesh->d_egeo, mesh->d_qdat, mesh->d_qnrm,
            mesh->d_evert, mesh->d_color_ptr, mesh->d_adj_ptr, mesh->d_adj, mesh->nq, mesh->d_reg, mesh->d_sing,
            mesh->nqs, mics, cp, k, c, rho, coef, red, nullptr, 0, nullptr, nullptr, At, Bt, Ahs_t, Bhs_t);
    }
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

IA_BOUNDS_READER(bounds_read_asm)

}  // namespace ia
