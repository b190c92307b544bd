// Transfer-matrix assembly kernels (FP64), batched over wavenumbers.
//
//  * monopole_kernel   plain ESM matrix G = exp(ikr)/(4 pi r)      (esmV.m:29-30)
//  * esm_system_kernel D^T, M_sq^T, M_hq^T of the reference esm()  (esm.cuh:1-36, :120-145)
//  * hels_kernel       h_n(kr) Y_n^m and its radial derivative       (hels.cuh:86-183, :222-323)
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

// --------------------------------------------------------------------------
// ESM
// --------------------------------------------------------------------------
// G_f(i, j), i = microphone (row), j = source (col).  Thread per (i, j);
// frequencies on grid.y.  Stores are coalesced along i.
__global__ void monopole_kernel(int l, int m, const double *__restrict__ mics, const double *__restrict__ src,
                                const double *__restrict__ kv, double2 *__restrict__ G)
{
    const int f = blockIdx.y;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)l * m) return;
    const int i = (int)(e % l), j = (int)(e / l);
    double dx = mics[i] - src[j], dy = mics[i + l] - src[j + m], dz = mics[i + 2 * l] - src[j + 2 * m];
    double r2 = dx * dx + dy * dy + dz * dz;
    double invr = rsqrt(r2);
    double r = r2 * invr;
    double2 g = green(kv[f] * r, invr * IA_INV4PI);
    G[(size_t)f * l * m + e] = g;
}

int monopole_batched(ia_context *ctx, int l, int m, int F, const double *mics, const double *src, const double *k,
                     double2 *G)
{
    long long total = (long long)l * m;
    dim3 g((unsigned)((total + 255) / 256), F);
    monopole_kernel<<<g, 256, 0, ctx->stream>>>(l, m, mics, src, k, G);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// Reference layout (CUDA/esm.cuh:130-142): DT[j + i*m] = D(surface i, source j),
// RHS = [M_sq^T | M_hq^T] (m x (m + l)), sources at r_i * r_ms.
__global__ void esm_system_kernel(int m, int l, const double *__restrict__ r_ms, const double *__restrict__ r_lh,
                                  double r_i, double k, double c, double rho, double2 *__restrict__ DT,
                                  double2 *__restrict__ RHS)
{
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long total = (long long)m * (m + l);
    if (e >= total) return;
    const int j = (int)(e % m);          // source
    const int col = (int)(e / m);        // surface point (col < m) or field point (col - m)
    const double qx = r_ms[j] * r_i, qy = r_ms[j + m] * r_i, qz = r_ms[j + 2 * m] * r_i;
    const double irck = rho * c * k;
    if (col < m) {
        const int i = col;
        double sx = r_ms[i], sy = r_ms[i + m], sz = r_ms[i + 2 * m];
        double dx = sx - qx, dy = sy - qy, dz = sz - qz;
        double R = sqrt(dx * dx + dy * dy + dz * dz);
        double cos_t = (sx * dx + sy * dy + sz * dz) / (sqrt(sx * sx + sy * sy + sz * sz) * R);
        double sn, cs;
        sincos(k * R, &sn, &cs);
        // D = ((ikR - 1)/(4 pi R^2)) e^{ikR} cos_t
        double2 ek = make_double2(cs, sn);
        double2 pre = make_double2(-1.0 / (4.0 * M_PI * R * R), k * R / (4.0 * M_PI * R * R));
        DT[j + (size_t)i * m] = zscale(zmul(pre, ek), cos_t);
        // M_sq = i rho k c e^{ikR}/(4 pi R)
        double2 g = zscale(ek, 1.0 / (4.0 * M_PI * R));
        RHS[j + (size_t)i * m] = make_double2(-irck * g.y, irck * g.x);
    } else {
        const int i = col - m;
        double dx = r_lh[i] - qx, dy = r_lh[i + l] - qy, dz = r_lh[i + 2 * l] - qz;
        double R = sqrt(dx * dx + dy * dy + dz * dz);
        double sn, cs;
        sincos(k * R, &sn, &cs);
        double2 g = make_double2(cs / (4.0 * M_PI * R), sn / (4.0 * M_PI * R));
        RHS[j + (size_t)(m + i) * m] = make_double2(-irck * g.y, irck * g.x);
    }
}

int esm_system(ia_context *ctx, int m, int l, const double *src, const double *mics, double r_i, double k, double c,
               double rho, double2 *DT, double2 *RHS)
{
    long long total = (long long)m * (m + l);
    esm_system_kernel<<<(unsigned)((total + 255) / 256), 256, 0, ctx->stream>>>(m, l, src, mics, r_i, k, c, rho, DT,
                                                                               RHS);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// --------------------------------------------------------------------------
// HELS.  One thread per (point, frequency) produces all (N+1)^2 columns:
//   j_n by Miller's downward recurrence normalised to j_0 = sin x / x (upward
//   when x > N, where it is stable), y_n by upward recurrence; h_n = j_n + i y_n
//   (hels.cuh:248-253), k h_n' = k (n h_n / x - h_{n+1}) (hels.cuh:250-251);
//   normalised associated Legendre functions with the Condon-Shortley phase by
//   the standard three-term recurrences, Y_n^{-m} = (-1)^m conj(Y_n^m)
//   (hels.cuh:128).  Column i = n^2 + n + m (hels.cuh:235).
// --------------------------------------------------------------------------
constexpr int HELS_MAX_ORDER = 40;

__device__ void sph_bessel(int N1, double x, double *jn, double *yn)
{
    // N1 = highest order needed (inclusive)
    double sx, cx;
    sincos(x, &sx, &cx);
    const double invx = 1.0 / x;
    yn[0] = -cx * invx;
    if (N1 >= 1) yn[1] = (-cx * invx - sx) * invx;
    for (int n = 2; n <= N1; ++n) yn[n] = (2 * n - 1) * invx * yn[n - 1] - yn[n - 2];
    const double j0 = sx * invx;
    if (x > (double)N1) {
        jn[0] = j0;
        if (N1 >= 1) jn[1] = (sx * invx - cx) * invx;
        for (int n = 2; n <= N1; ++n) jn[n] = (2 * n - 1) * invx * jn[n - 1] - jn[n - 2];
        return;
    }
    // Miller: start well above max(N1, x)
    int start = N1 + 16 + (int)(sqrt(40.0 * (N1 + 1)));
    double jp1 = 0.0, jc = 1e-300;
    for (int n = start; n > N1; --n) {
        double jm1 = (2 * n + 1) * invx * jc - jp1;
        jp1 = jc;
        jc = jm1;
        if (fabs(jc) > 1e250) { jc *= 1e-250; jp1 *= 1e-250; }
    }
    // jc = j_{N1} (unnormalised), jp1 = j_{N1+1}
    jn[N1] = jc;
    double nxt = jp1;
    for (int n = N1; n > 0; --n) {
        double jm1 = (2 * n + 1) * invx * jn[n] - nxt;
        nxt = jn[n];
        jn[n - 1] = jm1;
        if (fabs(jm1) > 1e250) {
            for (int t = n - 1; t <= N1; ++t) jn[t] *= 1e-250;
            nxt *= 1e-250;
        }
    }
    // normalise with whichever of the exact j_0, j_1 is larger (never both near a zero)
    const double j1 = (sx * invx - cx) * invx;
    const double scale = (fabs(j0) >= fabs(j1) || N1 < 1) ? j0 / jn[0] : j1 / jn[1];
    for (int n = 0; n <= N1; ++n) jn[n] *= scale;
}

__global__ void hels_kernel(int npts, const double *__restrict__ pts, int order, const double *__restrict__ kv,
                            double c, double rho, double2 *__restrict__ Me, double2 *__restrict__ Qe)
{
    const int f = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= npts) return;
    const int nt = (order + 1) * (order + 1);
    const double k = kv[f];
    const double az = pts[j], el = pts[j + npts], r = pts[j + 2 * npts];
    const double x = k * r;
    double jn[HELS_MAX_ORDER + 2], yn[HELS_MAX_ORDER + 2];
    sph_bessel(order + 1, x, jn, yn);
    const double ct = cos(el);
    const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    double2 *me = Me + (size_t)f * npts * nt;
    double2 *qe = Qe ? Qe + (size_t)f * npts * nt : nullptr;
    const double inv_irck_re = 0.0;            // 1/(i rho c k) = -i/(rho c k)
    const double inv_irck_im = -1.0 / (rho * c * k);
    (void)inv_irck_re;
    // P̄_m^m seeds
    double pmm = 0.28209479177387814;          // 1/sqrt(4 pi)
    for (int mm = 0; mm <= order; ++mm) {
        if (mm > 0) pmm *= -sqrt((2.0 * mm + 1.0) / (2.0 * mm)) * st;
        double sm_, cm_;
        sincos(mm * az, &sm_, &cm_);
        double p_nm2 = 0.0, p_nm1 = pmm;
        for (int nn = mm; nn <= order; ++nn) {
            double p;
            if (nn == mm) p = pmm;
            else if (nn == mm + 1) p = sqrt(2.0 * mm + 3.0) * ct * pmm;
            else {
                double a_n = sqrt((4.0 * nn * nn - 1.0) / ((double)nn * nn - (double)mm * mm));
                double a_n1 = sqrt((4.0 * (nn - 1.0) * (nn - 1.0) - 1.0) / ((nn - 1.0) * (nn - 1.0) - (double)mm * mm));
                p = a_n * (ct * p_nm1 - p_nm2 / a_n1);
            }
            if (nn > mm) { p_nm2 = p_nm1; p_nm1 = p; }
            else { p_nm2 = 0.0; p_nm1 = p; }
            const double2 Y = make_double2(p * cm_, p * sm_);
            const double2 h = make_double2(jn[nn], yn[nn]);
            const double2 h1 = make_double2(jn[nn + 1], yn[nn + 1]);
            const double2 dh = zscale(zsub(zscale(h, nn / x), h1), k);
            const int ip = nn * nn + nn + mm;
            me[j + (size_t)ip * npts] = zmul(h, Y);
            double2 qv = zmul(zmul(make_double2(0.0, inv_irck_im), dh), Y);
            if (qe) qe[j + (size_t)ip * npts] = qv;
            if (mm > 0) {
                const double sg = (mm & 1) ? -1.0 : 1.0;
                const double2 Yn = make_double2(sg * Y.x, -sg * Y.y);
                const int in_ = nn * nn + nn - mm;
                me[j + (size_t)in_ * npts] = zmul(h, Yn);
                if (qe) qe[j + (size_t)in_ * npts] = zmul(zmul(make_double2(0.0, inv_irck_im), dh), Yn);
            }
        }
    }
}

int hels_batched(ia_context *ctx, int npts, const double *pts, int order, int F, const double *k, double c,
                 double rho, double2 *Me, double2 *Qe)
{
    if (order < 0 || order > HELS_MAX_ORDER) return IA_ERR_TOO_LARGE;
    dim3 g((npts + 127) / 128, F);
    hels_kernel<<<g, 128, 0, ctx->stream>>>(npts, pts, order, k, c, rho, Me, Qe);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

}  // namespace ia
