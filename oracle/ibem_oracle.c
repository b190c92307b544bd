/* CPU restatement of the reference's IBEM collocation assembly.
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY: called by tests/, by __graft_entry__.smoke()
 * as the checker, and by bench.py's CPU-baseline leg.  The product path never
 * links or loads it.
 *
 * Follows the reference's CPU ibem() (CUDA/ibem.cuh:424-770), which is the
 * OpenBEM collocation scheme on linear triangles:
 *   element normal   n = (v0 - v2) x (v1 - v2), |n| = 2*area     (:502-511)
 *   quadrature point x_q = xi1 v0 + xi2 v1 + (1-xi1-xi2) v2     (:496-501)
 *   shape functions  N = (xi1, xi2, 1-xi1-xi2)
 *   g  = exp(ikr)/r,  ft = n.(x_q - x_o)/r^2                   (:512-517)
 *   B[o, v] += w N_v |n| g / 4pi                                (:514-516)
 *   A[o, v] += w N_v ft (ikr - 1) g / 4pi                       (:518-520)
 *   C[o]    += w (-ft/r) / 4pi   (all elements)                 (:527, :581)
 *   rows where o is a vertex of the element use that vertex's page of the
 *   singular rule (:490-541), the others the regular rule (:544-596)
 *   A[o,o]  -= 1 + C[o]                                          (:611-614)
 *   field rows and CHIEF rows: regular rule, no C term          (:623-735)
 *   B and B_hs are scaled by i rho c k                           (:743-746)
 * Outputs are column-major: A, B are (m+n_ch) x m, Ahs, Bhs are l x m.
 * Summation order is element-major like the reference, so results agree with
 * it to rounding.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double re, im; } zc;

static const double INV4PI = 0.079577471545947667884; /* 1/(4 pi) */

struct elem_geom { double v[3][3]; double nx, ny, nz, an; };

static void element(const double *r, int m, const int *e, int n, int i, struct elem_geom *g)
{
    for (int s = 0; s < 3; ++s) {
        int node = e[i + s * n];
        g->v[s][0] = r[node];
        g->v[s][1] = r[node + m];
        g->v[s][2] = r[node + 2 * m];
    }
    double a0 = g->v[0][0] - g->v[2][0], a1 = g->v[0][1] - g->v[2][1], a2 = g->v[0][2] - g->v[2][2];
    double b0 = g->v[1][0] - g->v[2][0], b1 = g->v[1][1] - g->v[2][1], b2 = g->v[1][2] - g->v[2][2];
    g->nx = a1 * b2 - a2 * b1;
    g->ny = a2 * b0 - a0 * b2;
    g->nz = a0 * b1 - a1 * b0;
    g->an = sqrt(g->nx * g->nx + g->ny * g->ny + g->nz * g->nz);
}

/* Integrate one element against one collocation point with a rule of nq
 * points stored SoA (xi1[nq], xi2[nq], w[nq]).  acc[0..2] get the A terms,
 * acc[3..5] the (unscaled) B terms, *ct the C term. */
static void integrate(const struct elem_geom *g, const double *x, double k, const double *rule, int nq,
                      zc acc[6], double *ct)
{
    for (int q = 0; q < nq; ++q) {
        double x1 = rule[q], x2 = rule[q + nq], w = rule[q + 2 * nq];
        double x3 = 1.0 - x1 - x2;
        double dx = x1 * g->v[0][0] + x2 * g->v[1][0] + x3 * g->v[2][0] - x[0];
        double dy = x1 * g->v[0][1] + x2 * g->v[1][1] + x3 * g->v[2][1] - x[1];
        double dz = x1 * g->v[0][2] + x2 * g->v[1][2] + x3 * g->v[2][2] - x[2];
        double r2 = dx * dx + dy * dy + dz * dz;
        double r = sqrt(r2);
        double kr = k * r;
        double gr = cos(kr) / r, gi = sin(kr) / r;
        double ft = (g->nx * dx + g->ny * dy + g->nz * dz) / r2;
        /* (ikr - 1) g */
        double tr = -gr - kr * gi, ti = kr * gr - gi;
        double N[3] = {x1, x2, x3};
        for (int v = 0; v < 3; ++v) {
            double sa = w * INV4PI * ft * N[v];
            double sb = w * INV4PI * g->an * N[v];
            acc[v].re += sa * tr;
            acc[v].im += sa * ti;
            acc[3 + v].re += sb * gr;
            acc[3 + v].im += sb * gi;
        }
        *ct += w * INV4PI * (-ft / r);
    }
}

/* Rows of an "outside point" block (field or CHIEF points): out_a/out_b are
 * ld x m column-major, rows row0..row0+np-1. */
static void point_rows(const double *r, int m, const int *e, int n, const double *pts, int np, double k,
                       const double *reg, int nq, zc *out_a, zc *out_b, int ld, int row0)
{
    struct elem_geom g;
    for (int i = 0; i < n; ++i) {
        element(r, m, e, n, i, &g);
        for (int p = 0; p < np; ++p) {
            double x[3] = {pts[p], pts[p + np], pts[p + 2 * np]};
            zc acc[6];
            double ct = 0.0;
            memset(acc, 0, sizeof(acc));
            integrate(&g, x, k, reg, nq, acc, &ct);
            for (int v = 0; v < 3; ++v) {
                int col = e[i + v * n];
                out_a[row0 + p + (size_t)col * ld].re += acc[v].re;
                out_a[row0 + p + (size_t)col * ld].im += acc[v].im;
                out_b[row0 + p + (size_t)col * ld].re += acc[3 + v].re;
                out_b[row0 + p + (size_t)col * ld].im += acc[3 + v].im;
            }
        }
    }
}

/* reg: regular rule SoA (3*nq); sing: singular rule, 3 pages of SoA (3*nqs
 * each).  A, B: (m+n_ch) x m; Ahs, Bhs: l x m; all zeroed here. */
void ora_ibem_assemble(int m, int l, int n, const double *r_ms, const int *e_n, const double *r_lh, double k,
                       int nq, const double *reg, int nqs, const double *sing, int n_ch, const double *cp,
                       double c, double rho, zc *A, zc *B, zc *Ahs, zc *Bhs)
{
    int mt = m + n_ch;
    memset(A, 0, sizeof(zc) * (size_t)mt * m);
    memset(B, 0, sizeof(zc) * (size_t)mt * m);
    memset(Ahs, 0, sizeof(zc) * (size_t)l * m);
    memset(Bhs, 0, sizeof(zc) * (size_t)l * m);
    double *cterm = (double *)calloc((size_t)m, sizeof(double));
    struct elem_geom g;
    for (int i = 0; i < n; ++i) {
        element(r_ms, m, e_n, n, i, &g);
        int vn[3] = {e_n[i], e_n[i + n], e_n[i + 2 * n]};
        for (int o = 0; o < m; ++o) {
            int slot = -1;
            for (int s = 0; s < 3; ++s)
                if (vn[s] == o) slot = s;
            double x[3] = {r_ms[o], r_ms[o + m], r_ms[o + 2 * m]};
            zc acc[6];
            double ct = 0.0;
            memset(acc, 0, sizeof(acc));
            if (slot >= 0)
                integrate(&g, x, k, sing + (size_t)3 * nqs * slot, nqs, acc, &ct);
            else
                integrate(&g, x, k, reg, nq, acc, &ct);
            for (int v = 0; v < 3; ++v) {
                A[o + (size_t)vn[v] * mt].re += acc[v].re;
                A[o + (size_t)vn[v] * mt].im += acc[v].im;
                B[o + (size_t)vn[v] * mt].re += acc[3 + v].re;
                B[o + (size_t)vn[v] * mt].im += acc[3 + v].im;
            }
            cterm[o] += ct;
        }
    }
    for (int o = 0; o < m; ++o) A[o + (size_t)o * mt].re -= 1.0 + cterm[o];
    free(cterm);
    point_rows(r_ms, m, e_n, n, r_lh, l, k, reg, nq, Ahs, Bhs, l, 0);
    if (n_ch > 0) point_rows(r_ms, m, e_n, n, cp, n_ch, k, reg, nq, A, B, mt, m);
    /* scale B by i rho c k */
    double s = rho * c * k;
    for (size_t t = 0; t < (size_t)mt * m; ++t) {
        double re = B[t].re;
        B[t].re = -s * B[t].im;
        B[t].im = s * re;
    }
    for (size_t t = 0; t < (size_t)l * m; ++t) {
        double re = Bhs[t].re;
        Bhs[t].re = -s * Bhs[t].im;
        Bhs[t].im = s * re;
    }
}

/* sinc resistance matrix, R_ij = w^2 rho A^2/(4 pi c) sinc(k r_ij), real
 * symmetric, column-major n x n. */
void ora_sinc_resistance(int n, const double *x, double k, double c, double rho, double area, double *R)
{
    double omega = k * c;
    double s = omega * omega * rho * area * area * INV4PI / c;
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            double dx = x[i] - x[j], dy = x[i + n] - x[j + n], dz = x[i + 2 * n] - x[j + 2 * n];
            double kr = k * sqrt(dx * dx + dy * dy + dz * dz);
            R[i + (size_t)j * n] = s * (kr == 0.0 ? 1.0 : sin(kr) / kr);
        }
}
