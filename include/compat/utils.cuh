// Drop-in replacement for the parts of the reference's CUDA/utils.cuh that
// belong to the inverse path: same names and signatures, outputs malloc'd by
// the callee.
//   to_pressure  <- CUDA/utils.cuh:199   (ia_to_pressure, on the GPU)
//   to_velocity  <- CUDA/utils.cuh:232   (ia_to_velocity, on the GPU)
//   sound_power  <- CUDA/utils.cuh:265   (ia_sound_power, on the GPU)
//   sphere       <- CUDA/utils.cuh:384   analytic pulsating sphere (input
//                   preparation, host): p = (a/r) rho c u (ika/(ika-1)) e^{ik(r-a)}
//   cartesian_2_spherical <- CUDA/utils.cuh:414  (az, el, r), same branch rules
//   geometry     <- CUDA/utils.cuh:291   gmsh v2.2 reader (ia_read_msh, host)
// The reference's debug printers/writers are not part of it.
#pragma once
#include <cmath>
#include "ia_compat_common.cuh"

inline void to_pressure(int m, int n, cuDoubleComplex *me, cuDoubleComplex *x, cuDoubleComplex **p)
{
    ia_compat_check(ia_to_pressure(m, n, (const ia_complex *)me, (const ia_complex *)x, (ia_complex **)p),
                    "to_pressure");
}

inline void to_velocity(int m, int n, cuDoubleComplex *qe, cuDoubleComplex *x, cuDoubleComplex **v)
{
    ia_compat_check(ia_to_velocity(m, n, (const ia_complex *)qe, (const ia_complex *)x, (ia_complex **)v),
                    "to_velocity");
}

inline void sound_power(int m, cuDoubleComplex *p, cuDoubleComplex *v, double *w, double s)
{
    ia_compat_check(ia_sound_power(m, (const ia_complex *)p, (const ia_complex *)v, w, s), "sound_power");
}

inline void sphere(double *r_ms, double *r_lh, cuDoubleComplex **p_s, cuDoubleComplex **p_h, cuDoubleComplex **v_s,
                   double k, double u, double a, int m, int l)
{
    const double c = C_AIR, rho = RHO_AIR;
    // ika / (ika - 1) = (ika)(-1 - ika) / (1 + (ka)^2)
    const double ka = k * a, den = 1.0 + ka * ka;
    const double fr = ka * ka / den, fi = -ka / den;
    auto field = [&](const double *P, int cnt, cuDoubleComplex *out) {
        for (int i = 0; i < cnt; ++i) {
            double r = std::sqrt(P[i] * P[i] + P[i + cnt] * P[i + cnt] + P[i + 2 * cnt] * P[i + 2 * cnt]);
            double amp = (a / r) * rho * c * u;
            double cs = std::cos(k * (r - a)), sn = std::sin(k * (r - a));
            out[i] = make_cuDoubleComplex(amp * (fr * cs - fi * sn), amp * (fr * sn + fi * cs));
        }
    };
    *p_s = (cuDoubleComplex *)std::malloc(sizeof(cuDoubleComplex) * (size_t)m);
    *v_s = (cuDoubleComplex *)std::malloc(sizeof(cuDoubleComplex) * (size_t)m);
    *p_h = (cuDoubleComplex *)std::malloc(sizeof(cuDoubleComplex) * (size_t)l);
    if (!*p_s || !*v_s || !*p_h) throw std::runtime_error("malloc");
    field(r_ms, m, *p_s);
    field(r_lh, l, *p_h);
    for (int i = 0; i < m; ++i) (*v_s)[i] = make_cuDoubleComplex(u, 0.0);
}

inline void cartesian_2_spherical(int m, double *r_xx, double **azelr)
{
    *azelr = (double *)std::malloc(sizeof(double) * 3 * (size_t)m);
    if (!*azelr) throw std::runtime_error("malloc");
    for (int i = 0; i < m; ++i) {
        double x = r_xx[i], y = r_xx[i + m], z = r_xx[i + 2 * m];
        double xy = x * x + y * y;
        (*azelr)[i + 2 * m] = std::sqrt(xy + z * z);
        (*azelr)[i] = std::atan2(y, x) + (y < 0 ? 2.0 * M_PI : 0.0);
        (*azelr)[i + m] = std::atan2(std::sqrt(xy), z) - (x < 0 ? 2.0 * M_PI : 0.0);
    }
}

// geometry <- CUDA/utils.cuh:291  gmsh v2.2 reader (ia_read_msh, host); throws
// where the reference calls exit()
inline void geometry(double **r_ms, double **r_lh, int **e_n, double k, double t, int *m_out, int *l_out, int *n_out,
                     char *file)
{
    ia_compat_check(ia_read_msh(file, k, t, r_ms, r_lh, e_n, m_out, l_out, n_out), "geometry");
}
