// Drop-in replacement for the reference's CUDA/hels.cuh: same names and
// signatures, outputs malloc'd by the callee, errors thrown as
// std::runtime_error.  Forwards to ia_hels (include/ia.h).
//   hels    <- CUDA/hels.cuh:222
//   helsgpu <- CUDA/hels.cuh:185  (r_ms_sg, r_lh_sg device pointers)
// Points are (azimuth, elevation, radius) structure-of-arrays, as produced by
// cartesian_2_spherical (include/compat/utils.cuh).
#pragma once
#include "ia_compat_common.cuh"

extern "C" inline void hels(int m, int l, double *r_ms_s, double *r_lh_s, cuDoubleComplex **m_e,
                            cuDoubleComplex **h, cuDoubleComplex **q_e, double k, int n_sh)
{
    ia_config cfg = ia_compat_config();
    ia_compat_check(ia_hels(m, l, r_ms_s, r_lh_s, (ia_complex **)m_e, (ia_complex **)h, (ia_complex **)q_e, k, n_sh,
                            &cfg),
                    "hels");
}

inline void helsgpu(int m, int l, double *r_ms_sg, double *r_lh_sg, cuDoubleComplex **me, cuDoubleComplex **he,
                    cuDoubleComplex **qe, double k, int n_sh)
{
    double *a = ia_compat_to_host(r_ms_sg, 3 * (size_t)m);
    double *b = ia_compat_to_host(r_lh_sg, 3 * (size_t)l);
    ia_config cfg = ia_compat_config();
    int st = ia_hels(m, l, a, b, (ia_complex **)me, (ia_complex **)he, (ia_complex **)qe, k, n_sh, &cfg);
    std::free(a);
    std::free(b);
    ia_compat_check(st, "helsgpu");
}
