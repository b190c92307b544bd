// Drop-in replacement for the reference's CUDA/esm.cuh: same names and
// signatures, outputs malloc'd by the callee, errors thrown as
// std::runtime_error.  Forwards to ia_esm (include/ia.h).
//   esm    <- CUDA/esm.cuh:112   (correct also for l != m)
//   esmgpu <- CUDA/esm.cuh:38    (r_msg, r_lhg are device pointers)
#pragma once
#include "ia_compat_common.cuh"

extern "C" inline void esm(int m, int l, double *r_ms, double *r_lh, cuDoubleComplex **m_e, cuDoubleComplex **h,
                           double k, double r_i)
{
    ia_config cfg = ia_compat_config();
    ia_compat_check(ia_esm(m, l, r_ms, r_lh, (ia_complex **)m_e, (ia_complex **)h, k, r_i, &cfg), "esm");
}

inline void esmgpu(int m, int l, double *r_msg, double *r_lhg, cuDoubleComplex **me, cuDoubleComplex **he, double k,
                   double r_i)
{
    double *r_ms = ia_compat_to_host(r_msg, 3 * (size_t)m);
    double *r_lh = ia_compat_to_host(r_lhg, 3 * (size_t)l);
    ia_config cfg = ia_compat_config();
    int st = ia_esm(m, l, r_ms, r_lh, (ia_complex **)me, (ia_complex **)he, k, r_i, &cfg);
    std::free(r_ms);
    std::free(r_lh);
    ia_compat_check(st, "esmgpu");
}
