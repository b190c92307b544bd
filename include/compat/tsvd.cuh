// Drop-in replacement for the reference's CUDA/tsvd.cuh: same names and
// signatures, outputs malloc'd by the callee, errors thrown as
// std::runtime_error.  Forwards to ia_csvd / ia_tsvd (include/ia.h).
//   csvd <- CUDA/tsvd.cuh:10   (u m x p, s p, v n x p, p = min(m, n))
//   tsvd <- CUDA/tsvd.cuh:122  (k outside [1, p] throws; the reference printed
//                               and left *x unset, CUDA/tsvd.cuh:124-126)
#pragma once
#include "ia_compat_common.cuh"

inline void csvd(int m, int n, cuDoubleComplex *a, cuDoubleComplex **u, double **s, cuDoubleComplex **v)
{
    ia_compat_check(ia_csvd(m, n, (const ia_complex *)a, (ia_complex **)u, s, (ia_complex **)v), "csvd");
}

inline void tsvd(int m, int n, int p, int k, cuDoubleComplex *u, double *s, cuDoubleComplex *v, cuDoubleComplex *b,
                 cuDoubleComplex **x)
{
    ia_compat_check(ia_tsvd(m, n, p, k, (const ia_complex *)u, s, (const ia_complex *)v, (const ia_complex *)b,
                            (ia_complex **)x),
                    "tsvd");
}
