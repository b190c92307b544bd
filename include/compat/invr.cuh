// Drop-in replacement for the reference's CUDA/invr.cuh: same names and
// signatures, outputs malloc'd by the callee, errors thrown as
// std::runtime_error.  Forwards to ia_invr (include/ia.h).
//   invr    <- CUDA/invr.cuh:457
//   invrgpu <- CUDA/invr.cuh:263  (r_msg, e_ng, r_lhg device pointers; cp host)
// Outputs: qe (m x n_am) the leading left singular vectors of G Z, he
// (l x n_am) = (A_hs Z - B_hs) qe, me (m x n_am) = Z qe, for any 1 <= n_am <= m
// (the reference's CPU invr() forms these only for n_am = m).  Singular
// vector phases are normalised (first component within 1e-6 of the largest
// magnitude real and positive), not zgesvd's.  Quadrature files as ibem.cuh.
#pragma once
#include "ibem.cuh"

extern "C" inline void invr(int m, int l, int n, double *r_ms, int *e_n, double *r_lh, cuDoubleComplex **m_e,
                            cuDoubleComplex **h, cuDoubleComplex **q_e, double k, int n_ch, double *cp, int n_am)
{
    std::vector<double> reg, sing;
    ia_rules rules;
    const ia_rules *rp = ia_compat_rules(reg, sing, rules, "invr");
    ia_config cfg = ia_compat_config();
    ia_compat_check(ia_invr(m, l, n, r_ms, e_n, r_lh, (ia_complex **)m_e, (ia_complex **)h, (ia_complex **)q_e, k,
                            n_ch, cp, n_am, rp, &cfg),
                    "invr");
}

inline void invrgpu(int m, int l, int n, double *r_msg, int *e_ng, double *r_lhg, cuDoubleComplex **me,
                    cuDoubleComplex **he, cuDoubleComplex **qe, double k, int n_ch, double *cp, int n_rm)
{
    double *r_ms = ia_compat_to_host(r_msg, 3 * (size_t)m);
    int *e_n = ia_compat_to_host(e_ng, 3 * (size_t)n);
    double *r_lh = ia_compat_to_host(r_lhg, 3 * (size_t)l);
    try {
        invr(m, l, n, r_ms, e_n, r_lh, me, he, qe, k, n_ch, cp, n_rm);
    } catch (...) {
        std::free(r_ms);
        std::free(e_n);
        std::free(r_lh);
        throw;
    }
    std::free(r_ms);
    std::free(e_n);
    std::free(r_lh);
}
