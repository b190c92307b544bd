// Drop-in replacement for the reference's CUDA/ibem.cuh: same names and
// signatures, outputs malloc'd by the callee, errors thrown as
// std::runtime_error.  Forwards to ia_ibem (include/ia.h).
//   ibem    <- CUDA/ibem.cuh:424
//   ibemgpu <- CUDA/ibem.cuh:263  (r_msg, e_ng, r_lhg device pointers; cp host)
// Quadrature: like the reference, IPF.txt (regular rule) and IPFs.txt
// (singular rule, one $PAGE per vertex) are read from the current directory
// (format of CUDA/ibem.cuh:265-312); when both are absent, ia_ibem's built-in
// rules are used instead of exiting; when either is present but does not
// parse (a missing partner file, a truncated table, a bad count), the call
// throws instead of using rules the caller did not ask for.
#pragma once
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>
#include "ia_compat_common.cuh"

// Returns true and fills reg (3*nq) / sing (9*nqs) when both files parse.
inline bool ia_compat_read_ipf(std::vector<double> &reg, int &nq, std::vector<double> &sing, int &nqs)
{
    FILE *fp = std::fopen("IPF.txt", "r");
    if (!fp) return false;
    char line[MAX_LINE];
    if (!std::fgets(line, MAX_LINE, fp)) { std::fclose(fp); return false; }
    nq = std::atoi(line);
    if (nq < 1) { std::fclose(fp); return false; }
    reg.assign(3 * (size_t)nq, 0.0);
    int i = 0;
    while (i < nq && std::fgets(line, MAX_LINE, fp)) {
        char *p;
        reg[i] = std::strtod(line, &p);
        reg[i + nq] = std::strtod(p, &p);
        reg[i + 2 * nq] = std::strtod(p, nullptr);
        ++i;
    }
    std::fclose(fp);
    if (i != nq) return false;
    fp = std::fopen("IPFs.txt", "r");
    if (!fp) return false;
    if (!std::fgets(line, MAX_LINE, fp)) { std::fclose(fp); return false; }
    nqs = std::atoi(line);
    if (nqs < 1) { std::fclose(fp); return false; }
    sing.assign(9 * (size_t)nqs, 0.0);
    int page = -1;
    i = 0;
    int count = 0;
    while (std::fgets(line, MAX_LINE, fp)) {
        if (std::strncmp(line, "$PAGE", 5) == 0) {
            page = std::atoi(line + 5) - 1;
            i = 0;
            continue;
        }
        if (page < 0 || page > 2 || i >= nqs) continue;
        char *p;
        double *P = sing.data() + (size_t)3 * nqs * page;
        P[i] = std::strtod(line, &p);
        P[i + nqs] = std::strtod(p, &p);
        P[i + 2 * nqs] = std::strtod(p, nullptr);
        ++i;
        ++count;
    }
    std::fclose(fp);
    return count == 3 * nqs;
}

// The quadrature rules for a call: null when neither file exists (built-in
// rules), the parsed tables otherwise; throws when a file exists but the pair
// does not parse.
inline const ia_rules *ia_compat_rules(std::vector<double> &reg, std::vector<double> &sing, ia_rules &rules,
                                       const char *who)
{
    FILE *a = std::fopen("IPF.txt", "r"), *b = std::fopen("IPFs.txt", "r");
    const bool any = a || b;
    if (a) std::fclose(a);
    if (b) std::fclose(b);
    if (!any) return nullptr;
    int nq = 0, nqs = 0;
    if (!ia_compat_read_ipf(reg, nq, sing, nqs))
        throw std::runtime_error(std::string(who) + ": IPF.txt / IPFs.txt present but malformed");
    rules.nq = nq;
    rules.regular = reg.data();
    rules.nqs = nqs;
    rules.singular = sing.data();
    return &rules;
}

extern "C" inline void ibem(int m, int l, int n, double *r_ms, int *e_n, double *r_lh, cuDoubleComplex **m_e,
                            cuDoubleComplex **h, double k, int n_ch, double *cp)
{
    std::vector<double> reg, sing;
    ia_rules rules;
    const ia_rules *rp = ia_compat_rules(reg, sing, rules, "ibem");
    ia_config cfg = ia_compat_config();
    ia_compat_check(ia_ibem(m, l, n, r_ms, e_n, r_lh, (ia_complex **)m_e, (ia_complex **)h, k, n_ch, cp, rp, &cfg),
                    "ibem");
}

inline void ibemgpu(int m, int l, int n, double *r_msg, int *e_ng, double *r_lhg, cuDoubleComplex **me,
                    cuDoubleComplex **he, double k, int n_ch, double *cp)
{
    double *r_ms = ia_compat_to_host(r_msg, 3 * (size_t)m);
    int *e_n = ia_compat_to_host(e_ng, 3 * (size_t)n);
    double *r_lh = ia_compat_to_host(r_lhg, 3 * (size_t)l);
    try {
        ibem(m, l, n, r_ms, e_n, r_lh, me, he, k, n_ch, cp);
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
