// gmsh v2.2 ASCII mesh reader (host code).
//
// Same result as the reference's geometry() (CUDA/utils.cuh:291-382) on the
// files it reads: the $Nodes block gives the nodes (structure of arrays),
// element type 2 (3-node triangle) with three distinct vertices gives the
// triangles (0-based, file order; degenerate ones are dropped as in
// utils.cuh:339-349), and the field points are the nodes scaled by
// 1 + (2 pi / k) t (utils.cuh:368-376).  Differences: a missing or
// malformed file returns IA_ERR_ARG instead of exit(); the number of tags of
// each element line is read from the line (the reference skips exactly two);
// CR-LF line ends are accepted.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <string>
#include <vector>
#include "ia_internal.h"

namespace {

bool next_line(FILE *fp, std::string &s)
{
    s.clear();
    char buf[4096];
    while (fgets(buf, sizeof buf, fp)) {
        s += buf;
        if (!s.empty() && s.back() == '\n') break;
    }
    if (s.empty()) return false;
    while (!s.empty() && (s.back() == '\n' || s.back() == '\r')) s.pop_back();
    return true;
}

bool seek_section(FILE *fp, const char *name)
{
    std::string s;
    while (next_line(fp, s))
        if (s == name) return true;
    return false;
}

}  // namespace

extern "C" int ia_read_msh(const char *file, double k, double t, double **r_ms, double **r_lh, int **e_n, int *m_out,
                           int *l_out, int *n_out)
{
    if (!file || !r_ms || !r_lh || !e_n || !m_out || !l_out || !n_out || !(k > 0.0)) return IA_ERR_ARG;
    *r_ms = nullptr;
    *r_lh = nullptr;
    *e_n = nullptr;
    FILE *fp = fopen(file, "r");
    if (!fp) return IA_ERR_ARG;
    std::string s;
    int status = IA_ERR_ARG;
    std::vector<double> xyz;
    std::vector<int> tri;
    long m = 0, ne = 0;
    do {
        if (!seek_section(fp, "$Nodes") || !next_line(fp, s)) break;
        m = strtol(s.c_str(), nullptr, 10);
        if (m <= 0 || m > (1L << 28)) break;
        xyz.resize(3 * (size_t)m);
        bool ok = true;
        for (long i = 0; i < m && ok; ++i) {
            if (!next_line(fp, s)) { ok = false; break; }
            char *p = const_cast<char *>(s.c_str()), *q;
            strtol(p, &q, 10);
            for (int d = 0; d < 3; ++d) {
                p = q;
                xyz[i + d * (size_t)m] = strtod(p, &q);
                if (q == p) ok = false;
            }
        }
        if (!ok || !seek_section(fp, "$Elements") || !next_line(fp, s)) break;
        ne = strtol(s.c_str(), nullptr, 10);
        if (ne < 0) break;
        for (long e = 0; e < ne && ok; ++e) {
            if (!next_line(fp, s)) { ok = false; break; }
            char *p = const_cast<char *>(s.c_str()), *q;
            strtol(p, &q, 10);                         // element number
            const long type = strtol(q, &p, 10);
            if (type != 2) continue;
            const long ntags = strtol(p, &q, 10);
            for (long g = 0; g < ntags; ++g) strtol(q, &q, 10);
            long v[3];
            for (int d = 0; d < 3; ++d) {
                p = q;
                v[d] = strtol(p, &q, 10) - 1;
                if (q == p || v[d] < 0 || v[d] >= m) ok = false;
            }
            if (ok && v[0] != v[1] && v[0] != v[2] && v[1] != v[2])
                for (int d = 0; d < 3; ++d) tri.push_back((int)v[d]);
        }
        if (ok) status = IA_OK;
    } while (0);
    fclose(fp);
    if (status) return status;
    const size_t n = tri.size() / 3;
    double *nodes = (double *)malloc(sizeof(double) * 3 * (size_t)m);
    double *field = (double *)malloc(sizeof(double) * 3 * (size_t)m);
    int *elems = (int *)malloc(sizeof(int) * 3 * (n ? n : 1));
    if (!nodes || !field || !elems) {
        free(nodes);
        free(field);
        free(elems);
        return IA_ERR_ALLOC;
    }
    const double scale = 1.0 + (2.0 * M_PI / k) * t;
    for (size_t i = 0; i < 3 * (size_t)m; ++i) {
        nodes[i] = xyz[i];
        field[i] = xyz[i] * scale;
    }
    for (size_t e = 0; e < n; ++e)
        for (int d = 0; d < 3; ++d) elems[e + d * n] = tri[3 * e + d];
    *r_ms = nodes;
    *r_lh = field;
    *e_n = elems;
    *m_out = (int)m;
    *l_out = (int)m;
    *n_out = (int)n;
    return IA_OK;
}
