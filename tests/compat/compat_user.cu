// A "user program" written against the reference's call surface: it includes
// the drop-in headers of include/compat/ and calls esm, ibem, invr, hels,
// csvd, tsvd, to_pressure and sound_power exactly as reference code would.  The
// test suite compiles it against libia.so, runs it on the GPU and compares
// what it writes with the oracle.
//
// usage: compat_user <in.bin> <out.bin>
//   in.bin : int32 m, l, n; double k, r_i; double r_ms[3m], r_lh[3l]; int32 e_n[3n]
//   out.bin: esm Me (m*m), He (l*m); ibem Z (m*m), H (l*m); hels Me, He, Qe (order 3);
//            csvd s (min(l,m)); tsvd x (m, k = 5); to_pressure p (l); sound_power w (1 double);
//            invr q_e (m*9), h (l*9), m_e (m*9)
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "esm.cuh"
#include "hels.cuh"
#include "ibem.cuh"
#include "invr.cuh"
#include "tsvd.cuh"
#include "utils.cuh"

template <class T>
static void put(FILE *f, const T *p, size_t n) { std::fwrite(p, sizeof(T), n, f); }

int main(int argc, char **argv)
{
    if (argc != 3) return 2;
    FILE *fi = std::fopen(argv[1], "rb");
    if (!fi) return 3;
    int dims[3];
    double kr[2];
    if (std::fread(dims, sizeof(int), 3, fi) != 3 || std::fread(kr, sizeof(double), 2, fi) != 2) return 4;
    const int m = dims[0], l = dims[1], n = dims[2];
    std::vector<double> r_ms(3 * (size_t)m), r_lh(3 * (size_t)l);
    std::vector<int> e_n(3 * (size_t)n);
    if (std::fread(r_ms.data(), sizeof(double), r_ms.size(), fi) != r_ms.size()) return 5;
    if (std::fread(r_lh.data(), sizeof(double), r_lh.size(), fi) != r_lh.size()) return 6;
    if (std::fread(e_n.data(), sizeof(int), e_n.size(), fi) != e_n.size()) return 7;
    std::fclose(fi);
    const double k = kr[0], r_i = kr[1];
    FILE *fo = std::fopen(argv[2], "wb");
    if (!fo) return 8;
    try {
        cuDoubleComplex *me, *he;
        esm(m, l, r_ms.data(), r_lh.data(), &me, &he, k, r_i);
        put(fo, me, (size_t)m * m);
        put(fo, he, (size_t)l * m);
        std::free(me);
        std::free(he);

        cuDoubleComplex *z, *h;
        ibem(m, l, n, r_ms.data(), e_n.data(), r_lh.data(), &z, &h, k, 0, nullptr);
        put(fo, z, (size_t)m * m);
        put(fo, h, (size_t)l * m);

        double *sph_s, *sph_h;
        cartesian_2_spherical(m, r_ms.data(), &sph_s);
        cartesian_2_spherical(l, r_lh.data(), &sph_h);
        cuDoubleComplex *hm, *hh, *hq;
        hels(m, l, sph_s, sph_h, &hm, &hh, &hq, k, 3);
        put(fo, hm, (size_t)m * 16);
        put(fo, hh, (size_t)l * 16);
        put(fo, hq, (size_t)m * 16);

        cuDoubleComplex *u, *v, *x, *p;
        double *s, w = 0.0;
        csvd(l, m, h, &u, &s, &v);
        const int pmin = l < m ? l : m;
        put(fo, s, (size_t)pmin);
        std::vector<cuDoubleComplex> b(l);
        for (int i = 0; i < l; ++i) b[i] = make_cuDoubleComplex(1.0 + 0.1 * i, -0.05 * i);
        tsvd(l, m, pmin, 5, u, s, v, b.data(), &x);
        put(fo, x, (size_t)m);
        to_pressure(l, m, h, x, &p);
        put(fo, p, (size_t)l);
        sound_power(l, p, b.data(), &w, 0.3);
        put(fo, &w, 1);
        cuDoubleComplex *rq, *rh, *rm;
        invr(m, l, n, r_ms.data(), e_n.data(), r_lh.data(), &rm, &rh, &rq, k, 0, nullptr, 9);
        put(fo, rq, (size_t)m * 9);
        put(fo, rh, (size_t)l * 9);
        put(fo, rm, (size_t)m * 9);
        std::free(rq);
        std::free(rh);
        std::free(rm);
        for (void *q : {(void *)z, (void *)h, (void *)sph_s, (void *)sph_h, (void *)hm, (void *)hh, (void *)hq,
                        (void *)u, (void *)s, (void *)v, (void *)x, (void *)p})
            std::free(q);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "compat_user: %s\n", e.what());
        std::fclose(fo);
        return 9;
    }
    std::fclose(fo);
    return 0;
}
