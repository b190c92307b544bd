// ia_invr: the reference-compatible BEM radiation-mode entry point (invr()
// CUDA/invr.cuh:457 and invrgpu() CUDA/invr.cuh:263): one wavenumber, host
// arrays in, malloc'd host outputs q_e (m x n_am, left singular vectors of the
// complex G Z), h (l x n_am) = (A_hs Z - B_hs) q_e and m_e (m x n_am) = Z q_e.
// Runs ia_bem_modes_complex_batch on a private context and stream.
#include <math.h>
#include <stdlib.h>
#include "ia_common.cuh"
#include "ia_internal.h"

using namespace ia;

extern "C" int ia_invr(int m, int l, int n, const double *r_ms, const int *e_n, const double *r_lh, ia_complex **m_e,
                       ia_complex **h, ia_complex **q_e, double k, int n_ch, const double *cp, int n_am,
                       const ia_rules *rules, const ia_config *cfg)
{
    if (m < 3 || l < 1 || n < 1 || !r_ms || !e_n || !r_lh || !m_e || !h || !q_e || !(k > 0.0) || n_ch < 0 ||
        n_am < 1 || n_am > m)
        return IA_ERR_ARG;
    if (n_ch > 0 && !cp) return IA_ERR_ARG;
    for (size_t i = 0; i < 3 * (size_t)l; ++i)
        if (!isfinite(r_lh[i])) return IA_ERR_NONFINITE;
    for (size_t i = 0; i < 3 * (size_t)n_ch; ++i)
        if (!isfinite(cp[i])) return IA_ERR_NONFINITE;
    ia_config dc;
    if (!cfg) { ia_config_default(&dc); cfg = &dc; }
    cudaStream_t stream;
    IA_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    int dev = 0;
    cudaGetDevice(&dev);
    ia_context *ctx = nullptr;
    int st = ia_create(&ctx, dev, (void *)stream);
    if (st) { cudaStreamDestroy(stream); return st; }
    ia_mesh *mesh = nullptr;
    void *scratch = nullptr;
    ia_complex *hq = nullptr, *hh = nullptr, *hm = nullptr;
    int hinfo = 0;
    do {
        st = ia_mesh_create(ctx, m, n, r_ms, e_n, rules, &mesh);
        if (st) break;
        const size_t nmo = (size_t)m * n_am, nlo = (size_t)l * n_am;
        size_t need = ws_round(24 * (size_t)l) + ws_round(24 * (size_t)(n_ch ? n_ch : 1)) + ws_round(8) +
                      2 * ws_round(16 * nmo) + ws_round(16 * nlo) + ws_round(8 * (size_t)n_am) + ws_round(4) + 4096;
        cudaError_t e = cudaMallocAsync(&scratch, need, stream);
        if (e != cudaSuccess) { st = cuda_status(e); break; }
        WsCursor cur{(char *)scratch, 0, need};
        double *dl = cur.take<double>(3 * (size_t)l);
        double *dcp = cur.take<double>(3 * (size_t)(n_ch ? n_ch : 1));
        double *dk = cur.take<double>(1);
        ia_complex *dq = cur.take<ia_complex>(nmo);
        ia_complex *dm = cur.take<ia_complex>(nmo);
        ia_complex *dh = cur.take<ia_complex>(nlo);
        double *ds = cur.take<double>(n_am);
        int *dinfo = cur.take<int>(1);
        if ((e = cudaMemcpyAsync(dl, r_lh, 24 * (size_t)l, cudaMemcpyHostToDevice, stream)) != cudaSuccess ||
            (n_ch && (e = cudaMemcpyAsync(dcp, cp, 24 * (size_t)n_ch, cudaMemcpyHostToDevice, stream)) != cudaSuccess) ||
            (e = cudaMemcpyAsync(dk, &k, 8, cudaMemcpyHostToDevice, stream)) != cudaSuccess) {
            st = cuda_status(e);
            break;
        }
        if ((st = ia_bem_modes_complex_batch(ctx, mesh, l, dl, n_ch, n_ch ? dcp : nullptr, 1, dk, n_am, cfg, dq, ds,
                                             dh, dm, dinfo)))
            break;
        hq = (ia_complex *)malloc(16 * nmo);
        hm = (ia_complex *)malloc(16 * nmo);
        hh = (ia_complex *)malloc(16 * nlo);
        if (!hq || !hm || !hh) { st = IA_ERR_ALLOC; break; }
        if ((e = cudaMemcpyAsync(&hinfo, dinfo, 4, cudaMemcpyDeviceToHost, stream)) != cudaSuccess ||
            (e = cudaMemcpyAsync(hq, dq, 16 * nmo, cudaMemcpyDeviceToHost, stream)) != cudaSuccess ||
            (e = cudaMemcpyAsync(hm, dm, 16 * nmo, cudaMemcpyDeviceToHost, stream)) != cudaSuccess ||
            (e = cudaMemcpyAsync(hh, dh, 16 * nlo, cudaMemcpyDeviceToHost, stream)) != cudaSuccess ||
            (e = cudaStreamSynchronize(stream)) != cudaSuccess) {
            st = cuda_status(e);
            break;
        }
    } while (0);
    if (scratch) cudaFreeAsync(scratch, stream);
    cudaStreamSynchronize(stream);
    if (mesh) ia_mesh_destroy(mesh);
    ia_destroy(ctx);
    cudaStreamDestroy(stream);
    if (st) {
        free(hq);
        free(hm);
        free(hh);
        return st;
    }
    *q_e = hq;
    *m_e = hm;
    *h = hh;
    if (hinfo & IA_INFO_NONFINITE) return IA_ERR_NONFINITE;
    if (hinfo & IA_INFO_SINGULAR) return IA_ERR_SINGULAR;
    return IA_OK;
}
