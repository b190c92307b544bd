// ia_ibem: the reference-compatible IBEM entry point (ibem() CUDA/ibem.cuh:424).
// Square systems use LU; CHIEF rows make the system overdetermined and it is
// solved in the least-squares sense by Householder QR, as the reference's
// zgels / ZZgels do (CUDA/ibem.cuh:752-755, :389-391).
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "ia_common.cuh"
#include "ia_internal.h"

using namespace ia;

extern "C" int ia_ibem(int m, int l, int n, const double *r_ms, const int *e_n, const double *r_lh, ia_complex **m_e,
                       ia_complex **h, double k, int n_ch, const double *cp, const ia_rules *rules,
                       const ia_config *cfg)
{
    if (m < 3 || l < 1 || n < 1 || !r_ms || !e_n || !r_lh || !m_e || !h || !(k > 0.0) || n_ch < 0) return IA_ERR_ARG;
    if (n_ch > 0 && !cp) return IA_ERR_ARG;
    for (size_t i = 0; i < 3 * (size_t)l; ++i)
        if (!isfinite(r_lh[i])) return IA_ERR_NONFINITE;
    for (size_t i = 0; i < 3 * (size_t)n_ch; ++i)
        if (!isfinite(cp[i])) return IA_ERR_NONFINITE;
    ia_config dc;
    if (!cfg) { ia_config_default(&dc); cfg = &dc; }
    // a private context: this call owns its stream and scratch
    cudaStream_t stream;
    IA_CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    int dev = 0;
    cudaGetDevice(&dev);
    ia_context *ctx = nullptr;
    int st = ia_create(&ctx, dev, (void *)stream);
    if (st) { cudaStreamDestroy(stream); return st; }
    ia_mesh *mesh = nullptr;
    void *scratch = nullptr;
    ia_complex *hz = nullptr, *hh = nullptr;
    int hinfo = 0;
    const int mt = m + n_ch;
    do {
        st = ia_mesh_create(ctx, m, n, r_ms, e_n, rules, &mesh);
        if (st) break;
        size_t need = ws_round(24 * (size_t)l) + ws_round(24 * (size_t)(n_ch ? n_ch : 1)) + ws_round(8) + 4 * ws_round(16 * (size_t)mt * m) +
                      3 * ws_round(16 * (size_t)l * m) + ws_round(4 * (size_t)m) + ws_round(4) + 8192;
        cudaError_t e = cudaMallocAsync(&scratch, need, stream);
        if (e != cudaSuccess) { st = cuda_status(e); break; }
        WsCursor cur{(char *)scratch, 0, need};
        double *dl = cur.take<double>(3 * (size_t)l);
        double *dcp = cur.take<double>(3 * (size_t)(n_ch ? n_ch : 1));
        double *dk = cur.take<double>(1);
        double2 *At = cur.take<double2>((size_t)mt * m);
        double2 *Bt = cur.take<double2>((size_t)mt * m);
        double2 *A = cur.take<double2>((size_t)mt * m);
        double2 *B = cur.take<double2>((size_t)mt * m);
        double2 *Aht = cur.take<double2>((size_t)l * m);
        double2 *Bht = cur.take<double2>((size_t)l * m);
        double2 *H = cur.take<double2>((size_t)l * m);
        int *ipiv = cur.take<int>(m);
        int *info = cur.take<int>(1);
        if ((e = cudaMemcpyAsync(dl, r_lh, 24 * (size_t)l, cudaMemcpyHostToDevice, stream)) != cudaSuccess ||
            (n_ch && (e = cudaMemcpyAsync(dcp, cp, 24 * (size_t)n_ch, cudaMemcpyHostToDevice, stream)) != cudaSuccess) ||
            (e = cudaMemcpyAsync(dk, &k, 8, cudaMemcpyHostToDevice, stream)) != cudaSuccess ||
            (e = cudaMemsetAsync(info, 0, 4, stream)) != cudaSuccess) {
            st = cuda_status(e);
            break;
        }
        if ((st = ibem_rows(ctx, mesh, l, dl, n_ch, dcp, 1, dk, cfg->c, cfg->rho, At, Bt, Aht, Bht))) break;
        // column-major A, B (mt x m), A_hs, B_hs (l x m)
        if ((st = ztranspose_batched(ctx, m, mt, At, m, 0, A, mt, 0, false, 1))) break;
        if ((st = ztranspose_batched(ctx, m, mt, Bt, m, 0, B, mt, 0, false, 1))) break;
        if ((st = ztranspose_batched(ctx, m, l, Bht, m, 0, H, l, 0, false, 1))) break;
        if ((st = ztranspose_batched(ctx, m, l, Aht, m, 0, Bht, l, 0, false, 1))) break;   // Bht := A_hs
        if (n_ch == 0) {
            if ((st = zgetrf_batched(ctx, m, A, mt, 0, ipiv, info, 1))) break;
            if ((st = zgetrs_batched(ctx, m, m, A, mt, 0, ipiv, B, mt, 0, 1))) break;
        } else {
            // least squares: Q^H [A | B], then R Z = (Q^H B)(1:m, :)
            if ((st = zgeqrs_batched(ctx, mt, m, A, mt, 0, m, B, mt, 0, 1))) break;
            if ((st = zbacksolve_upper_batched(ctx, m, m, A, mt, 0, B, mt, 0, 1))) break;
        }
        // H = A_hs Z - B_hs
        if ((st = zgemm_batched(ctx, OP_N, OP_N, l, m, m, make_double2(1.0, 0.0), Bht, l, 0, B, mt, 0,
                                make_double2(-1.0, 0.0), H, l, 0, 1)))
            break;
        // compact Z (ld mt -> m) into A's storage
        if ((st = zcopy2d_batched(ctx, m, m, B, mt, 0, A, m, 0, false, 1))) break;
        if ((e = cudaMemcpyAsync(&hinfo, info, 4, cudaMemcpyDeviceToHost, stream)) != cudaSuccess) { st = cuda_status(e); break; }
        hz = (ia_complex *)malloc(16 * (size_t)m * m);
        hh = (ia_complex *)malloc(16 * (size_t)l * m);
        if (!hz || !hh) { st = IA_ERR_ALLOC; break; }
        if ((e = cudaMemcpyAsync(hz, A, 16 * (size_t)m * m, cudaMemcpyDeviceToHost, stream)) != cudaSuccess ||
            (e = cudaMemcpyAsync(hh, H, 16 * (size_t)l * m, cudaMemcpyDeviceToHost, stream)) != cudaSuccess ||
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
        free(hz);
        free(hh);
        return st;
    }
    *m_e = hz;
    *h = hh;
    if (hinfo & IA_INFO_NONFINITE) return IA_ERR_NONFINITE;
    if (hinfo & IA_INFO_SINGULAR) return IA_ERR_SINGULAR;
    return IA_OK;
}
