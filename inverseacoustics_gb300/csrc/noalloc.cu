// ia_solve_batch_noalloc: the batched SVD / GCV / Tikhonov solve without any
// device allocation.
//
// Some callers cannot call cudaMalloc: a microphone-array acquisition loop
// that reconstructs every block of frames on a real-time thread, where an
// allocation's implicit device synchronisation and unbounded latency would
// drop samples; and code that records the solve into a CUDA graph during
// stream capture, where the allocator may not be called.  This entry point
// takes its scratch from one file-scope __device__ array of
// IA_NOALLOC_SCRATCH_BYTES instead of the context's workspace.  Every GPU that
// loads the library holds that array until the process exits.
//
// Host code cannot use the array's name as a device address: on the first
// call on each device (with that device current) the address is looked up
// with cudaGetSymbolAddress and cached.  That first call should therefore come
// before any stream capture.  Every call shares the one array and leaves the
// previous call's contents in it; nothing in it is assumed to start at zero.
// Calls that overlap on the GPU (two streams, or two host threads) race on it.
//
// The GEMM autotuner is held off for the duration of the call: timing kernel
// variants on a shape's first use would take a stream-ordered scratch
// allocation and an event synchronisation.  A tile choice already in the
// tuner's table is used; otherwise the default tile, which sums in the same
// order, so the results do not depend on it.
#include <mutex>
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

static __device__ __align__(256) unsigned char g_noalloc_scratch[IA_NOALLOC_SCRATCH_BYTES];

static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[64];

// Address of the scratch array on the current device (looked up once).
static int noalloc_scratch(void **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_status(e);
    if (dev < 0 || dev >= 64) return IA_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e);
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return IA_OK;
}

}  // namespace ia

using namespace ia;

extern "C" int ia_solve_batch_noalloc(ia_context *ctx, int m, int n, int F, const ia_complex *d_H, int nrhs,
                                      const ia_complex *d_b, const ia_config *cfg, ia_complex *d_x, double *d_lambda,
                                      double *d_s, int *d_info)
{
    if (!ctx || !cfg || m < 1 || n < 1 || F < 1 || nrhs < 1 || !d_H || !d_b || !d_x || !d_info) return IA_ERR_ARG;
    if (m > n || cfg->precision != IA_PREC_FP64) return IA_ERR_ARG;
    const size_t need = wide_solve_ws_bytes(m, n, nrhs, F);
    if (need > (size_t)IA_NOALLOC_SCRATCH_BYTES) return IA_ERR_TOO_LARGE;
    int dev = -1;
    IA_CUDA_TRY(cudaGetDevice(&dev));
    if (dev != ctx->device) return IA_ERR_ARG;
    void *scratch = nullptr;
    int st = noalloc_scratch(&scratch);
    if (st) return st;
    IA_CUDA_TRY(cudaMemsetAsync(d_info, 0, sizeof(int) * (size_t)F, ctx->stream));
    WsCursor cur{(char *)scratch, 0, (size_t)IA_NOALLOC_SCRATCH_BYTES};
    const int prev = ctx->no_tune;
    ctx->no_tune = 1;
    st = wide_solve_batched(ctx, m, n, F, (const double2 *)d_H, false, nrhs, (const double2 *)d_b, cfg,
                            (double2 *)d_x, d_lambda, d_s, d_info, cur);
    ctx->no_tune = prev;
    return st;
}
