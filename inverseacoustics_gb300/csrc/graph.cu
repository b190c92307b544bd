// CUDA graph capture and replay of batched calls.  A whole
// ia_*_solve_batch call (hundreds of kernels: assembly, blocked LU panels,
// GEMMs, QR, Jacobi, GCV) becomes one graph launch.
#include "ia_internal.h"

struct ia_graph {
    ia_context *ctx;
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    int kernels;
};

using namespace ia;

extern "C" {

int ia_capture_begin(ia_context *ctx)
{
    if (!ctx || ctx->capturing) return IA_ERR_ARG;
    if (ctx->stream == nullptr || ctx->stream == cudaStreamLegacy || ctx->stream == cudaStreamPerThread)
        return IA_ERR_ARG;
    // the side stream of split pipelines exists before the capture starts
    int st = ensure_side_stream(ctx);
    if (st) return st;
    IA_CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    ctx->capturing = 1;
    return IA_OK;
}

int ia_capture_end(ia_context *ctx, ia_graph **out)
{
    if (!ctx || !out || !ctx->capturing) return IA_ERR_ARG;
    *out = nullptr;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    ctx->capturing = 0;
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_status(e);
    }
    size_t n = 0;
    e = cudaGraphGetNodes(g, nullptr, &n);
    int kernels = 0;
    if (e == cudaSuccess && n) {
        cudaGraphNode_t *nodes = (cudaGraphNode_t *)malloc(sizeof(cudaGraphNode_t) * n);
        if (!nodes) {
            cudaGraphDestroy(g);
            return IA_ERR_ALLOC;
        }
        e = cudaGraphGetNodes(g, nodes, &n);
        for (size_t i = 0; e == cudaSuccess && i < n; ++i) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
        }
        free(nodes);
    }
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_status(e);
    }
    ia_graph *G = (ia_graph *)calloc(1, sizeof(ia_graph));
    if (!G) {
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(g);
        return IA_ERR_ALLOC;
    }
    G->ctx = ctx;
    G->graph = g;
    G->exec = exec;
    G->kernels = kernels;
    *out = G;
    return IA_OK;
}

int ia_graph_launch(ia_graph *G)
{
    if (!G) return IA_ERR_ARG;
    IA_CUDA_TRY(cudaGraphLaunch(G->exec, G->ctx->stream));
    G->ctx->launches += G->kernels;
    return IA_OK;
}

int ia_graph_kernel_count(const ia_graph *G) { return G ? G->kernels : -1; }

int ia_graph_destroy(ia_graph *G)
{
    if (!G) return IA_OK;
    cudaGraphExecDestroy(G->exec);
    cudaGraphDestroy(G->graph);
    free(G);
    return IA_OK;
}

}  // extern "C"
