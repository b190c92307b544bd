// C ABI of libia.so: contexts, workspace, meshes, the reference-compatible
// host entry points and the batched device pipelines.  See include/ia.h.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <functional>
#include <initializer_list>
#include <mutex>
#include <tuple>
#include <vector>
#include "ia_common.cuh"
#include "df32.cuh"
#include "ia_internal.h"

static thread_local int g_last_cuda_error = 0;

namespace ia {

int cuda_status(cudaError_t e)
{
    g_last_cuda_error = (int)e;
    if (e == cudaErrorMemoryAllocation) return IA_ERR_ALLOC;
    return IA_ERR_CUDA;
}

int ws_reserve(ia_context *ctx, size_t bytes)
{
    if (bytes <= ctx->ws_bytes) return IA_OK;
    if (ctx->capturing) return IA_ERR_CAPTURE;
    if (ctx->ws) {
        cudaError_t e = cudaFreeAsync(ctx->ws, ctx->stream);
        ctx->ws = nullptr;
        ctx->ws_bytes = 0;
        if (e != cudaSuccess) return cuda_status(e);
    }
    size_t grow = bytes + bytes / 8;
    cudaError_t e = cudaMallocAsync(&ctx->ws, grow, ctx->stream);
    if (e != cudaSuccess) {
        ctx->ws = nullptr;
        return cuda_status(e);
    }
    ctx->ws_bytes = grow;
    return IA_OK;
}

// ---- built-in quadrature rules ------------------------------------------
// Gauss-Legendre nodes/weights on [0, 1] by Newton iteration on P_n.
static void gauss_legendre01(int n, std::vector<double> &x, std::vector<double> &w)
{
    x.resize(n);
    w.resize(n);
    for (int i = 0; i < n; ++i) {
        double z = cos(M_PI * (i + 0.75) / (n + 0.5));
        double dp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; ++k) {
                double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            if (n == 1) { p1 = z; p0 = 1.0; }
            dp = n * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (fabs(dz) < 1e-16) break;
        }
        x[n - 1 - i] = 0.5 * (1.0 + z);      // ascending
        w[n - 1 - i] = 1.0 / ((1.0 - z * z) * dp * dp);
    }
}

// Radon's 7-point degree-5 triangle rule (weights scaled to sum 1/2).
static void radon7(std::vector<double> &rule)
{
    const double s15 = sqrt(15.0);
    const double a1 = (6.0 - s15) / 21.0, b1 = (9.0 + 2.0 * s15) / 21.0, w1 = (155.0 - s15) / 1200.0;
    const double a2 = (6.0 + s15) / 21.0, b2 = (9.0 - 2.0 * s15) / 21.0, w2 = (155.0 + s15) / 1200.0;
    const double pts[7][3] = {{1.0 / 3.0, 1.0 / 3.0, 9.0 / 40.0}, {a1, a1, w1}, {b1, a1, w1}, {a1, b1, w1},
                              {a2, a2, w2}, {b2, a2, w2}, {a2, b2, w2}};
    rule.assign(21, 0.0);
    for (int q = 0; q < 7; ++q) {
        rule[q] = pts[q][0];
        rule[q + 7] = pts[q][1];
        rule[q + 14] = 0.5 * pts[q][2];
    }
}

// Duffy rule for a singularity at vertex `page` (shape function of that vertex
// = 1): collapse the unit square onto the triangle at that vertex,
//   N_page = 1 - u, N_next = u (1 - v), N_prev = u v,  weight w_u w_v u.
static void duffy_rule(int nu, int nv, std::vector<double> &rule)
{
    std::vector<double> xu, wu, xv, wv;
    gauss_legendre01(nu, xu, wu);
    gauss_legendre01(nv, xv, wv);
    const int nq = nu * nv;
    rule.assign(9 * (size_t)nq, 0.0);
    for (int page = 0; page < 3; ++page) {
        double *P = rule.data() + (size_t)3 * nq * page;
        for (int a = 0; a < nu; ++a)
            for (int b = 0; b < nv; ++b) {
                int q = a * nv + b;
                double u = xu[a], v = xv[b];
                double N[3];
                N[page] = 1.0 - u;
                N[(page + 1) % 3] = u * (1.0 - v);
                N[(page + 2) % 3] = u * v;
                P[q] = N[0];
                P[q + nq] = N[1];
                P[q + 2 * nq] = wu[a] * wv[b] * u;
            }
    }
}

static int check_rule(int nq, const double *r)
{
    if (nq < 1 || !r) return IA_ERR_RULE;
    double s = 0.0;
    for (int q = 0; q < nq; ++q) {
        if (!isfinite(r[q]) || !isfinite(r[q + nq]) || !isfinite(r[q + 2 * nq])) return IA_ERR_RULE;
        s += r[q + 2 * nq];
    }
    return fabs(s - 0.5) < 1e-9 ? IA_OK : IA_ERR_RULE;
}

// ---- default context for the reference-compatible entry points ---------
static std::mutex g_compat_mu;
static ia_context *g_compat_ctx[64];

static ia_context *compat_context(int *st)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { *st = cuda_status(e); return nullptr; }
    if (dev < 0 || dev >= 64) { *st = IA_ERR_ARG; return nullptr; }
    if (!g_compat_ctx[dev]) {
        cudaStream_t s;
        e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (e != cudaSuccess) { *st = cuda_status(e); return nullptr; }
        int r = ia_create(&g_compat_ctx[dev], dev, (void *)s);
        if (r) { *st = r; return nullptr; }
    }
    *st = IA_OK;
    return g_compat_ctx[dev];
}

template <class T>
static int to_host_malloc(ia_context *ctx, const T *d, size_t count, T **out)
{
    T *h = (T *)malloc(sizeof(T) * (count ? count : 1));
    if (!h) return IA_ERR_ALLOC;
    cudaError_t e = cudaMemcpyAsync(h, d, sizeof(T) * count, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) { free(h); return cuda_status(e); }
    *out = h;
    return IA_OK;
}

static bool all_finite(const double *p, size_t n)
{
    for (size_t i = 0; i < n; ++i)
        if (!isfinite(p[i])) return false;
    return true;
}

int ensure_side_stream(ia_context *ctx)
{
    if (ctx->side[0]) return IA_OK;
    constexpr int NS = IA_SPLIT_PARTS, NE = IA_SPLIT_PARTS;
    cudaStream_t s[NS] = {};
    cudaEvent_t er[NE] = {}, ed[NE] = {}, ef = nullptr;
    // (Stream priorities that put part q's chain ahead of part q+1's assembly
    // measured slower: 2089 vs 2175 freq-solves/s on the 64-bin sphere; the
    // last part's assembly, and so its chain, then starts later.)
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < NS && e == cudaSuccess; ++i) e = cudaStreamCreateWithFlags(&s[i], cudaStreamNonBlocking);
    for (int i = 0; i < NE && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&er[i], cudaEventDisableTiming);
    for (int i = 0; i < NE && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&ed[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ef, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        for (int i = 0; i < NE; ++i) {
            if (er[i]) cudaEventDestroy(er[i]);
            if (ed[i]) cudaEventDestroy(ed[i]);
        }
        if (ef) cudaEventDestroy(ef);
        for (int i = 0; i < NS; ++i)
            if (s[i]) cudaStreamDestroy(s[i]);
        return cuda_status(e);
    }
    for (int i = 0; i < NS; ++i) ctx->side[i] = s[i];
    for (int i = 0; i < NE; ++i) {
        ctx->ev_rows[i] = er[i];
        ctx->ev_done[i] = ed[i];
    }
    ctx->ev_fork = ef;
    return IA_OK;
}

}  // namespace ia

using namespace ia;

// =========================================================================
extern "C" {

int ia_last_fallback_bins(const ia_context *ctx) { return ctx ? ctx->last_fallback : 0; }

void ia_config_default(ia_config *cfg)
{
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->c = 343.0;
    cfg->rho = 1.21;
    cfg->method = IA_METHOD_TIKHONOV_GCV;
    cfg->gcv_mode = IA_GCV_STANDARD;
    cfg->gcv_points = 200;
    cfg->gcv_lo = 0.0;
    cfg->gcv_hi = 0.0;
    cfg->lambda_fixed = 0.0;
    cfg->tsvd_k = 1;
    cfg->precision = IA_PREC_FP64;
    cfg->svd_max_sweeps = 40;
    cfg->refine_steps = 1;
    cfg->mode_iters = 10;
    cfg->mode_oversample = 16;
    cfg->gemm_slices = TC_SLICES_DEFAULT;
    cfg->mixed_guard = 1e-3;
    cfg->mixed_fallback = 1;
}

void ia_admm_config_default(ia_admm_config *cfg)
{
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->norm = IA_ADMM_L1;
    cfg->max_iters = 200;
    cfg->rho = 1.0;
    cfg->gamma = 1.0;
    cfg->epsilon = 1e-6;
    cfg->p = 0.5;
    cfg->gst_iters = 5;
    cfg->precision = IA_PREC_FP64;
}

const char *ia_status_string(int status)
{
    switch (status) {
    case IA_OK: return "ok";
    case IA_ERR_ARG: return "invalid argument";
    case IA_ERR_CUDA: return "CUDA runtime error";
    case IA_ERR_ALLOC: return "allocation failed";
    case IA_ERR_NOCONV: return "Jacobi iteration did not converge";
    case IA_ERR_SINGULAR: return "singular matrix";
    case IA_ERR_NONFINITE: return "non-finite value";
    case IA_ERR_RULE: return "invalid quadrature rule";
    case IA_ERR_TOO_LARGE: return "size above the entry point's limit";
    case IA_ERR_CAPTURE: return "workspace would grow during stream capture";
    default: return "unknown status";
    }
}

const char *ia_version(void) { return "ia-gb300 0.1 (sm_103a)"; }
int ia_config_size(void) { return (int)sizeof(ia_config); }
int ia_last_cuda_error(void) { return g_last_cuda_error; }

int ia_bounds_report(int *enabled, unsigned long long *count, const char **file, int *line, long long *index,
                     long long *extent)
{
    if (!enabled || !count || !file || !line || !index || !extent) return IA_ERR_ARG;
    *count = 0;
    *file = nullptr;
    *line = 0;
    *index = *extent = 0;
#ifndef IA_DEBUG_BOUNDS
    *enabled = 0;   // release build: nothing is checked, no device access
    return IA_OK;
#else
    *enabled = 1;
    const struct {
        const char *name;
        int (*read)(ia::IaBoundsSite *);
    } units[] = {{"dense.cu", ia::bounds_read_dense}, {"tc_gemm.cu", ia::bounds_read_tc},
                 {"svd.cu", ia::bounds_read_svd},     {"wide_solve.cu", ia::bounds_read_wide},
                 {"ibem_assemble.cu", ia::bounds_read_asm}};
    if (cudaDeviceSynchronize() != cudaSuccess) return IA_ERR_CUDA;
    for (const auto &u : units) {
        ia::IaBoundsSite site;
        const int st = u.read(&site);
        if (st) return st;
        if (site.count && !*file) {
            *file = u.name;
            *line = site.line;
            *index = site.index;
            *extent = site.extent;
        }
        *count += site.count;
    }
    return IA_OK;
#endif
}
void ia_free(void *p) { free(p); }

int ia_create(ia_context **out, int device, void *stream)
{
    if (!out) return IA_ERR_ARG;
    *out = nullptr;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_status(e);
    ia_context *c = (ia_context *)calloc(1, sizeof(ia_context));
    if (!c) return IA_ERR_ALLOC;
    c->device = device;
    c->stream = (cudaStream_t)stream;
    int sm = 0;
    cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device);
    c->sm_count = sm;
    *out = c;
    return IA_OK;
}

int ia_destroy(ia_context *ctx)
{
    if (!ctx) return IA_OK;
    for (int i = 0; i < IA_SPLIT_PARTS; ++i)
        if (ctx->side[i]) cudaStreamSynchronize(ctx->side[i]);
    if (ctx->ws) {
        cudaFreeAsync(ctx->ws, ctx->stream);
        cudaStreamSynchronize(ctx->stream);
    }
    if (ctx->side[0]) {
        for (int i = 0; i < IA_SPLIT_PARTS; ++i) {
            cudaEventDestroy(ctx->ev_rows[i]);
            cudaEventDestroy(ctx->ev_done[i]);
        }
        cudaEventDestroy(ctx->ev_fork);
        for (int i = 0; i < IA_SPLIT_PARTS; ++i) cudaStreamDestroy(ctx->side[i]);
    }
    if (ctx->dcount) cudaFree(ctx->dcount);
    free(ctx);
    return IA_OK;
}

int ia_set_stream(ia_context *ctx, void *stream)
{
    if (!ctx || ctx->capturing) return IA_ERR_ARG;
    cudaStream_t ns = (cudaStream_t)stream;
    if (ctx->ws && ns != ctx->stream) {
        // keep the workspace: work on the new stream waits for what the old
        // stream has queued on it
        cudaEvent_t ev;
        IA_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        cudaError_t e = cudaEventRecord(ev, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ns, ev, 0);
        cudaEventDestroy(ev);
        if (e != cudaSuccess) return cuda_status(e);
    }
    ctx->stream = ns;
    return IA_OK;
}

int ia_synchronize(ia_context *ctx)
{
    if (!ctx) return IA_ERR_ARG;
    IA_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return IA_OK;
}

long long ia_launch_count(const ia_context *ctx) { return ctx ? ctx->launches : 0; }

// ---- mesh -----------------------------------------------------------------
int ia_mesh_create(ia_context *ctx, int m, int n, const double *nodes, const int *elems, const ia_rules *rules,
                   ia_mesh **out)
{
    if (!ctx || !out || !nodes || !elems || m < 3 || n < 1) return IA_ERR_ARG;
    *out = nullptr;
    if (!all_finite(nodes, (size_t)3 * m)) return IA_ERR_NONFINITE;
    for (int i = 0; i < n; ++i) {
        int a = elems[i], b = elems[i + n], c = elems[i + 2 * n];
        if (a < 0 || b < 0 || c < 0 || a >= m || b >= m || c >= m) return IA_ERR_ARG;
        if (a == b || b == c || a == c) return IA_ERR_ARG;
    }
    {
        // two nodes at the same point give two equal collocation rows (a
        // singular system): refused, like a degenerate element
        std::vector<int> ord(m);
        for (int i = 0; i < m; ++i) ord[i] = i;
        auto key = [&](int i) { return std::make_tuple(nodes[i], nodes[i + m], nodes[i + 2 * m]); };
        std::sort(ord.begin(), ord.end(), [&](int x, int y) { return key(x) < key(y); });
        for (int i = 1; i < m; ++i)
            if (key(ord[i]) == key(ord[i - 1])) return IA_ERR_ARG;
    }
    std::vector<double> reg, sing;
    int nq, nqs;
    if (rules) {
        nq = rules->nq;
        nqs = rules->nqs;
        if (check_rule(nq, rules->regular)) return IA_ERR_RULE;
        for (int p = 0; p < 3; ++p)
            if (!rules->singular || check_rule(nqs, rules->singular + (size_t)3 * nqs * p)) return IA_ERR_RULE;
        reg.assign(rules->regular, rules->regular + 3 * (size_t)nq);
        sing.assign(rules->singular, rules->singular + 9 * (size_t)nqs);
    } else {
        radon7(reg);
        nq = 7;
        duffy_rule(4, 4, sing);
        nqs = 16;
    }
    // node -> elements
    std::vector<std::vector<int>> node_elems(m);
    for (int i = 0; i < n; ++i)
        for (int s = 0; s < 3; ++s) node_elems[elems[i + s * n]].push_back(i);
    // greedy colouring: no two elements of one colour share a vertex
    std::vector<int> color(n, -1);
    int ncolors = 0;
    std::vector<char> used;
    for (int i = 0; i < n; ++i) {
        used.assign(ncolors + 1, 0);
        for (int s = 0; s < 3; ++s)
            for (int o : node_elems[elems[i + s * n]])
                if (color[o] >= 0) used[color[o]] = 1;
        int c = 0;
        while (c < ncolors && used[c]) ++c;
        color[i] = c;
        if (c == ncolors) ++ncolors;
    }
    // balance: the assembly kernel walks a colour with IA_ASM_THREADS threads
    // and a barrier after it, so a colour of 129..256 elements costs two
    // rounds.  Move elements out of colours above that size into the smallest
    // colour with no neighbour in it (at least ceil(n / IA_ASM_THREADS)
    // colours), a few passes; greedy sizes like 177, 168, ..., 30, 2 become
    // all 128 on the icospheres.
    {
        const int cap = IA_ASM_THREADS;
        const int target = std::max(ncolors, (n + cap - 1) / cap);
        std::vector<int> size(target, 0);
        for (int i = 0; i < n; ++i) size[color[i]]++;
        std::vector<char> nbc(target);
        for (int pass = 0; pass < 20; ++pass) {
            int moved = 0;
            for (int i = 0; i < n; ++i) {
                const int c = color[i];
                if (size[c] <= cap) continue;
                std::fill(nbc.begin(), nbc.end(), 0);
                for (int s = 0; s < 3; ++s)
                    for (int o : node_elems[elems[i + s * n]])
                        if (o != i) nbc[color[o]] = 1;
                int best = -1;
                for (int d = 0; d < target; ++d)
                    if (!nbc[d] && size[d] < cap && (best < 0 || size[d] < size[best])) best = d;
                if (best >= 0) {
                    color[i] = best;
                    size[c]--;
                    size[best]++;
                    ++moved;
                }
            }
            if (!moved) break;
        }
        // drop colours left empty
        std::vector<int> remap(target, -1);
        ncolors = 0;
        for (int d = 0; d < target; ++d)
            if (size[d] > 0) remap[d] = ncolors++;
        for (int i = 0; i < n; ++i) color[i] = remap[color[i]];
    }
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return color[a] < color[b]; });
    std::vector<int> newidx(n);
    for (int t = 0; t < n; ++t) newidx[order[t]] = t;
    std::vector<int> cptr(ncolors + 1, 0);
    for (int i = 0; i < n; ++i) cptr[color[i] + 1]++;
    for (int c = 0; c < ncolors; ++c) cptr[c + 1] += cptr[c];
    std::vector<double> egeo((size_t)16 * n, 0.0);
    std::vector<int> evert((size_t)4 * n, 0);
    for (int t = 0; t < n; ++t) {
        int i = order[t];
        double v[3][3];
        for (int s = 0; s < 3; ++s) {
            int node = elems[i + s * n];
            evert[4 * t + s] = node;
            for (int d = 0; d < 3; ++d) v[s][d] = nodes[node + d * m];
        }
        evert[4 * t + 3] = color[i];
        double a0 = v[0][0] - v[2][0], a1 = v[0][1] - v[2][1], a2 = v[0][2] - v[2][2];
        double b0 = v[1][0] - v[2][0], b1 = v[1][1] - v[2][1], b2 = v[1][2] - v[2][2];
        double nx = a1 * b2 - a2 * b1, ny = a2 * b0 - a0 * b2, nz = a0 * b1 - a1 * b0;
        double *g = &egeo[(size_t)16 * t];
        for (int s = 0; s < 3; ++s)
            for (int d = 0; d < 3; ++d) g[3 * s + d] = v[s][d];
        g[9] = nx;
        g[10] = ny;
        g[11] = nz;
        g[12] = sqrt(nx * nx + ny * ny + nz * nz);
    }
    // regular-rule points per element (colour order), structure of arrays
    std::vector<double> qdat((size_t)9 * nq * n);
    for (int t = 0; t < n; ++t) {
        const double *g = &egeo[(size_t)16 * t];
        for (int q = 0; q < nq; ++q) {
            const double x1 = reg[q], x2 = reg[q + nq], w = reg[q + 2 * nq] * IA_INV4PI;
            const double N[3] = {x1, x2, 1.0 - x1 - x2};
            double *p = &qdat[(size_t)q * 9 * n + t];
            for (int d = 0; d < 3; ++d) p[(size_t)d * n] = N[0] * g[d] + N[1] * g[3 + d] + N[2] * g[6 + d];
            for (int v = 0; v < 3; ++v) {
                p[(size_t)(3 + v) * n] = w * N[v];
                p[(size_t)(6 + v) * n] = w * N[v] * g[12];
            }
        }
    }
    std::vector<double> qnrm((size_t)3 * n);
    for (int t = 0; t < n; ++t)
        for (int d = 0; d < 3; ++d) qnrm[(size_t)d * n + t] = egeo[(size_t)16 * t + 9 + d];
    // double-float copies (hi, lo) for the mixed-path assembly
    auto split = [](const std::vector<double> &src) {
        std::vector<float> out(2 * src.size());
        for (size_t i = 0; i < src.size(); ++i) {
            float h = (float)src[i];
            out[2 * i] = h;
            out[2 * i + 1] = (float)(src[i] - (double)h);
        }
        return out;
    };
    const std::vector<float> qdat_f = split(qdat), qnrm_f = split(qnrm);
    std::vector<int> aptr(m + 1, 0), adj;
    adj.reserve((size_t)3 * n);
    for (int o = 0; o < m; ++o) {
        std::vector<int> inc;
        for (int i : node_elems[o]) {
            int slot = elems[i] == o ? 0 : (elems[i + n] == o ? 1 : 2);
            inc.push_back(newidx[i] * 4 + slot);
        }
        std::sort(inc.begin(), inc.end());
        for (int v : inc) adj.push_back(v);
        aptr[o + 1] = (int)adj.size();
    }
    ia_mesh *M = (ia_mesh *)calloc(1, sizeof(ia_mesh));
    if (!M) return IA_ERR_ALLOC;
    M->ctx = ctx;
    M->m = m;
    M->n = n;
    M->ncolors = ncolors;
    M->nq = nq;
    M->nqs = nqs;
    cudaError_t e = cudaSuccess;
    auto up = [&](void **dst, const void *src, size_t bytes) {
        if (e != cudaSuccess) return;
        e = cudaMalloc(dst, bytes ? bytes : 16);
        if (e == cudaSuccess && bytes) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    };
    up((void **)&M->d_nodes, nodes, sizeof(double) * 3 * (size_t)m);
    up((void **)&M->d_egeo, egeo.data(), sizeof(double) * egeo.size());
    up((void **)&M->d_evert, evert.data(), sizeof(int) * evert.size());
    up((void **)&M->d_color_ptr, cptr.data(), sizeof(int) * cptr.size());
    up((void **)&M->d_adj_ptr, aptr.data(), sizeof(int) * aptr.size());
    up((void **)&M->d_adj, adj.data(), sizeof(int) * adj.size());
    up((void **)&M->d_reg, reg.data(), sizeof(double) * reg.size());
    up((void **)&M->d_sing, sing.data(), sizeof(double) * sing.size());
    up((void **)&M->d_qdat, qdat.data(), sizeof(double) * qdat.size());
    up((void **)&M->d_qnrm, qnrm.data(), sizeof(double) * qnrm.size());
    up((void **)&M->d_qdat_f, qdat_f.data(), sizeof(float) * qdat_f.size());
    up((void **)&M->d_qnrm_f, qnrm_f.data(), sizeof(float) * qnrm_f.size());
    {
        // (sin, cos)(j pi / 512) as double-float pairs, evaluated in long
        // double (x86 extended or Arm quad) so the argument carries more
        // bits than the FP64 result
        const long double pi_l = 3.14159265358979323846264338327950288L;
        std::vector<float> tab(4 * DF_TRIG_TABLE);
        for (int j = 0; j < DF_TRIG_TABLE; ++j) {
            const long double t = (long double)j * pi_l / (DF_TRIG_TABLE / 2);
            const double s = (double)sinl(t), c = (double)cosl(t);
            const float sh = (float)s, ch = (float)c;
            tab[4 * j] = sh;
            tab[4 * j + 1] = (float)(s - (double)sh);
            tab[4 * j + 2] = ch;
            tab[4 * j + 3] = (float)(c - (double)ch);
        }
        up((void **)&M->d_dftab, tab.data(), sizeof(float) * tab.size());
    }
    // node-node pattern (nodes sharing an element, the node itself included),
    // CSR with sorted columns: the sparsity of the surface mass matrix
    {
        std::vector<int> gptr(m + 1, 0), gidx;
        std::vector<int> row;
        for (int i = 0; i < m; ++i) {
            row.clear();
            row.push_back(i);
            for (int el : node_elems[i])
                for (int s2 = 0; s2 < 3; ++s2) row.push_back(elems[el + s2 * n]);
            std::sort(row.begin(), row.end());
            row.erase(std::unique(row.begin(), row.end()), row.end());
            gidx.insert(gidx.end(), row.begin(), row.end());
            gptr[i + 1] = (int)gidx.size();
        }
        M->gnnz = (int)gidx.size();
        up((void **)&M->d_gptr, gptr.data(), sizeof(int) * gptr.size());
        up((void **)&M->d_gidx, gidx.data(), sizeof(int) * gidx.size());
    }
    if (e == cudaSuccess) e = cudaMalloc((void **)&M->d_creg, sizeof(double) * (size_t)m);
    if (e != cudaSuccess) {
        ia_mesh_destroy(M);
        return cuda_status(e);
    }
    // complete before any stream of the context reads it
    int st = mesh_creg(ctx, M);
    if (!st) {
        const cudaError_t ce = cudaStreamSynchronize(ctx->stream);
        if (ce != cudaSuccess) st = cuda_status(ce);
    }
    if (st) {
        ia_mesh_destroy(M);
        return st;
    }
    *out = M;
    return IA_OK;
}

int ia_mesh_destroy(ia_mesh *M)
{
    if (!M) return IA_OK;
    cudaFree(M->d_nodes);
    cudaFree(M->d_egeo);
    cudaFree(M->d_evert);
    cudaFree(M->d_color_ptr);
    cudaFree(M->d_adj_ptr);
    cudaFree(M->d_adj);
    cudaFree(M->d_gptr);
    cudaFree(M->d_gidx);
    cudaFree(M->d_reg);
    cudaFree(M->d_sing);
    cudaFree(M->d_qdat);
    cudaFree(M->d_qnrm);
    cudaFree(M->d_qdat_f);
    cudaFree(M->d_qnrm_f);
    cudaFree(M->d_dftab);
    cudaFree(M->d_creg);
    free(M);
    return IA_OK;
}

// ---- batched device entry points ------------------------------------------
// info words are bit sets OR-ed by the kernels: every batched call that takes
// one starts from zero
static int clear_info(ia_context *ctx, int *d_info, int F)
{
    if (d_info) IA_CUDA_TRY(cudaMemsetAsync(d_info, 0, sizeof(int) * (size_t)F, ctx->stream));
    return IA_OK;
}

int ia_monopole_batch(ia_context *ctx, int l, int m, int F, const double *d_mics, const double *d_src,
                      const double *d_k, ia_complex *d_G)
{
    if (!ctx || l < 1 || m < 1 || F < 1 || !d_mics || !d_src || !d_k || !d_G) return IA_ERR_ARG;
    return monopole_batched(ctx, l, m, F, d_mics, d_src, d_k, (double2 *)d_G);
}

int ia_ibem_assemble_batch(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int n_ch,
                           const double *d_cp, int F, const double *d_k, const ia_config *cfg, ia_complex *d_At,
                           ia_complex *d_Bt, ia_complex *d_Ahs_t, ia_complex *d_Bhs_t)
{
    if (!ctx || !mesh || !cfg || F < 1 || l < 0 || n_ch < 0 || !d_k) return IA_ERR_ARG;
    if ((l > 0 && !d_mics) || (n_ch > 0 && !d_cp)) return IA_ERR_ARG;
    const bool mixed = cfg->precision == IA_PREC_MIXED;
    // the double-float assembly's geometry table lives in the workspace
    float2 *G = nullptr;
    const size_t gbytes = mixed ? ibem_geom_bytes(mesh, mesh->m + n_ch + l) : 0;
    if (gbytes) {
        const int st = ws_reserve(ctx, gbytes);
        if (st) return st;
        G = reinterpret_cast<float2 *>(ctx->ws);
    }
    return ibem_rows(ctx, mesh, l, d_mics, n_ch, d_cp, F, d_k, cfg->c, cfg->rho, (double2 *)d_At, (double2 *)d_Bt,
                     (double2 *)d_Ahs_t, (double2 *)d_Bhs_t, mixed, false, G);
}

// H^T (m x l per frequency) into Ht, given workspace for A^T, B^T, pivots.
static int ibem_transfer_t(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int F,
                           const double *d_k, const ia_config *cfg, double2 *At, double2 *Bt, int *ipiv,
                           double2 *Ahs_t, double2 *Ht, int *d_info, cudaEvent_t ev_rows = nullptr)
{
    const int m = mesh->m;
    int st;
    {
        NvtxRange r("ia.assembly");
        st = ibem_rows(ctx, mesh, l, d_mics, 0, nullptr, F, d_k, cfg->c, cfg->rho, At, Bt, Ahs_t, Ht);
    }
    if (st) return st;
    if (ev_rows) IA_CUDA_TRY(cudaEventRecord(ev_rows, ctx->stream));
    NvtxRange r("ia.transfer");
    const long long sMM = (long long)m * m, sML = (long long)m * l;
    // LU of M = A^T; solve M Y = A_hs^T  ->  Y = W^T, W = A_hs A^-1
    st = zgetrf_batched(ctx, m, At, m, sMM, ipiv, d_info, F);
    if (st) return st;
    st = zgetrs_batched(ctx, m, l, At, m, sMM, ipiv, Ahs_t, m, sML, F);
    if (st) return st;
    // H^T = B^T Y - B_hs^T  (in place over B_hs^T)
    return zgemm_batched(ctx, OP_N, OP_N, m, l, m, make_double2(1.0, 0.0), Bt, m, sMM, Ahs_t, m, sML,
                         make_double2(-1.0, 0.0), Ht, m, sML, F);
}

// the FP64-level products of the mixed transfer run on the tensor cores
static bool tc_products(const ia_config *cfg, int m) { return tc_products_ok(cfg->gemm_slices, m); }

// The assembly's geometry table: in the transfer's own workspace, or (the
// staggered parts of one solve) one table that the first part writes and
// the later parts, which start after the first part's assembly, read.
struct GeomTable {
    float2 *p;
    bool build;
};

// with_table: the transfer's workspace holds its own geometry table
static size_t transfer_mixed_ws_bytes(const ia_mesh *mesh, int l, int F, const ia_config *cfg, bool with_table = true)
{
    const int m = mesh->m;
    size_t b = ws_round(8 * (size_t)m * m * F) + ws_round(8 * (size_t)m * l * F) + 3 * ws_round(16 * (size_t)m * l * F) +
               (with_table ? ws_round(ibem_geom_bytes(mesh, m + l)) : 0);
    if (tc_products(cfg, m))
        b += tc_planes_bytes(m, m, cfg->gemm_slices, false, F) + tc_planes_bytes(l, m, cfg->gemm_slices, true, F) +
             1024;
    return b;
}

// Mixed transfer: FP32 LU of M = A^T; Y = M^-1 A_hs^T by FP32 solves refined
// with FP64-level residuals R = A_hs^T - M Y (cfg->refine_steps times);
// H^T = B^T Y - B_hs^T.  The two FP64-level products (m x l x m) run on the
// tensor cores (BF16 slices of M, B^T and Y; cfg->gemm_slices) or, with
// gemm_slices 0, as double-float CUDA-core GEMMs.  Matrices in, H^T out in FP64.
static int ibem_transfer_t_mixed(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int F,
                                 const double *d_k, const ia_config *cfg, double2 *At, double2 *Bt, int *ipiv,
                                 double2 *Ahs_t, double2 *Ht, int *d_info, WsCursor &cur,
                                 cudaEvent_t ev_rows = nullptr, const GeomTable *shared_geom = nullptr)
{
    const int m = mesh->m;
    float2 *M32 = cur.take<float2>((size_t)m * m * F);
    float2 *Y32 = cur.take<float2>((size_t)m * l * F);
    double2 *Y = cur.take<double2>((size_t)m * l * F);
    double2 *R = cur.take<double2>((size_t)m * l * F);
    float4 *Y4 = cur.take<float4>((size_t)m * l * F);
    const size_t gbytes = ibem_geom_bytes(mesh, m + l);
    float2 *G = nullptr;
    bool build_geom = true;
    if (shared_geom) {
        G = gbytes ? shared_geom->p : nullptr;
        build_geom = shared_geom->build;
    } else if (gbytes) {
        G = cur.take<float2>(gbytes / sizeof(float2));
    }
    if (cur.off > cur.cap) return IA_ERR_ALLOC;
    // A^T and B^T arrive as double-float pairs (float4, the size of double2)
    float4 *At4 = reinterpret_cast<float4 *>(At), *Bt4 = reinterpret_cast<float4 *>(Bt);
    int st;
    {
        NvtxRange r("ia.assembly");
        st = ibem_rows(ctx, mesh, l, d_mics, 0, nullptr, F, d_k, cfg->c, cfg->rho, At, Bt, Ahs_t, Ht, true, true, G,
                       build_geom);
    }
    if (st) return st;
    if (ev_rows) IA_CUDA_TRY(cudaEventRecord(ev_rows, ctx->stream));
    NvtxRange r("ia.transfer");
    const long long sMM = (long long)m * m, sML = (long long)m * l;
    if ((st = df_hi_batched(ctx, (size_t)sMM * F, At4, M32))) return st;
    if ((st = getrf_batched<float2>(ctx, m, M32, m, sMM, ipiv, d_info, F))) return st;
    if ((st = copy2d_batched<double2, float2>(ctx, m, l, Ahs_t, m, sML, Y32, m, sML, false, F))) return st;
    if ((st = getrs_batched<float2>(ctx, m, l, M32, m, sMM, ipiv, Y32, m, sML, F))) return st;
    if ((st = copy2d_batched<float2, double2>(ctx, m, l, Y32, m, sML, Y, m, sML, false, F))) return st;
    // tensor-core products: slice planes of the m x m operand (M, later B^T,
    // in one region) and of Y
    const bool tcg = tc_products(cfg, m);
    const int S = cfg->gemm_slices;
    TcPlanes Pm{}, Py{};
    WsCursor cm{nullptr, 0, 0}, cy{nullptr, 0, 0};
    if (tcg) {
        const size_t bm = tc_planes_bytes(m, m, S, false, F), by = tc_planes_bytes(l, m, S, true, F);
        cm = WsCursor{(char *)cur.take<unsigned char>(bm), 0, bm};
        cy = WsCursor{(char *)cur.take<unsigned char>(by), 0, by};
        if (cur.off > cur.cap) return IA_ERR_ALLOC;
        if (cfg->refine_steps > 0 &&
            (st = tc_slice(ctx, false, OP_N, At4, m, sMM, m, m, S, F, Pm, cm)))
            return st;
    }
    for (int it = 0; it < cfg->refine_steps; ++it) {
        if ((st = zcopy2d_batched(ctx, m, l, Ahs_t, m, sML, R, m, sML, false, F))) return st;
        if (tcg) {
            cy.off = 0;
            if ((st = tc_slice(ctx, true, OP_N, Y, m, sML, l, m, S, F, Py, cy))) return st;
            if ((st = tc_gemm(ctx, Pm, Py, m, l, -1.0, 1.0, R, m, sML, F, d_info))) return st;
        } else {
            if ((st = split_df_batched(ctx, (size_t)sML * F, Y, Y4))) return st;
            if ((st = dfgemm4_batched(ctx, OP_N, OP_N, m, l, m, -1.0, At4, m, sMM, Y4, m, sML, 1.0, R, m, sML, F)))
                return st;
        }
        if ((st = copy2d_batched<double2, float2>(ctx, m, l, R, m, sML, Y32, m, sML, false, F))) return st;
        if ((st = getrs_batched<float2>(ctx, m, l, M32, m, sMM, ipiv, Y32, m, sML, F))) return st;
        if ((st = add2d_batched<float2>(ctx, m, l, Y32, m, sML, Y, m, sML, F))) return st;
    }
    if (tcg) {
        cm.off = 0;
        cy.off = 0;
        if ((st = tc_slice(ctx, false, OP_N, Bt4, m, sMM, m, m, S, F, Pm, cm))) return st;
        if ((st = tc_slice(ctx, true, OP_N, Y, m, sML, l, m, S, F, Py, cy))) return st;
        return tc_gemm(ctx, Pm, Py, m, l, 1.0, -1.0, Ht, m, sML, F, d_info);
    }
    if ((st = split_df_batched(ctx, (size_t)sML * F, Y, Y4))) return st;
    return dfgemm4_batched(ctx, OP_N, OP_N, m, l, m, 1.0, Bt4, m, sMM, Y4, m, sML, -1.0, Ht, m, sML, F);
}

int ia_ibem_transfer_batch(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int F,
                           const double *d_k, const ia_config *cfg, ia_complex *d_H, int *d_info)
{
    if (!ctx || !mesh || !cfg || F < 1 || l < 1 || !d_mics || !d_k || !d_H || !d_info) return IA_ERR_ARG;
    const int m = mesh->m;
    const bool mixed = cfg->precision == IA_PREC_MIXED;
    size_t need = ws_round(sizeof(double2) * (size_t)m * m * F) * 2 + ws_round(sizeof(int) * (size_t)m * F) +
                  ws_round(sizeof(double2) * (size_t)m * l * F) * 2 + (mixed ? transfer_mixed_ws_bytes(mesh, l, F, cfg) : 0);
    int st = ws_reserve(ctx, need);
    if (!st) st = clear_info(ctx, d_info, F);
    if (st) return st;
    WsCursor cur{(char *)ctx->ws, 0, ctx->ws_bytes};
    double2 *At = cur.take<double2>((size_t)m * m * F);
    double2 *Bt = cur.take<double2>((size_t)m * m * F);
    int *ipiv = cur.take<int>((size_t)m * F);
    double2 *Ahs = cur.take<double2>((size_t)m * l * F);
    double2 *Ht = cur.take<double2>((size_t)m * l * F);
    if (mixed) st = ibem_transfer_t_mixed(ctx, mesh, l, d_mics, F, d_k, cfg, At, Bt, ipiv, Ahs, Ht, d_info, cur);
    else st = ibem_transfer_t(ctx, mesh, l, d_mics, F, d_k, cfg, At, Bt, ipiv, Ahs, Ht, d_info);
    if (st) return st;
    return ztranspose_batched(ctx, m, l, Ht, m, (long long)m * l, (double2 *)d_H, l, (long long)m * l, false, F);
}

int ia_hels_batch(ia_context *ctx, int l, const double *d_pts, int n_sh, int F, const double *d_k, ia_complex *d_H)
{
    if (!ctx || l < 1 || !d_pts || n_sh < 0 || F < 1 || !d_k || !d_H) return IA_ERR_ARG;
    return hels_batched(ctx, l, d_pts, n_sh, F, d_k, 343.0, 1.21, (double2 *)d_H, nullptr);
}

int ia_svd_batch(ia_context *ctx, int m, int n, int F, const ia_complex *d_A, ia_complex *d_U, double *d_s,
                 ia_complex *d_V, int *d_info)
{
    if (!ctx || m < 1 || n < 1 || F < 1 || !d_A || !d_s || !d_info) return IA_ERR_ARG;
    int st = ws_reserve(ctx, svd_workspace_bytes(m, n, F));
    if (!st) st = clear_info(ctx, d_info, F);
    if (st) return st;
    const int M = m >= n ? m : n, N = m >= n ? n : m;
    WsCursor cur{(char *)ctx->ws, 0, ctx->ws_bytes};
    double2 *Y = cur.take<double2>((size_t)M * N * F);
    double2 *Vacc = cur.take<double2>((size_t)N * N * F);
    return svd_batched(ctx, m, n, (const double2 *)d_A, false, (double2 *)d_U, d_s, (double2 *)d_V, F, 40, d_info,
                       Y, Vacc);
}

int ia_regularize_batch(ia_context *ctx, int m, int n, int F, const ia_complex *d_U, const double *d_s,
                        const ia_complex *d_V, int nrhs, const ia_complex *d_b, const ia_config *cfg,
                        ia_complex *d_x, double *d_lambda)
{
    if (!ctx || !cfg || m < 1 || n < 1 || F < 1 || nrhs < 1 || !d_U || !d_s || !d_V || !d_b || !d_x) return IA_ERR_ARG;
    const int p = m < n ? m : n;
    return regularize_batched(ctx, m, n, p, F, (const double2 *)d_U, d_s, (const double2 *)d_V, nrhs,
                              (const double2 *)d_b, cfg, (double2 *)d_x, d_lambda);
}

// SVD + regularisation on an operator given as A (m x n) or its transpose.
// The mixed wide solve rebuilds x in data space, x = H^H U diag(phi / s) beta,
// which needs s only where phi / s stays small for unresolved s (Tikhonov,
// TSVD).  The damped SVD weights every component by 1/(s + lambda), so it
// takes the FP64 wide solve in both precisions.
static bool use_mixed_wide(int m, int n, const ia_config *cfg)
{
    const bool damped = cfg->method == IA_METHOD_DSVD_FIXED || cfg->method == IA_METHOD_DSVD_LCURVE ||
                        cfg->method == IA_METHOD_DSVD_QUASIOPT;
    return m <= n && cfg->precision == IA_PREC_MIXED && !damped;
}

static int solve_core(ia_context *ctx, int m, int n, int F, const double2 *A, bool transposed, int nrhs,
                      const double2 *b, const ia_config *cfg, double2 *x, double *lambda, double *s_out, int *info,
                      WsCursor &cur)
{
    NvtxRange r("ia.solve");
    if (use_mixed_wide(m, n, cfg))
        return wide_solve_mixed_batched(ctx, m, n, F, A, transposed, nrhs, b, cfg, x, lambda, s_out, info, cur);
    if (m <= n) return wide_solve_batched(ctx, m, n, F, A, transposed, nrhs, b, cfg, x, lambda, s_out, info, cur);
    const int p = m < n ? m : n;
    const int M = m >= n ? m : n;
    double2 *Y = cur.take<double2>((size_t)M * p * F);
    double2 *Vacc = cur.take<double2>((size_t)p * p * F);
    double2 *U = cur.take<double2>((size_t)m * p * F);
    double2 *V = cur.take<double2>((size_t)n * p * F);
    double *s = s_out ? s_out : cur.take<double>((size_t)p * F);
    int st = svd_batched(ctx, m, n, A, transposed, U, s, V, F, cfg->svd_max_sweeps, info, Y, Vacc);
    if (st) return st;
    return regularize_batched(ctx, m, n, p, F, U, s, V, nrhs, b, cfg, x, lambda);
}

// ---- FP64 fallback of mixed solves ----------------------------------------
// A per-bin array of an entry point: bin f's data at base + f * bytes
// (base null: the caller did not ask for that output).
struct BinSpan {
    const void *base;
    size_t bytes;
};

// gather (dst bin j <- src bin idx[j]) or scatter (dst bin idx[j] <- src bin
// j) of Fb bins of `words` 32-bit words each; grid.y runs over the bins
__global__ void move_bins_kernel(const uint32_t *__restrict__ src, uint32_t *__restrict__ dst, size_t words,
                                 const int *__restrict__ idx, int scatter)
{
    const int j = blockIdx.y;
    const size_t so = (size_t)(scatter ? j : idx[j]) * words, d0 = (size_t)(scatter ? idx[j] : j) * words;
    for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < words; w += (size_t)gridDim.x * blockDim.x)
        dst[d0 + w] = src[so + w];
}

static int move_bins(ia_context *ctx, const void *src, void *dst, size_t bytes, const int *d_idx, int Fb,
                     bool scatter)
{
    const size_t words = bytes / 4;
    int blocks = (int)((words + 255) / 256);
    if (blocks > 64) blocks = 64;
    move_bins_kernel<<<dim3(blocks, Fb), 256, 0, ctx->stream>>>((const uint32_t *)src, (uint32_t *)dst, words, d_idx,
                                                                scatter ? 1 : 0);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// redo(Fb, in, out, info, cfg): the entry point with cfg on Fb compact bins
using RedoFn = std::function<int(int, void *const *, void *const *, int *, const ia_config *)>;

// The bins idx of a finished batched call, solved again with rc on compact
// copies of their per-bin inputs; the outputs and info words replace the
// first attempt's.  The index list and compact copies live in one
// stream-ordered allocation released before the function returns.
static int redo_bins(ia_context *ctx, const std::vector<int> &idx, int *d_info, std::initializer_list<BinSpan> ins,
                     std::initializer_list<BinSpan> outs, const RedoFn &redo, const ia_config *rc)
{
    const int Fb = (int)idx.size();
    size_t bytes = 2 * ws_round(sizeof(int) * (size_t)Fb);
    for (const BinSpan &a : ins) bytes += ws_round(a.bytes * Fb);
    for (const BinSpan &a : outs) bytes += a.base ? ws_round(a.bytes * Fb) : 0;
    char *blk = nullptr;
    IA_CUDA_TRY(cudaMallocAsync((void **)&blk, bytes, ctx->stream));
    WsCursor cur{blk, 0, bytes};
    int *d_idx = cur.take<int>((size_t)Fb);
    int *c_info = cur.take<int>((size_t)Fb);
    std::vector<void *> cin, cout;
    int st = IA_OK;
    cudaError_t e = cudaMemcpyAsync(d_idx, idx.data(), sizeof(int) * (size_t)Fb, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) st = cuda_status(e);
    for (const BinSpan &a : ins) {
        void *c = cur.take<char>(a.bytes * Fb);
        cin.push_back(c);
        if (!st) st = move_bins(ctx, a.base, c, a.bytes, d_idx, Fb, false);
    }
    for (const BinSpan &a : outs) cout.push_back(a.base ? (void *)cur.take<char>(a.bytes * Fb) : nullptr);
    if (!st) st = redo(Fb, cin.data(), cout.data(), c_info, rc);
    size_t i = 0;
    for (const BinSpan &a : outs) {
        if (!st && a.base) st = move_bins(ctx, cout[i], const_cast<void *>(a.base), a.bytes, d_idx, Fb, true);
        ++i;
    }
    if (!st) st = move_bins(ctx, c_info, d_info, sizeof(int), d_idx, Fb, true);
    e = cudaFreeAsync(blk, ctx->stream);
    if (!st && e != cudaSuccess) st = cuda_status(e);
    // the index list's host copy must outlive its transfer
    e = cudaStreamSynchronize(ctx->stream);
    if (!st && e != cudaSuccess) st = cuda_status(e);
    return st;
}

// the configuration of the fallback solve: FP64, and the automatic part
// split (the caller's explicit split need not divide the fallback's bins)
static ia_config fp64_config(const ia_config *cfg)
{
    ia_config c = *cfg;
    c.precision = IA_PREC_FP64;
    c.pipeline_parts = 0;
    return c;
}

// eigen-refinement steps of the mixed retry
constexpr int MIXED_RETRY_STEPS = 3;

// After a batched solve issued on ctx->stream: with the mixed path and
// cfg->mixed_fallback, the bins whose info word is set are solved again.
// A bin flagged only IA_INFO_UNRESOLVED (its eigen-decomposition failed the
// trace check: Ogita-Aishima steps that did not settle, as on the symmetric
// plate array's near-degenerate pairs) first gets the mixed path once more
// with MIXED_RETRY_STEPS refinement steps (that call's own fallback takes
// what still fails to FP64); every other flagged bin (lambda below the mixed
// floor, solver flags) goes to the FP64 path directly.  One host
// synchronisation when nothing is flagged; nothing happens while the stream
// is capturing, where the flags stay for the caller.
static int fp64_fallback(ia_context *ctx, const ia_config *cfg, int F, int *d_info, std::initializer_list<BinSpan> ins,
                         std::initializer_list<BinSpan> outs, const RedoFn &redo)
{
    ctx->last_fallback = 0;
    if (cfg->precision != IA_PREC_MIXED || !cfg->mixed_fallback) return IA_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    IA_CUDA_TRY(cudaStreamIsCapturing(ctx->stream, &cs));
    if (cs != cudaStreamCaptureStatusNone || ctx->capturing) return IA_OK;
    std::vector<int> h((size_t)F);
    IA_CUDA_TRY(cudaMemcpyAsync(h.data(), d_info, sizeof(int) * (size_t)F, cudaMemcpyDeviceToHost, ctx->stream));
    IA_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    const bool can_retry = cfg->refine_steps < MIXED_RETRY_STEPS;
    std::vector<int> retry, fp64;
    for (int f = 0; f < F; ++f) {
        if (!h[f]) continue;
        if (can_retry && h[f] == IA_INFO_UNRESOLVED) retry.push_back(f);
        else fp64.push_back(f);
    }
    int st = IA_OK;
    if (!retry.empty()) {
        ia_config rc = *cfg;
        rc.refine_steps = MIXED_RETRY_STEPS;
        rc.pipeline_parts = 0;
        st = redo_bins(ctx, retry, d_info, ins, outs, redo, &rc);
    }
    if (!st && !fp64.empty()) {
        const ia_config rc = fp64_config(cfg);
        st = redo_bins(ctx, fp64, d_info, ins, outs, redo, &rc);
    }
    if (!st) ctx->last_fallback = (int)(retry.size() + fp64.size());
    return st;
}

static size_t solve_ws_bytes(int m, int n, int F, int nrhs, const ia_config *cfg)
{
    if (use_mixed_wide(m, n, cfg)) return wide_solve_mixed_ws_bytes(m, n, nrhs, F);
    if (m <= n) return wide_solve_ws_bytes(m, n, nrhs, F);
    const int p = m < n ? m : n;
    const int M = m >= n ? m : n;
    return ws_round(sizeof(double2) * (size_t)M * p * F) + ws_round(sizeof(double2) * (size_t)p * p * F) +
           ws_round(sizeof(double2) * (size_t)m * p * F) + ws_round(sizeof(double2) * (size_t)n * p * F) +
           ws_round(sizeof(double) * (size_t)p * F) + 1024;
}

int ia_solve_batch(ia_context *ctx, int m, int n, int F, const ia_complex *d_H, int nrhs, const ia_complex *d_b,
                   const ia_config *cfg, ia_complex *d_x, double *d_lambda, double *d_s, int *d_info)
{
    if (!ctx || !cfg || m < 1 || n < 1 || F < 1 || nrhs < 1 || !d_H || !d_b || !d_x || !d_info) return IA_ERR_ARG;
    int st = ws_reserve(ctx, solve_ws_bytes(m, n, F, nrhs, cfg));
    if (!st) st = clear_info(ctx, d_info, F);
    if (st) return st;
    WsCursor cur{(char *)ctx->ws, 0, ctx->ws_bytes};
    st = solve_core(ctx, m, n, F, (const double2 *)d_H, false, nrhs, (const double2 *)d_b, cfg, (double2 *)d_x,
                    d_lambda, d_s, d_info, cur);
    if (st) return st;
    const int p = m < n ? m : n;
    return fp64_fallback(
        ctx, cfg, F, d_info, {{d_H, 16 * (size_t)m * n}, {d_b, 16 * (size_t)nrhs * m}},
        {{d_x, 16 * (size_t)nrhs * n}, {d_lambda, 8 * (size_t)nrhs}, {d_s, 8 * (size_t)p}},
        [&](int Fb, void *const *in, void *const *out, int *info, const ia_config *rc) {
            return ia_solve_batch(ctx, m, n, Fb, (const ia_complex *)in[0], nrhs, (const ia_complex *)in[1], rc,
                                  (ia_complex *)out[0], (double *)out[1], (double *)out[2], info);
        });
}

static size_t ibem_solve_ws_bytes(const ia_mesh *mesh, int l, int F, int nrhs, const ia_config *cfg,
                                  bool with_table = true)
{
    const bool mixed = cfg->precision == IA_PREC_MIXED;
    const int m = mesh->m;
    return ws_round(sizeof(double2) * (size_t)m * m * F) * 2 + ws_round(sizeof(int) * (size_t)m * F) +
           ws_round(sizeof(double2) * (size_t)m * l * F) * 2 + solve_ws_bytes(l, m, F, nrhs, cfg) +
           (mixed ? transfer_mixed_ws_bytes(mesh, l, F, cfg, with_table) : 0);
}

// the whole IBEM pipeline for F bins on ctx->stream; ev_rows (if given) is
// recorded when the assembly has been issued
static int ibem_solve_part(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int F,
                           const double *d_k, int nrhs, const double2 *p, const ia_config *cfg, double2 *x,
                           double *lambda, double *s, int *info, WsCursor &cur, cudaEvent_t ev_rows,
                           const GeomTable *shared_geom = nullptr)
{
    const int m = mesh->m;
    double2 *At = cur.take<double2>((size_t)m * m * F);
    double2 *Bt = cur.take<double2>((size_t)m * m * F);
    int *ipiv = cur.take<int>((size_t)m * F);
    double2 *Ahs = cur.take<double2>((size_t)m * l * F);
    double2 *Ht = cur.take<double2>((size_t)m * l * F);
    int st;
    if (cfg->precision == IA_PREC_MIXED)
        st = ibem_transfer_t_mixed(ctx, mesh, l, d_mics, F, d_k, cfg, At, Bt, ipiv, Ahs, Ht, info, cur, ev_rows,
                                   shared_geom);
    else st = ibem_transfer_t(ctx, mesh, l, d_mics, F, d_k, cfg, At, Bt, ipiv, Ahs, Ht, info, ev_rows);
    if (st) return st;
    return solve_core(ctx, l, m, F, Ht, true, nrhs, p, cfg, x, lambda, s, info, cur);
}

int ia_ibem_solve_batch(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int F,
                        const double *d_k, int nrhs, const ia_complex *d_p, const ia_config *cfg, ia_complex *d_x,
                        double *d_lambda, double *d_s, int *d_info)
{
    if (!ctx || !mesh || !cfg || l < 1 || F < 1 || nrhs < 1 || !d_mics || !d_k || !d_p || !d_x || !d_info)
        return IA_ERR_ARG;
    const int m = mesh->m;
    // Staggered parts: the bins are solved as P parts (4 when F is a multiple
    // of 16 and at least 32, 2 when a multiple of 8 and at least 16), each on
    // its own stream, part q starting when part q-1's assembly is done.  So
    // the latency-bound stages of one part (LU panels, Jacobi, QR: one CTA
    // per frequency) run beside the throughput-bound stages of the others,
    // and only the last part's chain is left exposed at the end.  Each part
    // has its own workspace region; the mixed assembly's geometry table is
    // one region after them, written by the first part and read by all (a
    // part starts after the previous part's assembly).  Frequencies stay in the assembly's
    // blocks (4 bins in FP64, 1 in double-float; parts are multiples of 4)
    // and every later kernel works per frequency, so the results are bitwise
    // those of one F-bin pass.
    int parts = (F >= 32 && F % 16 == 0) ? 4 : (F >= 16 && F % 8 == 0) ? 2 : 1;
    if (cfg->pipeline_parts) {
        parts = cfg->pipeline_parts;
        if (parts < 1 || parts > IA_SPLIT_PARTS || F % parts || (parts > 1 && (F / parts) % 4)) return IA_ERR_ARG;
    }
    const int Fp = F / parts;
    const size_t need = ibem_solve_ws_bytes(mesh, l, Fp, nrhs, cfg, parts == 1);
    const size_t gshared = parts > 1 && cfg->precision == IA_PREC_MIXED ? ibem_geom_bytes(mesh, m + l) : 0;
    const size_t goff = ws_round(need * parts);
    int st = ws_reserve(ctx, goff + gshared);
    if (!st) st = clear_info(ctx, d_info, F);
    if (st) return st;
    const int p = l < m ? l : m;
    auto fallback = [&]() {
        return fp64_fallback(
            ctx, cfg, F, d_info, {{d_k, sizeof(double)}, {d_p, 16 * (size_t)nrhs * l}},
            {{d_x, 16 * (size_t)nrhs * m}, {d_lambda, 8 * (size_t)nrhs}, {d_s, 8 * (size_t)p}},
            [&](int Fb, void *const *in, void *const *out, int *info, const ia_config *rc) {
                return ia_ibem_solve_batch(ctx, mesh, l, d_mics, Fb, (const double *)in[0], nrhs,
                                           (const ia_complex *)in[1], rc, (ia_complex *)out[0], (double *)out[1],
                                           (double *)out[2], info);
            });
    };
    if (parts == 1) {
        WsCursor cur{(char *)ctx->ws, 0, ctx->ws_bytes};
        st = ibem_solve_part(ctx, mesh, l, d_mics, F, d_k, nrhs, (const double2 *)d_p, cfg, (double2 *)d_x, d_lambda,
                             d_s, d_info, cur, nullptr);
        return st ? st : fallback();
    }
    if ((st = ensure_side_stream(ctx))) return st;
    cudaStream_t main = ctx->stream;
    // fork: every part runs on its own stream, after the work already queued
    // on the caller's stream
    cudaError_t e = cudaEventRecord(ctx->ev_fork, main);
    int q = 0;
    for (; q < parts && !st && e == cudaSuccess; ++q) {
        const int f0 = q * Fp;
        cudaStream_t sq = ctx->side[q];
        if ((e = cudaStreamWaitEvent(sq, q == 0 ? ctx->ev_fork : ctx->ev_rows[q - 1], 0)) != cudaSuccess) break;
        ctx->stream = sq;
        ctx->tail_part = q + 1 == parts;
        WsCursor cur{(char *)ctx->ws + need * q, 0, need};
        const GeomTable geom{reinterpret_cast<float2 *>((char *)ctx->ws + goff), q == 0};
        st = ibem_solve_part(ctx, mesh, l, d_mics, Fp, d_k + f0, nrhs, (const double2 *)d_p + (size_t)f0 * nrhs * l,
                             cfg, (double2 *)d_x + (size_t)f0 * nrhs * m,
                             d_lambda ? d_lambda + (size_t)f0 * nrhs : nullptr, d_s ? d_s + (size_t)f0 * p : nullptr,
                             d_info + f0, cur, q + 1 < parts ? ctx->ev_rows[q] : nullptr, &geom);
        ctx->stream = main;
        ctx->tail_part = 0;
        if (!st && cur.off > need) st = IA_ERR_ALLOC;   // workspace accounting broken: the parts would overlap
    }
    // join every started part's stream back into the caller's stream
    for (int j = 0; j < q; ++j) {
        cudaError_t ej = cudaEventRecord(ctx->ev_done[j], ctx->side[j]);
        if (ej == cudaSuccess) ej = cudaStreamWaitEvent(main, ctx->ev_done[j], 0);
        if (e == cudaSuccess) e = ej;
    }
    if (st) return st;
    if (e != cudaSuccess) return cuda_status(e);
    return fallback();
}

int ia_esm_solve_batch(ia_context *ctx, int l, int m, const double *d_mics, const double *d_src, int F,
                       const double *d_k, int nrhs, const ia_complex *d_p, const ia_config *cfg, ia_complex *d_x,
                       double *d_lambda, double *d_s, int *d_info)
{
    if (!ctx || !cfg || l < 1 || m < 1 || F < 1 || nrhs < 1 || !d_mics || !d_src || !d_k || !d_p || !d_x || !d_info)
        return IA_ERR_ARG;
    size_t need = ws_round(sizeof(double2) * (size_t)l * m * F) + solve_ws_bytes(l, m, F, nrhs, cfg);
    int st = ws_reserve(ctx, need);
    if (!st) st = clear_info(ctx, d_info, F);
    if (st) return st;
    WsCursor cur{(char *)ctx->ws, 0, ctx->ws_bytes};
    double2 *G = cur.take<double2>((size_t)l * m * F);
    st = monopole_batched(ctx, l, m, F, d_mics, d_src, d_k, G);
    if (st) return st;
    st = solve_core(ctx, l, m, F, G, false, nrhs, (const double2 *)d_p, cfg, (double2 *)d_x, d_lambda, d_s, d_info,
                    cur);
    if (st) return st;
    const int p = l < m ? l : m;
    return fp64_fallback(
        ctx, cfg, F, d_info, {{d_k, sizeof(double)}, {d_p, 16 * (size_t)nrhs * l}},
        {{d_x, 16 * (size_t)nrhs * m}, {d_lambda, 8 * (size_t)nrhs}, {d_s, 8 * (size_t)p}},
        [&](int Fb, void *const *in, void *const *out, int *info, const ia_config *rc) {
            return ia_esm_solve_batch(ctx, l, m, d_mics, d_src, Fb, (const double *)in[0], nrhs,
                                      (const ia_complex *)in[1], rc, (ia_complex *)out[0], (double *)out[1],
                                      (double *)out[2], info);
        });
}

int ia_hels_solve_batch(ia_context *ctx, int l, const double *d_pts, int n_sh, int F, const double *d_k, int nrhs,
                        const ia_complex *d_p, const ia_config *cfg, ia_complex *d_x, double *d_lambda,
                        double *d_s, int *d_info)
{
    if (!ctx || !cfg || l < 1 || n_sh < 0 || F < 1 || nrhs < 1 || !d_pts || !d_k || !d_p || !d_x || !d_info)
        return IA_ERR_ARG;
    const int nt = (n_sh + 1) * (n_sh + 1);
    size_t need = ws_round(sizeof(double2) * (size_t)l * nt * F) + solve_ws_bytes(l, nt, F, nrhs, cfg);
    int st = ws_reserve(ctx, need);
    if (!st) st = clear_info(ctx, d_info, F);
    if (st) return st;
    WsCursor cur{(char *)ctx->ws, 0, ctx->ws_bytes};
    double2 *H = cur.take<double2>((size_t)l * nt * F);
    st = hels_batched(ctx, l, d_pts, n_sh, F, d_k, cfg->c, cfg->rho, H, nullptr);
    if (st) return st;
    st = solve_core(ctx, l, nt, F, H, false, nrhs, (const double2 *)d_p, cfg, (double2 *)d_x, d_lambda, d_s, d_info,
                    cur);
    if (st) return st;
    const int p = l < nt ? l : nt;
    return fp64_fallback(
        ctx, cfg, F, d_info, {{d_k, sizeof(double)}, {d_p, 16 * (size_t)nrhs * l}},
        {{d_x, 16 * (size_t)nrhs * nt}, {d_lambda, 8 * (size_t)nrhs}, {d_s, 8 * (size_t)p}},
        [&](int Fb, void *const *in, void *const *out, int *info, const ia_config *rc) {
            return ia_hels_solve_batch(ctx, l, d_pts, n_sh, Fb, (const double *)in[0], nrhs,
                                       (const ia_complex *)in[1], rc, (ia_complex *)out[0], (double *)out[1],
                                       (double *)out[2], info);
        });
}

int ia_sinc_resistance_batch(ia_context *ctx, int n, const double *d_x, int F, const double *d_k, double area,
                             const ia_config *cfg, double *d_R)
{
    if (!ctx || n < 1 || F < 1 || !d_x || !d_k || !d_R || !(area > 0.0)) return IA_ERR_ARG;
    ia_config dc;
    if (!cfg) { ia_config_default(&dc); cfg = &dc; }
    return sinc_resistance_batched(ctx, n, d_x, F, d_k, area, cfg->c, cfg->rho, d_R, nullptr);
}

int ia_radiation_modes_batch(ia_context *ctx, int n, int F, const double *d_R, int nmodes, const ia_config *cfg,
                             double *d_lambda, double *d_modes, int *d_info)
{
    if (!ctx || !cfg || n < 1 || F < 1 || nmodes < 1 || nmodes > n || !d_R || !d_lambda || !d_modes || !d_info ||
        cfg->mode_iters < 0 || cfg->mode_oversample < 0)
        return IA_ERR_ARG;
    int st = ws_reserve(ctx, radiation_modes_ws_bytes(n, F, nmodes, cfg));
    if (!st) st = clear_info(ctx, d_info, F);
    if (st) return st;
    WsCursor cur{(char *)ctx->ws, 0, ctx->ws_bytes};
    return radiation_modes_batched(ctx, n, F, d_R, nmodes, cfg, d_lambda, d_modes, d_info, cur);
}

int ia_esm_design_batch(ia_context *ctx, int l, int m, int F, int nrhs, const double *d_mics,
                        const double *d_surface, const double *d_retreat, const double *d_k, const double *d_loglam,
                        const ia_complex *d_q, const ia_complex *d_noise, double *d_err, double *d_grad_mics,
                        double *d_grad_retreat, double *d_grad_loglam, int *d_info)
{
    if (!ctx || l < 1 || m < l || F < 1 || nrhs < 1 || nrhs > 32 || !d_mics || !d_surface || !d_retreat || !d_k ||
        !d_loglam || !d_q || !d_err || !d_info)
        return IA_ERR_ARG;
    const int ng = (d_grad_mics != nullptr) + (d_grad_retreat != nullptr) + (d_grad_loglam != nullptr);
    if (ng != 0 && ng != 3) return IA_ERR_ARG;
    int st = ws_reserve(ctx, esm_design_ws_bytes(l, m, F, nrhs));
    if (!st) st = clear_info(ctx, d_info, F);
    if (st) return st;
    WsCursor cur{(char *)ctx->ws, 0, ctx->ws_bytes};
    return esm_design_batched(ctx, l, m, F, nrhs, d_mics, d_surface, d_retreat, d_k, d_loglam, (const double2 *)d_q,
                              (const double2 *)d_noise, d_err, d_grad_mics, d_grad_retreat, d_grad_loglam, d_info,
                              cur);
}

static int bem_modes_entry(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int n_ch,
                           const double *d_cp, int F, const double *d_k, int nmodes, const ia_config *cfg, bool cplx,
                           void *d_Ur, double *d_sr, ia_complex *d_Hr, ia_complex *d_Pr, int *d_info)
{
    if (!ctx || !mesh || !cfg || l < 1 || n_ch < 0 || (n_ch > 0 && !d_cp) || F < 1 || nmodes < 1 ||
        nmodes > mesh->m || !d_mics || !d_k || !d_Ur || !d_sr || !d_Hr || !d_info || cfg->mode_iters < 0 ||
        cfg->mode_oversample < 0)
        return IA_ERR_ARG;
    int st = ws_reserve(ctx, bem_modes_ws_bytes(mesh, l, n_ch, F, nmodes, cfg, cplx));
    if (!st) st = clear_info(ctx, d_info, F);
    if (st) return st;
    WsCursor cur{(char *)ctx->ws, 0, ctx->ws_bytes};
    return bem_modes_batched(ctx, mesh, l, d_mics, n_ch, d_cp, F, d_k, nmodes, cfg, cplx, d_Ur, d_sr,
                             (double2 *)d_Hr, (double2 *)d_Pr, d_info, cur);
}

int ia_bem_modes_batch(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int n_ch,
                       const double *d_cp, int F, const double *d_k, int nmodes, const ia_config *cfg, double *d_Ur,
                       double *d_sr, ia_complex *d_Hr, ia_complex *d_Pr, int *d_info)
{
    return bem_modes_entry(ctx, mesh, l, d_mics, n_ch, d_cp, F, d_k, nmodes, cfg, false, d_Ur, d_sr, d_Hr, d_Pr,
                           d_info);
}

int ia_bem_modes_complex_batch(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int n_ch,
                               const double *d_cp, int F, const double *d_k, int nmodes, const ia_config *cfg,
                               ia_complex *d_Ur, double *d_sr, ia_complex *d_Hr, ia_complex *d_Pr, int *d_info)
{
    return bem_modes_entry(ctx, mesh, l, d_mics, n_ch, d_cp, F, d_k, nmodes, cfg, true, d_Ur, d_sr, d_Hr, d_Pr,
                           d_info);
}

int ia_admm_batch(ia_context *ctx, int l, int m, int F, const ia_complex *d_H, int nrhs, const ia_complex *d_p,
                  const double *d_lambda0, const ia_admm_config *acfg, const ia_complex *d_x0, ia_complex *d_c,
                  int *d_iters, int *d_info)
{
    if (!ctx || !acfg || l < 1 || m < 1 || F < 1 || nrhs < 1 || !d_H || !d_p || !d_lambda0 || !d_c || !d_info)
        return IA_ERR_ARG;
    if (acfg->norm < IA_ADMM_L1 || acfg->norm > IA_ADMM_LP || acfg->max_iters < 0 || !(acfg->rho > 0.0) ||
        !isfinite(acfg->rho) || !isfinite(acfg->gamma) || !(acfg->epsilon >= 0.0))
        return IA_ERR_ARG;
    if (acfg->norm == IA_ADMM_LP && (!(acfg->p > 0.0 && acfg->p <= 1.0) || acfg->gst_iters < 0)) return IA_ERR_ARG;
    if (acfg->precision != IA_PREC_FP64 && acfg->precision != IA_PREC_MIXED) return IA_ERR_ARG;
    int st = ws_reserve(ctx, admm_ws_bytes(l, m, F, nrhs));
    if (!st) st = clear_info(ctx, d_info, F);
    if (st) return st;
    WsCursor cur{(char *)ctx->ws, 0, ctx->ws_bytes};
    return admm_batched(ctx, l, m, F, (const double2 *)d_H, nrhs, (const double2 *)d_p, d_lambda0, acfg,
                        (const double2 *)d_x0, (double2 *)d_c, d_iters, d_info, cur);
}

int ia_sound_power_batch(ia_context *ctx, int n, int F, const double *d_R, int nrhs, const ia_complex *d_v,
                         double *d_W)
{
    if (!ctx || n < 1 || F < 1 || nrhs < 1 || !d_R || !d_v || !d_W) return IA_ERR_ARG;
    int st = ws_reserve(ctx, sound_power_ws_bytes(n, F));
    if (st) return st;
    WsCursor cur{(char *)ctx->ws, 0, ctx->ws_bytes};
    return sound_power_batched(ctx, n, F, d_R, nrhs, (const double2 *)d_v, d_W, cur);
}

}  // extern "C"

// ---- reference-compatible host entry points -------------------------------
// Device scratch for one compat call: a single cudaMallocAsync block on the
// compat context's stream, released at the end of the call.
struct CompatScratch {
    ia_context *ctx;
    char *base = nullptr;
    size_t off = 0, cap = 0;
    int alloc(size_t bytes)
    {
        cap = bytes;
        cudaError_t e = cudaMallocAsync((void **)&base, bytes, ctx->stream);
        return e == cudaSuccess ? IA_OK : cuda_status(e);
    }
    template <class T>
    T *take(size_t count)
    {
        size_t a = (off + 255) & ~size_t(255);
        off = a + count * sizeof(T);
        return reinterpret_cast<T *>(base + a);
    }
    ~CompatScratch()
    {
        if (base) {
            cudaFreeAsync(base, ctx->stream);
            cudaStreamSynchronize(ctx->stream);
        }
    }
};

#define IA_TRY(x)                \
    do {                         \
        int r__ = (x);           \
        if (r__) return r__;     \
    } while (0)
#define IA_CTRY(x) IA_CUDA_TRY(x)

extern "C" {

int ia_esm(int m, int l, const double *r_ms, const double *r_lh, ia_complex **m_e, ia_complex **h, double k,
           double r_i, const ia_config *cfg)
{
    if (m < 1 || l < 1 || !r_ms || !r_lh || !m_e || !h || !(k > 0.0)) return IA_ERR_ARG;
    if (!all_finite(r_ms, 3 * (size_t)m) || !all_finite(r_lh, 3 * (size_t)l) || !isfinite(r_i)) return IA_ERR_NONFINITE;
    ia_config dc;
    if (!cfg) { ia_config_default(&dc); cfg = &dc; }
    std::lock_guard<std::mutex> lk(g_compat_mu);
    int st;
    ia_context *ctx = compat_context(&st);
    if (!ctx) return st;
    CompatScratch sc{ctx};
    size_t need = ws_round(24 * (size_t)(m + l)) + ws_round(16 * (size_t)m * m) + ws_round(16 * (size_t)m * (m + l)) +
                  ws_round(16 * (size_t)m * (m + l)) + ws_round(4 * (size_t)m) + ws_round(4) + 4096;
    IA_TRY(sc.alloc(need));
    double *dr = sc.take<double>(3 * (size_t)m);
    double *dl = sc.take<double>(3 * (size_t)l);
    double2 *DT = sc.take<double2>((size_t)m * m);
    double2 *RHS = sc.take<double2>((size_t)m * (m + l));
    double2 *OUT = sc.take<double2>((size_t)m * (m + l));
    int *ipiv = sc.take<int>(m);
    int *info = sc.take<int>(1);
    IA_CTRY(cudaMemcpyAsync(dr, r_ms, 24 * (size_t)m, cudaMemcpyHostToDevice, ctx->stream));
    IA_CTRY(cudaMemcpyAsync(dl, r_lh, 24 * (size_t)l, cudaMemcpyHostToDevice, ctx->stream));
    IA_CTRY(cudaMemsetAsync(info, 0, 4, ctx->stream));
    IA_TRY(esm_system(ctx, m, l, dr, dl, r_i, k, cfg->c, cfg->rho, DT, RHS));
    IA_TRY(zgetrf_batched(ctx, m, DT, m, 0, ipiv, info, 1));
    IA_TRY(zgetrs_batched(ctx, m, m + l, DT, m, 0, ipiv, RHS, m, 0, 1));
    // Me = X[:, :m]^T, He = X[:, m:]^T
    IA_TRY(ztranspose_batched(ctx, m, m, RHS, m, 0, OUT, m, 0, false, 1));
    IA_TRY(ztranspose_batched(ctx, m, l, RHS + (size_t)m * m, m, 0, OUT + (size_t)m * m, l, 0, false, 1));
    int hinfo = 0;
    IA_CTRY(cudaMemcpyAsync(&hinfo, info, 4, cudaMemcpyDeviceToHost, ctx->stream));
    ia_complex *me = nullptr, *he = nullptr;
    IA_TRY(to_host_malloc(ctx, (const ia_complex *)OUT, (size_t)m * m, &me));
    int r = to_host_malloc(ctx, (const ia_complex *)(OUT + (size_t)m * m), (size_t)l * m, &he);
    if (r) { free(me); return r; }
    *m_e = me;
    *h = he;
    if (hinfo & IA_INFO_NONFINITE) return IA_ERR_NONFINITE;
    if (hinfo & IA_INFO_SINGULAR) return IA_ERR_SINGULAR;
    return IA_OK;
}

int ia_hels(int m, int l, const double *r_ms_s, const double *r_lh_s, ia_complex **m_e, ia_complex **h,
            ia_complex **q_e, double k, int n_sh, const ia_config *cfg)
{
    if (m < 1 || l < 1 || !r_ms_s || !r_lh_s || !m_e || !h || !q_e || !(k > 0.0) || n_sh < 0) return IA_ERR_ARG;
    if (!all_finite(r_ms_s, 3 * (size_t)m) || !all_finite(r_lh_s, 3 * (size_t)l)) return IA_ERR_NONFINITE;
    ia_config dc;
    if (!cfg) { ia_config_default(&dc); cfg = &dc; }
    std::lock_guard<std::mutex> lk(g_compat_mu);
    int st;
    ia_context *ctx = compat_context(&st);
    if (!ctx) return st;
    const int nt = (n_sh + 1) * (n_sh + 1);
    CompatScratch sc{ctx};
    IA_TRY(sc.alloc(ws_round(24 * (size_t)(m + l)) + ws_round(8) + 3 * ws_round(16 * (size_t)nt * (m > l ? m : l)) +
                    4096));
    double *dr = sc.take<double>(3 * (size_t)m);
    double *dl = sc.take<double>(3 * (size_t)l);
    double *dk = sc.take<double>(1);
    double2 *Me = sc.take<double2>((size_t)m * nt);
    double2 *Qe = sc.take<double2>((size_t)m * nt);
    double2 *He = sc.take<double2>((size_t)l * nt);
    IA_CTRY(cudaMemcpyAsync(dr, r_ms_s, 24 * (size_t)m, cudaMemcpyHostToDevice, ctx->stream));
    IA_CTRY(cudaMemcpyAsync(dl, r_lh_s, 24 * (size_t)l, cudaMemcpyHostToDevice, ctx->stream));
    IA_CTRY(cudaMemcpyAsync(dk, &k, 8, cudaMemcpyHostToDevice, ctx->stream));
    IA_TRY(hels_batched(ctx, m, dr, n_sh, 1, dk, cfg->c, cfg->rho, Me, Qe));
    IA_TRY(hels_batched(ctx, l, dl, n_sh, 1, dk, cfg->c, cfg->rho, He, nullptr));
    ia_complex *a = nullptr, *b = nullptr, *c = nullptr;
    IA_TRY(to_host_malloc(ctx, (const ia_complex *)Me, (size_t)m * nt, &a));
    int r = to_host_malloc(ctx, (const ia_complex *)He, (size_t)l * nt, &b);
    if (!r) r = to_host_malloc(ctx, (const ia_complex *)Qe, (size_t)m * nt, &c);
    if (r) { free(a); free(b); return r; }
    *m_e = a;
    *h = b;
    *q_e = c;
    return IA_OK;
}

int ia_csvd(int m, int n, const ia_complex *a, ia_complex **u, double **s, ia_complex **v)
{
    if (m < 1 || n < 1 || !a || !u || !s || !v) return IA_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_compat_mu);
    int st;
    ia_context *ctx = compat_context(&st);
    if (!ctx) return st;
    const int p = m < n ? m : n, M = m > n ? m : n;
    CompatScratch sc{ctx};
    IA_TRY(sc.alloc(ws_round(16 * (size_t)m * n) + ws_round(16 * (size_t)M * p) + ws_round(16 * (size_t)p * p) +
                    ws_round(16 * (size_t)m * p) + ws_round(16 * (size_t)n * p) + ws_round(8 * (size_t)p) + 4096));
    double2 *A = sc.take<double2>((size_t)m * n);
    double2 *Y = sc.take<double2>((size_t)M * p);
    double2 *Vacc = sc.take<double2>((size_t)p * p);
    double2 *U = sc.take<double2>((size_t)m * p);
    double2 *V = sc.take<double2>((size_t)n * p);
    double *S = sc.take<double>(p);
    int *info = sc.take<int>(1);
    IA_CTRY(cudaMemcpyAsync(A, a, 16 * (size_t)m * n, cudaMemcpyHostToDevice, ctx->stream));
    IA_CTRY(cudaMemsetAsync(info, 0, 4, ctx->stream));
    IA_TRY(svd_batched(ctx, m, n, A, false, U, S, V, 1, 60, info, Y, Vacc));
    int hinfo = 0;
    IA_CTRY(cudaMemcpyAsync(&hinfo, info, 4, cudaMemcpyDeviceToHost, ctx->stream));
    ia_complex *hu = nullptr, *hv = nullptr;
    double *hs = nullptr;
    IA_TRY(to_host_malloc(ctx, (const ia_complex *)U, (size_t)m * p, &hu));
    int r = to_host_malloc(ctx, (const ia_complex *)V, (size_t)n * p, &hv);
    if (!r) r = to_host_malloc(ctx, S, (size_t)p, &hs);
    if (r) { free(hu); free(hv); return r; }
    *u = hu;
    *v = hv;
    *s = hs;
    if (hinfo & IA_INFO_NONFINITE) return IA_ERR_NONFINITE;
    if (hinfo & IA_INFO_NOCONV) return IA_ERR_NOCONV;
    return IA_OK;
}

int ia_tsvd(int m, int n, int p, int k, const ia_complex *u, const double *s, const ia_complex *v,
            const ia_complex *b, ia_complex **x)
{
    if (m < 1 || n < 1 || p < 1 || !u || !s || !v || !b || !x) return IA_ERR_ARG;
    if (k < 1 || k > p) return IA_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_compat_mu);
    int st;
    ia_context *ctx = compat_context(&st);
    if (!ctx) return st;
    CompatScratch sc{ctx};
    IA_TRY(sc.alloc(ws_round(16 * (size_t)m * p) + ws_round(8 * (size_t)p) + ws_round(16 * (size_t)n * p) +
                    ws_round(16 * (size_t)m) + ws_round(16 * (size_t)n) + 4096));
    double2 *U = sc.take<double2>((size_t)m * p);
    double *S = sc.take<double>(p);
    double2 *V = sc.take<double2>((size_t)n * p);
    double2 *B = sc.take<double2>(m);
    double2 *X = sc.take<double2>(n);
    IA_CTRY(cudaMemcpyAsync(U, u, 16 * (size_t)m * p, cudaMemcpyHostToDevice, ctx->stream));
    IA_CTRY(cudaMemcpyAsync(S, s, 8 * (size_t)p, cudaMemcpyHostToDevice, ctx->stream));
    // the reference copies only the first k columns of V (CUDA/tsvd.cuh:143-144)
    IA_CTRY(cudaMemsetAsync(V, 0, 16 * (size_t)n * p, ctx->stream));
    IA_CTRY(cudaMemcpyAsync(V, v, 16 * (size_t)n * k, cudaMemcpyHostToDevice, ctx->stream));
    IA_CTRY(cudaMemcpyAsync(B, b, 16 * (size_t)m, cudaMemcpyHostToDevice, ctx->stream));
    ia_config cfg;
    ia_config_default(&cfg);
    cfg.method = IA_METHOD_TSVD;
    cfg.tsvd_k = k;
    IA_TRY(regularize_batched(ctx, m, n, p, 1, U, S, V, 1, B, &cfg, X, nullptr));
    return to_host_malloc(ctx, (const ia_complex *)X, (size_t)n, x);
}

static int matvec_compat(int m, int n, const ia_complex *a, const ia_complex *x, ia_complex **y)
{
    if (m < 1 || n < 1 || !a || !x || !y) return IA_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_compat_mu);
    int st;
    ia_context *ctx = compat_context(&st);
    if (!ctx) return st;
    CompatScratch sc{ctx};
    IA_TRY(sc.alloc(ws_round(16 * (size_t)m * n) + ws_round(16 * (size_t)n) + ws_round(16 * (size_t)m) + 1024));
    double2 *A = sc.take<double2>((size_t)m * n);
    double2 *X = sc.take<double2>(n);
    double2 *Y = sc.take<double2>(m);
    IA_CTRY(cudaMemcpyAsync(A, a, 16 * (size_t)m * n, cudaMemcpyHostToDevice, ctx->stream));
    IA_CTRY(cudaMemcpyAsync(X, x, 16 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
    IA_TRY(zgemm_batched(ctx, OP_N, OP_N, m, 1, n, make_double2(1.0, 0.0), A, m, 0, X, n, 0, make_double2(0.0, 0.0), Y,
                         m, 0, 1));
    return to_host_malloc(ctx, (const ia_complex *)Y, (size_t)m, y);
}

int ia_to_pressure(int m, int n, const ia_complex *me, const ia_complex *x, ia_complex **p)
{
    return matvec_compat(m, n, me, x, p);
}

int ia_to_velocity(int m, int n, const ia_complex *qe, const ia_complex *x, ia_complex **v)
{
    return matvec_compat(m, n, qe, x, v);
}

int ia_sound_power(int m, const ia_complex *p, const ia_complex *v, double *w, double s)
{
    if (m < 1 || !p || !v || !w) return IA_ERR_ARG;
    std::lock_guard<std::mutex> lk(g_compat_mu);
    int st;
    ia_context *ctx = compat_context(&st);
    if (!ctx) return st;
    CompatScratch sc{ctx};
    IA_TRY(sc.alloc(ws_round(16 * (size_t)m) * 2 + ws_round(16) + 1024));
    double2 *P = sc.take<double2>(m);
    double2 *Vv = sc.take<double2>(m);
    double2 *D = sc.take<double2>(1);
    IA_CTRY(cudaMemcpyAsync(P, p, 16 * (size_t)m, cudaMemcpyHostToDevice, ctx->stream));
    IA_CTRY(cudaMemcpyAsync(Vv, v, 16 * (size_t)m, cudaMemcpyHostToDevice, ctx->stream));
    // v^H p as a 1 x 1 product
    IA_TRY(zgemm_batched(ctx, OP_C, OP_N, 1, 1, m, make_double2(1.0, 0.0), Vv, m, 0, P, m, 0, make_double2(0.0, 0.0), D,
                         1, 0, 1));
    double2 hd;
    IA_CTRY(cudaMemcpyAsync(&hd, D, 16, cudaMemcpyDeviceToHost, ctx->stream));
    IA_CTRY(cudaStreamSynchronize(ctx->stream));
    *w = 0.5 * hd.x * (s / m);
    return IA_OK;
}

}  // extern "C"
