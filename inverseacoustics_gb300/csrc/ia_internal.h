// Internal declarations shared by the libia.so translation units.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stddef.h>
#include <stdint.h>
#include "../../include/ia.h"

// staggered parts of a large IBEM batch, one stream each: at most
// IA_SPLIT_PARTS (ia_config.pipeline_parts), 4 by default for F >= 32
#define IA_SPLIT_PARTS 8

struct ia_context {
    int device;
    cudaStream_t stream;
    void *ws;              // stream-ordered workspace (grow-only)
    size_t ws_bytes;
    long long launches;    // kernels launched through this context
    int sm_count;
    int capturing;         // between ia_capture_begin and ia_capture_end
    int no_tune;           // the autotuner may not time variants (allocation-free calls)
    int last_fallback;     // bins the last batched solve recomputed in FP64 (mixed_fallback)
    int tail_part;         // the last part of a staggered pipeline is running (its chain ends the pass:
                           // latency-bound stages may take more SMs per bin)
    int *dcount;           // small device counters (the GPU-wide Jacobi's per-bin flags), lazily allocated
    size_t dcount_n;
    // streams and events of the staggered IBEM pipeline (one stream per part;
    // ev_fork orders them after the caller's stream), created at their first
    // use or by ia_capture_begin (ensure_side_stream)
    cudaStream_t side[IA_SPLIT_PARTS];
    cudaEvent_t ev_rows[IA_SPLIT_PARTS], ev_done[IA_SPLIT_PARTS], ev_fork;
};

namespace ia {
int ensure_side_stream(ia_context *ctx);
}

// threads per CTA of the IBEM assembly kernel; mesh colours are balanced to it
#define IA_ASM_THREADS 128

struct ia_mesh {
    ia_context *ctx;
    int m, n;              // nodes, triangles
    int ncolors;
    int nq, nqs;           // regular / singular rule sizes
    double *d_nodes;       // 3 x m SoA
    double *d_egeo;        // n x 16 per element (colour order): v0 v1 v2 (9), normal (3), |n|, pad
    int *d_evert;          // n x 4 per element (colour order): 3 vertex indices, pad
    int *d_color_ptr;      // ncolors + 1
    int *d_adj_ptr;        // m + 1: incident (element, slot) list per node
    int *d_adj;            // 3n: element index (colour order) * 4 + slot
    double *d_reg;         // 3 x nq
    double *d_sing;        // 9 x nqs
    double *d_qdat;        // regular-rule points: [q][x, y, z, w N_v / 4pi (3), w N_v |n| / 4pi (3)][element]
    double *d_qnrm;        // element normals [3][element]
    float *d_qdat_f;       // d_qdat as double-float (hi, lo) pairs
    float *d_qnrm_f;       // d_qnrm as double-float (hi, lo) pairs
    float4 *d_dftab;       // 1024 x (sin hi, sin lo, cos hi, cos lo)(j pi / 512) for the double-float assembly
    double *d_creg;        // m: the regular elements' C term per node (FP64), for the double-float assembly
    int *d_gptr, *d_gidx;  // node-node pattern, CSR (m + 1, gnnz): nodes sharing an element
    int gnnz;
};

namespace ia {

// ---- host-side NVTX range over the launches of one pipeline stage (shows
// the stage on a profiler's timeline; a no-op when no tool is attached)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// ---- error plumbing
int cuda_status(cudaError_t e);
#define IA_CUDA_TRY(expr)                                  \
    do {                                                   \
        cudaError_t e__ = (expr);                          \
        if (e__ != cudaSuccess) return ia::cuda_status(e__); \
    } while (0)
#define IA_LAUNCH_CHECK(ctx)                               \
    do {                                                   \
        (ctx)->launches++;                                 \
        cudaError_t e__ = cudaGetLastError();              \
        if (e__ != cudaSuccess) return ia::cuda_status(e__); \
    } while (0)

// workspace carving: returns IA_OK / IA_ERR_ALLOC
int ws_reserve(ia_context *ctx, size_t bytes);
struct WsCursor {
    char *base;
    size_t off, cap;
    template <class T>
    T *take(size_t count)
    {
        size_t a = (off + 255) & ~size_t(255);
        off = a + count * sizeof(T);
        return reinterpret_cast<T *>(base + a);
    }
};
inline size_t ws_round(size_t b) { return (b + 255) & ~size_t(255); }

// ---- dense kernels (dense.cu)
enum Op { OP_N = 0, OP_T = 1, OP_C = 2 };
// T = double2 (FP64) or float2 (FP32); instantiated in dense.cu
template <class T>
int gemm_batched(ia_context *ctx, Op opa, Op opb, int M, int N, int K, T alpha, const T *A, int lda, long long sA,
                 const T *B, int ldb, long long sB, T beta, T *C, int ldc, long long sC, int batch);
template <class T>
int getrf_batched(ia_context *ctx, int n, T *A, int lda, long long sA, int *ipiv, int *info, int batch);
template <class T>
int getrs_batched(ia_context *ctx, int n, int nrhs, const T *LU, int lda, long long sA, const int *ipiv, T *B,
                  int ldb, long long sB, int batch);
// X = U^-1 X for the upper triangle of LU (n x n), X n x nrhs
template <class T>
int backsolve_upper_batched(ia_context *ctx, int n, int nrhs, const T *LU, int lda, long long sA, T *B, int ldb,
                            long long sB, int batch);
// out[f] (cols x rows) = op(in[f]) (rows x cols), transposed, optionally conjugated
template <class T>
int transpose_batched(ia_context *ctx, int rows, int cols, const T *in, int ldi, long long si, T *out, int ldo,
                      long long so, bool conj, int batch);
// out = in (optionally conjugated), converting the element type
template <class TI, class TO>
int copy2d_batched(ia_context *ctx, int rows, int cols, const TI *in, int ldi, long long si, TO *out, int ldo,
                   long long so, bool conj, int batch);

inline int zgemm_batched(ia_context *ctx, Op opa, Op opb, int M, int N, int K, double2 alpha, const double2 *A,
                         int lda, long long sA, const double2 *B, int ldb, long long sB, double2 beta, double2 *C,
                         int ldc, long long sC, int batch)
{
    return gemm_batched<double2>(ctx, opa, opb, M, N, K, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, batch);
}
inline int zgetrf_batched(ia_context *ctx, int n, double2 *A, int lda, long long sA, int *ipiv, int *info, int batch)
{
    return getrf_batched<double2>(ctx, n, A, lda, sA, ipiv, info, batch);
}
inline int zgetrs_batched(ia_context *ctx, int n, int nrhs, const double2 *LU, int lda, long long sA, const int *ipiv,
                          double2 *B, int ldb, long long sB, int batch)
{
    return getrs_batched<double2>(ctx, n, nrhs, LU, lda, sA, ipiv, B, ldb, sB, batch);
}
inline int zbacksolve_upper_batched(ia_context *ctx, int n, int nrhs, const double2 *LU, int lda, long long sA,
                                    double2 *B, int ldb, long long sB, int batch)
{
    return backsolve_upper_batched<double2>(ctx, n, nrhs, LU, lda, sA, B, ldb, sB, batch);
}
inline int ztranspose_batched(ia_context *ctx, int rows, int cols, const double2 *in, int ldi, long long si,
                              double2 *out, int ldo, long long so, bool conj, int batch)
{
    return transpose_batched<double2>(ctx, rows, cols, in, ldi, si, out, ldo, so, conj, batch);
}
inline int zcopy2d_batched(ia_context *ctx, int rows, int cols, const double2 *in, int ldi, long long si, double2 *out,
                           int ldo, long long so, bool conj, int batch)
{
    return copy2d_batched<double2, double2>(ctx, rows, cols, in, ldi, si, out, ldo, so, conj, batch);
}
// Householder QR of A (rows x cols, rows >= cols) applied to [A | B] in place:
// on exit the upper triangle of A is R and B holds Q^H B.
int zgeqrs_batched(ia_context *ctx, int rows, int cols, double2 *A, int lda, long long sA, int nrhs, double2 *B,
                   int ldb, long long sB, int batch);

// C = alpha op(A) op(B) + beta C with FP64 inputs and output, products and
// sums in double-float (FP32 pairs) arithmetic (dfgemm.cu); op in {N, C}
int dfgemm_batched(ia_context *ctx, Op opa, Op opb, int M, int N, int K, double alpha, const double2 *A, int lda,
                   long long sA, const double2 *B, int ldb, long long sB, double beta, double2 *C, int ldc,
                   long long sC, int batch);
// the same with operands already split to float4 (re hi, im hi, re lo, im lo)
int dfgemm4_batched(ia_context *ctx, Op opa, Op opb, int M, int N, int K, double alpha, const float4 *A, int lda,
                    long long sA, const float4 *B, int ldb, long long sB, double beta, double2 *C, int ldc,
                    long long sC, int batch);
int split_df_batched(ia_context *ctx, size_t count, const double2 *in, float4 *out);
int df_hi_batched(ia_context *ctx, size_t count, const float4 *in, float2 *out);

// ---- tensor-core GEMM at FP64-level accuracy (tc_gemm.cu): operands cut
// into S balanced base-64 BF16 slices (Ozaki scheme), pair products on the
// tcgen05 pipe with exact FP32 level sums in TMEM
#define TC_SLICES_MIN 6
#define TC_SLICES_MAX 8
#define TC_SLICES_DEFAULT 7
struct TcPlanes {
    __nv_bfloat16 *p;   // [batch][S][rows][Kp] BF16 digits
    int *e;             // [batch][R] power-of-two scale exponents
    int R, rows, Kp, S; // R rows of op(A) (rows = R) or columns of op(B) (rows = 2 R)
};
size_t tc_planes_bytes(int R, int K, int S, bool role_b, int batch);
// cfg->gemm_slices selects the sliced GEMM for an inner dimension K (a slice
// count in range and exact FP32 level sums: S 1024 Kp <= 2^24)
inline bool tc_products_ok(int S, int K)
{
    return S >= TC_SLICES_MIN && S <= TC_SLICES_MAX && (long long)S * 1024 * ((2 * K + 7) & ~7) <= (1ll << 24);
}
// role_b false: A (M x K) = op(X); true: B (K x N) = op(X); R = M or N
int tc_slice(ia_context *ctx, bool role_b, Op op, const double2 *X, int ld, long long sX, int R, int K, int S,
             int batch, TcPlanes &out, WsCursor &cur);
int tc_slice(ia_context *ctx, bool role_b, Op op, const float4 *X, int ld, long long sX, int R, int K, int S,
             int batch, TcPlanes &out, WsCursor &cur);
// both operands of one product (A role: op(A) M x K, B role: op(B) K x N) in
// one launch
int tc_slice_pair(ia_context *ctx, Op opa, const double2 *A, int lda, long long sA, int M, Op opb, const double2 *B,
                  int ldb, long long sB, int N, int K, int S, int batch, TcPlanes &pa, TcPlanes &pb, WsCursor &cur);
// C (M x N complex FP64) = alpha A B + beta C; info (per batch entry, may be
// null) gets IA_INFO_TIMEOUT when a pipeline wait ran out
int tc_gemm(ia_context *ctx, const TcPlanes &A, const TcPlanes &B, int M, int N, double alpha, double beta,
            double2 *C, int ldc, long long sC, int batch, int *info);

// ---- SVD (svd.cu): Jacobi on Y (M x N, M >= N) in place; V (N x N) accumulated
int jacobi_svd_batched(ia_context *ctx, int M, int N, double2 *Y, double2 *V, int batch, int max_sweeps, int *info);
// Jacobi on Y (M x N) with only the first Mdot rows in the dot products
template <class T>
int jacobi_rows_batched(ia_context *ctx, int M, int Mdot, int N, T *Y, T *V, int batch, int max_sweeps, int *info);
// sigma, normalised sorted outputs: Uy (M x N) <- Y/sigma, Vs (N x N) <- V, both column-permuted to
// descending sigma.  Either output may be null.
int svd_finalize_batched(ia_context *ctx, int M, int N, const double2 *Y, const double2 *V, double *s,
                         double2 *Uy, double2 *Vs, int batch, int *info);
// full batched compact SVD of A (m x n) -> U (m x p), s, V (n x p); transposed_input: A given as A^T (n x m).
// Y (max(m,n) x p per matrix) and Vacc (p x p per matrix) are caller-provided workspace.
int svd_batched(ia_context *ctx, int m, int n, const double2 *A, bool transposed_input, double2 *U, double *s,
                double2 *V, int batch, int max_sweeps, int *info, double2 *Y, double2 *Vacc);
size_t svd_workspace_bytes(int m, int n, int batch);

// ---- regularisation (regularize.cu)
int regularize_batched(ia_context *ctx, int m, int n, int p, int batch, const double2 *U, const double *s,
                       const double2 *V, int nrhs, const double2 *b, const ia_config *cfg, double2 *x,
                       double *lambda);

// from projected beta (F x nrhs x p): z = phi .* beta, lambda per (f, rhs);
// bnorm2 (||b||^2 per (f, rhs)) may be null when m <= p (delta0 = 0)
int gcv_beta_batched(ia_context *ctx, int m, int p, int batch, const double *s, int nrhs, const double2 *beta,
                     const double *bnorm2, const ia_config *cfg, double2 *z, double *lambda);

// ---- regularised solve of wide / square operators (wide_solve.cu)
// A (m x n, m <= n) given as A or as A^T; x F x (n x nrhs).  Householder QR
// of A^H when n > m, one-sided Jacobi on R with U^H b carried as extra rows,
// GCV / Tikhonov, x = Q [U_R (phi .* beta); 0].
size_t wide_solve_ws_bytes(int m, int n, int nrhs, int batch);
int wide_solve_batched(ia_context *ctx, int m, int n, int batch, const double2 *A, bool transposed, int nrhs,
                       const double2 *b, const ia_config *cfg, double2 *x, double *lambda, double *s_out, int *info,
                       WsCursor &cur);
// mixed solve: eigenvectors X and eigenvalues of H H^H from an FP32 QR +
// one-sided Jacobi start, double-float Ogita-Aishima steps, Newton-Schulz and
// an FP64 two-sided Jacobi on X^H (H H^H) X; then s, U^H b, GCV, the
// back-projection and the precision guard (IA_INFO_PRECISION in info[f] for
// a bin whose lambda (TSVD: s_k) is below cfg->mixed_guard s_1,
// IA_INFO_UNRESOLVED for one whose sum of s^2 misses ||H_f||_F^2 by more than
// 1e-9 relative)
size_t wide_solve_mixed_ws_bytes(int m, int n, int nrhs, int batch);
int wide_solve_mixed_batched(ia_context *ctx, int m, int n, int batch, const double2 *A, bool transposed, int nrhs,
                             const double2 *b, const ia_config *cfg, double2 *x, double *lambda, double *s_out,
                             int *info, WsCursor &cur);
// Householder QR (reflectors below the diagonal, tau per column) and the
// explicit product X = Q [W; 0] (wide_solve.cu)
template <class T>
int qr_batched(ia_context *ctx, int rows, int cols, T *A, int lda, long long sA, T *tau, int batch);
template <class T>
int apply_q_batched(ia_context *ctx, int rows, int cols, const T *Y, const T *tau, int ncol, const T *W, int ldw,
                    long long sW, T *X, long long sX, int batch);
// out += in (FP32 or FP64 in, FP64 out), rows x cols per matrix
template <class TI>
int add2d_batched(ia_context *ctx, int rows, int cols, const TI *in, int ldi, long long si, double2 *out, int ldo,
                  long long so, int batch);

// ---- assembly (assemble.cu)
int monopole_batched(ia_context *ctx, int l, int m, int F, const double *mics, const double *src, const double *k,
                     double2 *G);
int esm_system(ia_context *ctx, int m, int l, const double *src, const double *mics, double r_i, double k, double c,
               double rho, double2 *DT, double2 *RHS);
// df32: regular-element arithmetic in double-float (mixed path) instead of FP64;
// split_ab (with df32): At and Bt are written as float4 (re hi, im hi, re lo, im lo)
int mesh_creg(ia_context *ctx, ia_mesh *mesh);
// two-sided FP64 Jacobi eigensolver of batch Hermitian N x N matrices S (in
// place, diagonalised), rotations accumulated into X (start it at the
// identity for the eigenvectors), LAM <- diag(S), unsorted; IA_INFO_NOCONV at
// the sweep cap
int herm_jacobi_batched(ia_context *ctx, int N, double2 *S, double2 *X, double *LAM, int max_sweeps, int batch,
                        int *info);
// debug builds: each instrumented translation unit's bounds record (read and cleared)
struct IaBoundsSite;
int bounds_read_dense(IaBoundsSite *out);
int bounds_read_tc(IaBoundsSite *out);
int bounds_read_svd(IaBoundsSite *out);
int bounds_read_wide(IaBoundsSite *out);
int bounds_read_asm(IaBoundsSite *out);
// gtab (double-float only): scratch of ibem_geom_bytes(mesh, m + n_ch + l)
// bytes for the per-call geometry table, or null to compute it inline;
// build_gtab false: the table already holds these rows' geometry
int ibem_rows(ia_context *ctx, const ia_mesh *mesh, int l, const double *mics, int n_ch, const double *cp, int F,
              const double *k, double c, double rho, double2 *At, double2 *Bt, double2 *Ahs_t, double2 *Bhs_t,
              bool df32 = false, bool split_ab = false, float2 *gtab = nullptr, bool build_gtab = true);
// bytes of the double-float assembly's geometry table for `rows` rows; 0
// when it is above the size the assembly uses a table for
size_t ibem_geom_bytes(const ia_mesh *mesh, int rows);
int hels_batched(ia_context *ctx, int npts, const double *pts, int order, int F, const double *k, double c,
                 double rho, double2 *Me, double2 *Qe);

// ---- radiation modes (radiation.cu)
// R (F x n x n FP64) and optionally an FP32 copy R32
int sinc_resistance_batched(ia_context *ctx, int n, const double *x, int F, const double *k, double area, double c,
                            double rho, double *R, float *R32);
// leading eigenpairs of the symmetric R, or (gram) of R R^T for a general R:
// left singular vectors, lambda = squared singular values
size_t radiation_modes_ws_bytes(int n, int F, int nm, const ia_config *cfg, bool gram = false);
int radiation_modes_batched(ia_context *ctx, int n, int F, const double *R, int nm, const ia_config *cfg,
                            double *lambda, double *modes, int *info, WsCursor &cur, bool gram = false);
// BEM radiation modes (bem_modes.cu)
// (cplx: Ur is double2 m x nm per frequency, modes of G Z; else double, of Re(G Z))
size_t bem_modes_ws_bytes(const ia_mesh *mesh, int l, int n_ch, int F, int nm, const ia_config *cfg, bool cplx);
int bem_modes_batched(ia_context *ctx, const ia_mesh *mesh, int l, const double *mics, int n_ch, const double *cp,
                      int F, const double *k, int nm, const ia_config *cfg, bool cplx, void *Ur, double *sr,
                      double2 *Hr, double2 *Pr, int *info, WsCursor &cur);
size_t sound_power_ws_bytes(int n, int F);

// ---- ADMM (admm.cu)
size_t admm_ws_bytes(int l, int m, int F, int nrhs);
int admm_batched(ia_context *ctx, int l, int m, int F, const double2 *H, int nrhs, const double2 *P,
                 const double *lam0, const ia_admm_config *acfg, const double2 *x0, double2 *c, int *iters,
                 int *info, WsCursor &cur);

// ---- differentiable ESM design (adjoint.cu); gm == nullptr: forward only
size_t esm_design_ws_bytes(int l, int m, int F, int R);
int esm_design_batched(ia_context *ctx, int l, int m, int F, int R, const double *mics, const double *surf,
                       const double *retreat, const double *k, const double *loglam, const double2 *q,
                       const double2 *noise, double *err, double *gm, double *gd, double *gl, int *info,
                       WsCursor &cur);
int sound_power_batched(ia_context *ctx, int n, int F, const double *R, int nrhs, const double2 *v, double *W,
                        WsCursor &cur);

}  // namespace ia
