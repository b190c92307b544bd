/* ia.h -- C ABI of the GB300-native inverse-acoustics library (libia.so).
 *
 * Two layers:
 *
 * 1. Reference-compatible entry points.  Same argument order and meaning as
 *    the reference's CUDA headers' functions: host input arrays, outputs malloc'd
 *    by the callee and released by the caller (here with ia_free or free()).
 *    Where the reference throws or exit()s, these return a status code.
 *
 *      ia_esm   <- esm()   CUDA/esm.cuh:112   (and esmgpu() CUDA/esm.cuh:38)
 *      ia_ibem  <- ibem()  CUDA/ibem.cuh:424  (and ibemgpu() CUDA/ibem.cuh:263)
 *      ia_invr  <- invr()  CUDA/invr.cuh:457  (and invrgpu() CUDA/invr.cuh:291)
 *      ia_hels  <- hels()  CUDA/hels.cuh:222  (and helsgpu() CUDA/hels.cuh:185)
 *      ia_csvd  <- csvd()  CUDA/tsvd.cuh:10
 *      ia_tsvd  <- tsvd()  CUDA/tsvd.cuh:122
 *      ia_to_pressure / ia_to_velocity / ia_sound_power
 *               <- to_pressure / to_velocity / sound_power CUDA/utils.cuh:199,232,265
 *
 * 2. Device-resident batched entry points (the GB300 path).  All array
 *    arguments named d_* are device pointers; one call processes F
 *    frequencies, each an independent problem.  Calls are ordered on the
 *    context's CUDA stream and do not synchronise the host unless stated.
 *
 * Conventions (as the reference): complex numbers are interleaved double
 * pairs (the layout of cuDoubleComplex); matrices are column-major; point
 * sets are structure-of-arrays x[0..n), y[0..n), z[0..n) (CUDA/esm.cuh:9);
 * triangle connectivity is e_n[i + j*n], 0-based (CUDA/ibem.cuh:10).  The
 * outgoing wave is exp(+ikr) (CUDA/esm.cuh:16).  A batch of F matrices of
 * size r x c is stored as F consecutive column-major r x c blocks.
 *
 * Every function returns an ia_status; nothing throws across this ABI.
 */
#ifndef IA_H
#define IA_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { double re, im; } ia_complex;

typedef enum {
    IA_OK = 0,
    IA_ERR_ARG = 1,          /* invalid argument (null pointer, bad size, k out of range) */
    IA_ERR_CUDA = 2,         /* CUDA runtime error (see ia_last_cuda_error) */
    IA_ERR_ALLOC = 3,        /* host or device allocation failed */
    IA_ERR_NOCONV = 4,       /* a Jacobi iteration hit its sweep cap (per-frequency info says which) */
    IA_ERR_SINGULAR = 5,     /* an exactly zero pivot in an LU factorisation */
    IA_ERR_NONFINITE = 6,    /* NaN or Inf in an input or a result */
    IA_ERR_RULE = 7,         /* invalid quadrature rule */
    IA_ERR_TOO_LARGE = 8,    /* size above a fixed limit of the called entry point */
    IA_ERR_CAPTURE = 9       /* the call would allocate during stream capture: run it once uncaptured first */
} ia_status;

/* per-frequency info words written by the batched solvers (bit flags) */
#define IA_INFO_NOCONV    1  /* Jacobi sweep cap reached */
#define IA_INFO_SINGULAR  2  /* zero pivot */
#define IA_INFO_NONFINITE 4  /* NaN/Inf met */
#define IA_INFO_TIMEOUT   8  /* a bounded device-side wait ran out (the entry's output is not written) */
#define IA_INFO_PRECISION 16 /* mixed path: the bin's regularisation level is below the mixed floor
                                (mixed_guard) and the bin was not recomputed in FP64 (fallback off, or
                                the stream was capturing) */
#define IA_INFO_UNRESOLVED 32 /* mixed path: the bin's eigen-decomposition failed the trace check
                                 (sum s^2 against ||H||_F^2) and was not solved again; with
                                 IA_INFO_PRECISION too when its spectrum reaches the Gram floor
                                 sqrt(N eps) s_1 */

enum { IA_GCV_STANDARD = 0, IA_GCV_REFERENCE = 1 };
enum { IA_PREC_FP64 = 0, IA_PREC_MIXED = 1 };
/* Regularisation: filter and lambda selector.  Tikhonov filter s^2/(s^2+l^2)
 * (MATLAB/regtools/tikhonovG.m), damped SVD s/(s+l) (dsvdG.m), TSVD
 * (tsvdG.m); lambda by GCV (gcvG.m), the L-curve corner (l_curveG.m,
 * lcfunG.m), the quasi-optimality criterion (quasioptG.m) or lambda_fixed.
 * The grid-based selectors share gcv_points.  With IA_PREC_MIXED the damped-SVD
 * methods run the FP64 solve (their 1/(s + lambda) weights keep the
 * components of singular values the mixed path does not resolve). */
enum {
    IA_METHOD_TIKHONOV_GCV = 0,
    IA_METHOD_TSVD = 1,
    IA_METHOD_TIKHONOV_FIXED = 2,
    IA_METHOD_TIKHONOV_LCURVE = 3,
    IA_METHOD_TIKHONOV_QUASIOPT = 4,
    IA_METHOD_DSVD_FIXED = 5,
    IA_METHOD_DSVD_LCURVE = 6,
    IA_METHOD_DSVD_QUASIOPT = 7
};

typedef struct {
    double c;              /* speed of sound [m/s]; reference C_AIR (CUDA/constants.cuh:2) */
    double rho;            /* density [kg/m^3]; reference RHO_AIR (CUDA/constants.cuh:5) */
    int method;            /* IA_METHOD_* */
    int gcv_mode;          /* IA_GCV_STANDARD (Hansen's Tikhonov GCV) or IA_GCV_REFERENCE (gcvG.m as written) */
    int gcv_points;        /* grid size, 200 in gcvG.m:20 */
    double gcv_lo;         /* fixed log-spaced grid [gcv_lo, gcv_hi]; both 0 selects */
    double gcv_hi;         /*   regtools' grid max(s_p, 16 eps s_1) .. s_1 (gcvG.m:28-30) */
    double lambda_fixed;   /* lambda for IA_METHOD_TIKHONOV_FIXED / IA_METHOD_DSVD_FIXED */
    int tsvd_k;            /* truncation index for IA_METHOD_TSVD, 1 <= k <= p */
    int precision;         /* IA_PREC_FP64 or IA_PREC_MIXED */
    int svd_max_sweeps;    /* Jacobi sweep cap (default 40) */
    int refine_steps;      /* refinement steps of the mixed path: LU residual steps and
                              eigen-refinement steps (default 1; each squares the error) */
    int mode_iters;        /* radiation modes: subspace iterations (default 10; FP32 in the
                              mixed path, which then adds refine_steps FP64 ones) */
    int mode_oversample;   /* radiation modes: subspace vectors beyond the requested modes (default 16) */
    int gemm_slices;       /* the mixed path's FP64-level complex products (IBEM refinement residual and
                              transfer product): 6..8 = tensor-core GEMM on that many BF16 slices per
                              operand (default 7); 0 = double-float CUDA-core GEMM */
    double mixed_guard;    /* mixed solves: the smallest lambda / s_1 (TSVD: s_k / s_1) the mixed path
                              answers (default 1e-3).  Below it the Gram-based mixed eigensolver does not
                              resolve the singular values that decide the solution (IA_INFO_PRECISION);
                              a bin whose sum of s_i^2 misses ||H||_F^2 by more than 1e-9 relative fails
                              too (IA_INFO_UNRESOLVED), as does a bin with any solver flag. */
    int pipeline_parts;    /* IBEM batches: staggered parts, one stream each (0 = automatic: 4 when F is a
                              multiple of 16 and >= 32, 2 when a multiple of 8 and >= 16, else 1;
                              explicit: 1..8 dividing F into parts of a multiple of 4 bins) */
    int mixed_fallback;    /* 1 (default): bins that fail the guard are solved again before the call
                              returns -- IA_INFO_UNRESOLVED alone by the mixed path with 3 eigen-
                              refinement steps first, everything else (and what fails again) by the
                              FP64 path (one host synchronisation per call; skipped while the stream
                              is capturing, where such bins keep their flags); 0: never */
} ia_config;

/* quadrature rules for IBEM: barycentric (xi1, xi2, w) structure-of-arrays,
 * weights summing to 1/2 as in the reference's IPF.txt / IPFs.txt
 * (CUDA/ibem.cuh:276-311).  singular holds 3 pages (one per vertex of the
 * element, the vertex with shape function 1 at the singular point), each
 * 3*nqs doubles. */
typedef struct {
    int nq;
    const double *regular;   /* 3*nq   : xi1[nq], xi2[nq], w[nq] */
    int nqs;
    const double *singular;  /* 9*nqs  : page0, page1, page2 */
} ia_rules;

/* ADMM sparse / regularised inversion (MATLAB/ADMMG.m:1-90; its arguments
 * rho, gamma, epsilon, Nm, nor and, for nor = 3, p and N). */
enum { IA_ADMM_L1 = 1, IA_ADMM_L2 = 2, IA_ADMM_LP = 3 };
typedef struct {
    int norm;         /* IA_ADMM_L1 (soft threshold), IA_ADMM_L2, IA_ADMM_LP (generalised soft threshold) */
    int max_iters;    /* Nm: iterations per continuation stage (L1, Lp) or in all (L2) */
    double rho;       /* augmented-Lagrangian weight, > 0 */
    double gamma;     /* dual step factor */
    double epsilon;   /* stop when ||c - c_old||, ||c - x|| and ||u - u_old|| are all <= epsilon */
    double p;         /* Lp exponent, 0 < p <= 1 (IA_ADMM_LP) */
    int gst_iters;    /* N: fixed-point steps of the generalised soft threshold (IA_ADMM_LP) */
    int precision;    /* IA_PREC_FP64, or IA_PREC_MIXED: the iteration's matrix-vector products in
                         double-float (FP32 pairs, ~48-bit significand); setup, shrink and norms FP64 */
} ia_admm_config;

void ia_config_default(ia_config *cfg);
/* norm L1, max_iters 200, rho 1, gamma 1, epsilon 1e-6, p 0.5, gst_iters 5, FP64 */
void ia_admm_config_default(ia_admm_config *cfg);
/* sizeof(ia_config), for bindings that mirror the struct */
int ia_config_size(void);
const char *ia_status_string(int status);
const char *ia_version(void);
int ia_last_cuda_error(void);
void ia_free(void *p);

/* Debug aid with no counterpart in the reference (which has no checks of its
 * own): in the debug build of the library (libia_debug.so, compiled with
 * IA_DEBUG_BOUNDS) the main kernels test their global-memory indexes against
 * the buffers' extents, skip an access that fails and record it.  This call
 * reports the records since the previous call and clears them: *enabled = 1
 * when the library was built with the checks (0: release build, nothing
 * checked), *count = the number of failed tests, and for the first failure its
 * source file name (static string, or NULL), line, index and extent.  It
 * copies from the device and so waits for the device's queued work. */
int ia_bounds_report(int *enabled, unsigned long long *count, const char **file, int *line, long long *index,
                     long long *extent);

/* gmsh v2.2 ASCII mesh reader; replaces geometry() (CUDA/utils.cuh:291).
 * Nodes r_ms (3 x m SoA), triangles e_n (element type 2 with three distinct
 * vertices, 0-based, 3 x n SoA, file order) and field points
 * r_lh = r_ms (1 + (2 pi / k) t) (3 x m), all malloc'd by the callee (free
 * with ia_free).  Host only, no GPU needed.  A missing or malformed file
 * returns IA_ERR_ARG (the reference calls exit()). */
int ia_read_msh(const char *file, double k, double t, double **r_ms, double **r_lh, int **e_n, int *m, int *l,
                int *n);

/* ---------------------------------------------------------------- layer 1 */

/* ESM: Me = M_sq D^-1 (m x m), He = M_hq D^-1 (l x m), sources at r_ms*r_i.
 * Replaces esm() CUDA/esm.cuh:112 (correct for l != m, where the reference's
 * M_hq leading dimension is wrong). */
int ia_esm(int m, int l, const double *r_ms, const double *r_lh, ia_complex **m_e, ia_complex **h,
           double k, double r_i, const ia_config *cfg);

/* IBEM: Z = A \ (i rho c k B) (m x m) and H = A_hs Z - i rho c k B_hs (l x m).
 * n triangles e_n, n_ch CHIEF points cp (least squares when n_ch > 0).
 * rules == NULL selects the built-in 7-point regular / 4x4 Duffy singular rules.
 * Replaces ibem() CUDA/ibem.cuh:424 (which reads IPF.txt/IPFs.txt from the cwd). */
int ia_ibem(int m, int l, int n, const double *r_ms, const int *e_n, const double *r_lh, ia_complex **m_e,
            ia_complex **h, double k, int n_ch, const double *cp, const ia_rules *rules, const ia_config *cfg);

/* BEM radiation modes at one wavenumber: q_e (m x n_am) the leading left
 * singular vectors of the complex G Z (phase as ia_bem_modes_complex_batch),
 * h (l x n_am) = (A_hs Z - B_hs) q_e, m_e (m x n_am) = Z q_e; 1 <= n_am <= m.
 * Replaces invr() CUDA/invr.cuh:457 and invrgpu() CUDA/invr.cuh:263 (whose
 * GPU version computes these products for any n_am; the CPU version only for
 * n_am = m, invr.cuh:904,907).  rules as ia_ibem. */
int ia_invr(int m, int l, int n, const double *r_ms, const int *e_n, const double *r_lh, ia_complex **m_e,
            ia_complex **h, ia_complex **q_e, double k, int n_ch, const double *cp, int n_am, const ia_rules *rules,
            const ia_config *cfg);

/* HELS: Me (m x nt), He (l x nt), Qe (m x nt), nt = (n_sh+1)^2, column
 * i = n^2 + n + m.  Points in (az, el, r) structure-of-arrays.
 * Replaces hels() CUDA/hels.cuh:222. */
int ia_hels(int m, int l, const double *r_ms_s, const double *r_lh_s, ia_complex **m_e, ia_complex **h,
            ia_complex **q_e, double k, int n_sh, const ia_config *cfg);

/* Compact SVD a = u diag(s) v^H: u m x p, s p, v n x p, p = min(m, n),
 * s descending.  Replaces csvd() CUDA/tsvd.cuh:10 (which returns v n x n
 * when m >= n; the first p columns agree). */
int ia_csvd(int m, int n, const ia_complex *a, ia_complex **u, double **s, ia_complex **v);

/* x = V(:,1:k) diag(1/s(1:k)) U(:,1:p)^H b.  Returns IA_ERR_ARG for k
 * outside [1, p] (the reference prints and leaves *x unset,
 * CUDA/tsvd.cuh:124-126).  Replaces tsvd() CUDA/tsvd.cuh:122. */
int ia_tsvd(int m, int n, int p, int k, const ia_complex *u, const double *s, const ia_complex *v,
            const ia_complex *b, ia_complex **x);

/* p = Me x, v = Qe x (m x n times n); W = 1/2 Re(v^H p) S/m.
 * Replace CUDA/utils.cuh:199, :232, :265. */
int ia_to_pressure(int m, int n, const ia_complex *me, const ia_complex *x, ia_complex **p);
int ia_to_velocity(int m, int n, const ia_complex *qe, const ia_complex *x, ia_complex **v);
int ia_sound_power(int m, const ia_complex *p, const ia_complex *v, double *w, double s);

/* ---------------------------------------------------------------- layer 2 */

typedef struct ia_context ia_context;
typedef struct ia_mesh ia_mesh;

/* stream: a cudaStream_t (NULL = legacy default stream). */
int ia_create(ia_context **ctx, int device, void *stream);
int ia_destroy(ia_context *ctx);
int ia_set_stream(ia_context *ctx, void *stream);
int ia_synchronize(ia_context *ctx);
/* number of kernels this context has launched since creation */
long long ia_launch_count(const ia_context *ctx);

/* CUDA graphs of batched calls (no reference counterpart: the reference
 * creates streams and handles per call).  Between ia_capture_begin and
 * ia_capture_end the context's stream records instead of running; the
 * recorded kernels, copies and memsets replay with ia_graph_launch on the
 * context's current stream, reading and writing the same device buffers, so a
 * caller refills its input buffers and replays.  The context's stream must be
 * a created stream (not the legacy default one).  A captured call must not
 * grow the workspace: run it once uncaptured first (otherwise it returns
 * IA_ERR_CAPTURE).  The graph holds pointers into the context's workspace:
 * keep the context alive and do not run larger calls on it before the last
 * replay. */
/* Autotuner.  GEMM-type kernels come in several tile shapes; the first call
 * of each (kernel, shape, transposition, batch) outside stream capture times
 * every shape on scratch outputs and keeps the fastest in a process-wide
 * table.  All shapes sum in the same order, so results do not depend on the
 * choice.  Environment: IA_TUNE=0 disables tuning (first shape everywhere);
 * IA_TUNE_FILE=<path> loads choices from, and appends new ones to, a text
 * file.  ia_tune_reset forgets the table and re-reads the environment. */
int ia_tune_table_size(void);
void ia_tune_reset(void);

/* Number of bins the last batched solve on ctx (ia_solve_batch and the
 * ia_*_solve_batch pipelines) handed from the mixed path to the FP64 path
 * (mixed_fallback); 0 after an FP64 call.  No reference counterpart. */
int ia_last_fallback_bins(const ia_context *ctx);

typedef struct ia_graph ia_graph;
int ia_capture_begin(ia_context *ctx);
int ia_capture_end(ia_context *ctx, ia_graph **graph);
int ia_graph_launch(ia_graph *graph);
/* kernel nodes in the graph */
int ia_graph_kernel_count(const ia_graph *graph);
int ia_graph_destroy(ia_graph *graph);

/* Upload a triangle mesh (host arrays) with its quadrature rules; builds the
 * element geometry, the element colouring and the node-to-element adjacency
 * used by the gather-form assembly. */
int ia_mesh_create(ia_context *ctx, int m, int n, const double *nodes, const int *elems, const ia_rules *rules,
                   ia_mesh **mesh);
int ia_mesh_destroy(ia_mesh *mesh);

/* G_f(i,j) = exp(i k_f r_ij)/(4 pi r_ij), microphones d_mics (3 x l SoA) by
 * sources d_src (3 x m SoA): the plain ESM transfer matrix, F x (l x m). */
int ia_monopole_batch(ia_context *ctx, int l, int m, int F, const double *d_mics, const double *d_src,
                      const double *d_k, ia_complex *d_G);

/* IBEM system rows for F wavenumbers, row-major rows (each collocation row
 * contiguous, i.e. the column-major transpose):
 *   d_At, d_Bt : F x (m x mt)  columns = surface rows 0..m-1 then CHIEF rows
 *   d_Ahs_t, d_Bhs_t : F x (m x l)  columns = field rows
 * B terms scaled by i rho c k.  Any of the outputs may be NULL only together
 * with its partner.  IA_PREC_MIXED keeps a per-call table of the
 * frequency-independent point geometry (8 x 3 x rows x nq x elements bytes,
 * used up to 1 GiB) in the context's workspace, so it may return
 * IA_ERR_CAPTURE like the solvers. */
int ia_ibem_assemble_batch(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int n_ch,
                           const double *d_cp, int F, const double *d_k, const ia_config *cfg, ia_complex *d_At,
                           ia_complex *d_Bt, ia_complex *d_Ahs_t, ia_complex *d_Bhs_t);

/* IBEM transfer matrices H_f = A_hs A^-1 B - B_hs (F x (l x m)), without
 * forming Z (an l-right-hand-side solve); square systems only (n_ch = 0). */
int ia_ibem_transfer_batch(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int F,
                           const double *d_k, const ia_config *cfg, ia_complex *d_H, int *d_info);

/* HELS field matrix He (F x (l x nt)) at points (az, el, r) d_pts. */
int ia_hels_batch(ia_context *ctx, int l, const double *d_pts, int n_sh, int F, const double *d_k,
                  ia_complex *d_H);

/* Batched compact SVD of F matrices m x n: d_U F x (m x p), d_s F x p,
 * d_V F x (n x p), p = min(m, n); d_U / d_V may be NULL. */
int ia_svd_batch(ia_context *ctx, int m, int n, int F, const ia_complex *d_A, ia_complex *d_U, double *d_s,
                 ia_complex *d_V, int *d_info);

/* Regularised solves from SVD factors: for each frequency f and right-hand
 * side r, x = V diag(phi) U^H b with phi from cfg->method (Tikhonov with the
 * GCV lambda, TSVD, or a fixed lambda).  d_b F x (m x nrhs), d_x F x (n x nrhs),
 * d_lambda F x nrhs (lambda used; 0 for TSVD). */
int ia_regularize_batch(ia_context *ctx, int m, int n, int F, const ia_complex *d_U, const double *d_s,
                        const ia_complex *d_V, int nrhs, const ia_complex *d_b, const ia_config *cfg,
                        ia_complex *d_x, double *d_lambda);

/* One frequency-solve per frequency: SVD of d_H (F x (m x n)), regularised
 * solution of H x = b.  d_s (F x p) and d_info (F) may be NULL. */
int ia_solve_batch(ia_context *ctx, int m, int n, int F, const ia_complex *d_H, int nrhs, const ia_complex *d_b,
                   const ia_config *cfg, ia_complex *d_x, double *d_lambda, double *d_s, int *d_info);

/* Batched complex GEMM, C = alpha op(A) op(B) + beta C (op: 0 N, 1 T, 2 C),
 * FP64 operands and output on the device; replaces the reference's
 * cublasZgemm (CUDA/ibem.cuh:398).  precision IA_PREC_FP64: FP64 CUDA-core
 * GEMM.  IA_PREC_MIXED: tensor-core GEMM on BF16 slices (Ozaki scheme) with
 * `slices` slices per operand (6..8, 0 = 7), exact FP32 level sums in tensor
 * memory; error at most (4 slices + 8) 2^(-6 slices) of max|A row|
 * max|B col| per product term (8e-12 at 7 slices, 1.4e-13 at 8);
 * needs slices * 2048 * K <= 2^24 (K <= 1170 at 7 slices, else
 * IA_ERR_TOO_LARGE).  d_info (batch ints, may be NULL) gets IA_INFO_TIMEOUT
 * for an entry whose pipeline wait ran out. */
int ia_zgemm_batch(ia_context *ctx, int opa, int opb, int M, int N, int K, double alpha, const ia_complex *d_A,
                   int lda, long long sA, const ia_complex *d_B, int ldb, long long sB, double beta,
                   ia_complex *d_C, int ldc, long long sC, int batch, int precision, int slices, int *d_info);

/* Size of the device array that ia_solve_batch_noalloc works in. */
#define IA_NOALLOC_SCRATCH_BYTES (16u << 20)

/* ia_solve_batch without any device allocation (no counterpart in the
 * reference).  For callers that may not allocate device memory: a real-time
 * acquisition loop, where cudaMalloc's implicit synchronisation and latency
 * would drop frames, or code recording the solve into a CUDA graph during
 * stream capture.  Scratch comes from one static device array of
 * IA_NOALLOC_SCRATCH_BYTES (held by every GPU that loads the library until
 * exit).  Wide or square operators only (m <= n), FP64 path; larger problems
 * return IA_ERR_TOO_LARGE.  The first call on a device looks the array's
 * address up and should come before any stream capture.  The call never
 * times GEMM tile variants (the autotuner's table is read, not filled), so it
 * neither allocates nor synchronises on a shape's first use.  All calls share
 * the array: calls that overlap on the GPU race. */
int ia_solve_batch_noalloc(ia_context *ctx, int m, int n, int F, const ia_complex *d_H, int nrhs,
                           const ia_complex *d_b, const ia_config *cfg, ia_complex *d_x, double *d_lambda,
                           double *d_s, int *d_info);

/* The whole IBEM pipeline for F frequencies: assembly, H, SVD, GCV/Tikhonov.
 * d_p F x (l x nrhs) measured pressures, d_x F x (m x nrhs) surface velocity. */
int ia_ibem_solve_batch(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int F,
                        const double *d_k, int nrhs, const ia_complex *d_p, const ia_config *cfg, ia_complex *d_x,
                        double *d_lambda, double *d_s, int *d_info);

/* The ESM pipeline (plain monopole G, sources given) for F frequencies. */
int ia_esm_solve_batch(ia_context *ctx, int l, int m, const double *d_mics, const double *d_src, int F,
                       const double *d_k, int nrhs, const ia_complex *d_p, const ia_config *cfg, ia_complex *d_x,
                       double *d_lambda, double *d_s, int *d_info);

/* Radiation resistance matrices of n baffled radiators of equal area at
 * d_x (3 x n SoA) for F wavenumbers:
 *   R_f(i,j) = omega^2 rho A^2 / (4 pi c) sinc(k_f r_ij),  omega = k_f c,
 * real symmetric, column-major, d_R F x (n x n) FP64; c and rho from cfg.
 * The reference names this model for its radiation-mode configuration but
 * has no code for it (its BEM variant is invr(), CUDA/invr.cuh:457). */
int ia_sinc_resistance_batch(ia_context *ctx, int n, const double *d_x, int F, const double *d_k, double area,
                             const ia_config *cfg, double *d_R);

/* Leading radiation modes: the nmodes largest eigenvalues (descending) and
 * orthonormal eigenvectors of each real symmetric positive semidefinite
 * R_f (d_R F x (n x n)), by subspace iteration on nmodes + cfg->mode_oversample
 * vectors and an FP64 Rayleigh-Ritz step.  d_lambda F x nmodes, d_modes
 * F x (n x nmodes), each mode's largest component positive.  Eigenvalues at
 * rounding level (below ~1e-15 lambda_1) carry no digits.  No reference
 * counterpart (the reference's invr() takes an SVD of a BEM resistance
 * matrix, MATLAB/invrV.m:65-119). */
int ia_radiation_modes_batch(ia_context *ctx, int n, int F, const double *d_R, int nmodes, const ia_config *cfg,
                             double *d_lambda, double *d_modes, int *d_info);

/* BEM radiation modes of a closed surface, F wavenumbers; replaces invr()
 * (CUDA/invr.cuh:457), specified by MATLAB/invrS.m:18-170.  Z = A \ B (the
 * IBEM surface system; least squares when n_ch > 0 CHIEF points d_cp 3 x n_ch
 * add rows, as invr.cuh:860 zgels and invrS.m:159), G the surface mass matrix,
 * R = Re(G Z), U_r the nmodes leading left singular vectors of R (d_Ur
 * F x (m x nmodes), real, each column's first component within 1e-6 of its
 * largest magnitude positive; d_sr F x nmodes, descending), H_r =
 * (A_hs Z - B_hs) U_r at the field points d_mics (d_Hr F x (l x nmodes)),
 * P_r = Z U_r the modal surface pressures (d_Pr F x (m x nmodes), or NULL).
 * The outputs have the sizes invrS.m gives for any n_am (invr.cuh:904,907 use
 * n_am as the inner dimension, which is H U and Z U only for n_am = m).
 * Singular vectors by subspace iteration on R R^T (cfg->mode_iters,
 * mode_oversample; FP32 iterations with IA_PREC_MIXED, which also assembles
 * in double-float). */
int ia_bem_modes_batch(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int n_ch,
                       const double *d_cp, int F, const double *d_k, int nmodes, const ia_config *cfg, double *d_Ur,
                       double *d_sr, ia_complex *d_Hr, ia_complex *d_Pr, int *d_info);

/* As ia_bem_modes_batch, with the modes of the complex G Z itself, as the
 * C++ invr() takes them (CUDA/invr.cuh:868-889 zgesvd of G Z): d_Ur
 * F x (m x nmodes) complex, each column's phase fixed so that its first
 * component within 1e-6 of its largest magnitude is real and positive (the
 * phase of a singular vector is arbitrary; zgesvd's is not reproduced).
 * While p = nmodes + max(nmodes, mode_oversample) is at most m / 2, the
 * leading modes by subspace iteration on the real representation of
 * (G Z)(G Z)^H with p vectors: 2 mode_iters + 4 max(1, refine_steps) FP64
 * iterations, or with IA_PREC_MIXED (double-float assembly) 2 mode_iters FP32
 * and 4 max(1, refine_steps) double-float ones.  Otherwise the FP64 one-sided
 * Jacobi SVD of the whole G Z (cfg->svd_max_sweeps). */
int ia_bem_modes_complex_batch(ia_context *ctx, const ia_mesh *mesh, int l, const double *d_mics, int n_ch,
                               const double *d_cp, int F, const double *d_k, int nmodes, const ia_config *cfg,
                               ia_complex *d_Ur, double *d_sr, ia_complex *d_Hr, ia_complex *d_Pr, int *d_info);

/* ADMM inversion of F independent systems H_f c = p_f, each with nrhs
 * right-hand sides: d_H F x (l x m), d_p F x (l x nrhs), d_lambda0 F x nrhs
 * (lambda_0 of each system), d_x0 F x (m x nrhs) the starting x or NULL for
 * A \ b (least squares when m <= l; the minimum-norm solution when m > l,
 * where MATLAB's backslash gives a pivoting-dependent basic solution).
 * Returns d_c F x (m x nrhs) (ADMMG.m's output c), d_iters F x nrhs (c-updates
 * run, or NULL) and d_info (IA_INFO_NOCONV: no stage met epsilon).  FP64.
 * Replaces MATLAB/ADMMG.m:1-90 (function ADMM). */
int ia_admm_batch(ia_context *ctx, int l, int m, int F, const ia_complex *d_H, int nrhs, const ia_complex *d_p,
                  const double *d_lambda0, const ia_admm_config *acfg, const ia_complex *d_x0, ia_complex *d_c,
                  int *d_iters, int *d_info);

/* Sound power W_f,r = 1/2 Re(v^H R_f v) of F x nrhs velocity fields
 * d_v F x (n x nrhs) (the reference's 1/2 Re(v^H p), CUDA/utils.cuh:265-280,
 * with p = R v): d_W F x nrhs. */
int ia_sound_power_batch(ia_context *ctx, int n, int F, const double *d_R, int nrhs, const ia_complex *d_v,
                         double *d_W);

/* Differentiable ESM array design (no reference counterpart; the operator is
 * the plain monopole G of MATLAB/esmV.m:29-30, the inverse Tikhonov,
 * MATLAB/regtools/tikhonovG.m:26-30).  Equivalent sources
 * s_j = u_j (1 - retreat / |u_j|) from surface points d_surface (3 x m),
 * microphones d_mics (3 x l, l <= m), source fields d_q F x (m x nrhs),
 * pressures p = G q + noise (d_noise F x (l x nrhs), or NULL), reconstruction
 * q^ = G^H (G G^H + lambda_f^2 I)^-1 p with lambda_f = exp(d_loglam[f]).
 * d_err F x nrhs receives ||q^ - q|| / ||q||; the gradients of their mean with
 * respect to the microphone coordinates (d_grad_mics 3 x l SoA), the retreat
 * (d_grad_retreat, 1) and the log lambdas (d_grad_loglam, F) come from a
 * hand-written adjoint.  The retreat is a device scalar so optimisers can
 * update it without a host round trip.  The three gradient pointers are all
 * NULL (forward only) or all set.  nrhs <= 32.  FP64. */
int ia_esm_design_batch(ia_context *ctx, int l, int m, int F, int nrhs, const double *d_mics,
                        const double *d_surface, const double *d_retreat, const double *d_k, const double *d_loglam,
                        const ia_complex *d_q, const ia_complex *d_noise, double *d_err, double *d_grad_mics,
                        double *d_grad_retreat, double *d_grad_loglam, int *d_info);

/* The HELS pipeline (He of order n_sh at field points) for F frequencies. */
int ia_hels_solve_batch(ia_context *ctx, int l, const double *d_pts, int n_sh, int F, const double *d_k, int nrhs,
                        const ia_complex *d_p, const ia_config *cfg, ia_complex *d_x, double *d_lambda,
                        double *d_s, int *d_info);

#ifdef __cplusplus
}
#endif
#endif /* IA_H */
