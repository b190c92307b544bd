/* Fortran-name LAPACK/BLAS entry points for the reference's CPU path.
 *
 * Test infrastructure only (linked into oracle/_ref/libiaref.so).  The
 * reference declares plain Fortran symbols (CUDA/utils.cuh:10-30); the only
 * LAPACK in this image is scipy's bundled OpenBLAS, which exports them with a
 * "scipy_" prefix.  Each function below forwards one call unchanged.
 */
typedef struct { double re, im; } zc;

extern void scipy_zgels_(const char *, int *, int *, int *, zc *, int *, zc *, int *, zc *, int *, int *);
extern void scipy_zgemm_(const char *, const char *, int *, int *, int *, zc *, zc *, int *, zc *, int *, zc *, zc *, int *);
extern void scipy_zlacpy_(const char *, int *, int *, zc *, int *, zc *, int *);
extern void scipy_zaxpy_(int *, zc *, zc *, int *, zc *, int *);
extern void scipy_zscal_(int *, zc *, zc *, int *);
extern void scipy_zgesvd_(const char *, const char *, int *, int *, zc *, int *, double *, zc *, int *, zc *, int *, zc *, int *, double *, int *);
extern void scipy_zgemv_(const char *, int *, int *, zc *, zc *, int *, zc *, int *, zc *, zc *, int *);
extern void scipy_zimatcopy_(const char *, const char *, int *, int *, zc *, zc *, int *, int *);

void zgels_(const char *t, int *m, int *n, int *r, zc *a, int *lda, zc *b, int *ldb, zc *w, int *lw, int *info)
{ scipy_zgels_(t, m, n, r, a, lda, b, ldb, w, lw, info); }
void zgemm_(const char *ta, const char *tb, int *m, int *n, int *k, zc *al, zc *a, int *lda, zc *b, int *ldb, zc *be, zc *c, int *ldc)
{ scipy_zgemm_(ta, tb, m, n, k, al, a, lda, b, ldb, be, c, ldc); }
void zlacpy_(const char *u, int *m, int *n, zc *a, int *lda, zc *b, int *ldb) { scipy_zlacpy_(u, m, n, a, lda, b, ldb); }
void zaxpy_(int *n, zc *al, zc *x, int *ix, zc *y, int *iy) { scipy_zaxpy_(n, al, x, ix, y, iy); }
void zscal_(int *n, zc *al, zc *x, int *ix) { scipy_zscal_(n, al, x, ix); }
void zgesvd_(const char *ju, const char *jv, int *m, int *n, zc *a, int *lda, double *s, zc *u, int *ldu, zc *vt, int *ldvt,
             zc *w, int *lw, double *rw, int *info)
{ scipy_zgesvd_(ju, jv, m, n, a, lda, s, u, ldu, vt, ldvt, w, lw, rw, info); }
void zgemv_(const char *t, int *m, int *n, zc *al, zc *a, int *lda, zc *x, int *ix, zc *be, zc *y, int *iy)
{ scipy_zgemv_(t, m, n, al, a, lda, x, ix, be, y, iy); }
void zimatcopy_(const char *o, const char *t, int *m, int *n, zc *al, zc *a, int *lda, int *ldb)
{ scipy_zimatcopy_(o, t, m, n, al, a, lda, ldb); }
