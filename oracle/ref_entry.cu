// Translation unit that compiles the reference's own CPU path (header-only
// CUDA/*.cuh of LuisCorralR/InverseAcoustics) into oracle/_ref/libiaref.so.
//
// Test infrastructure only: nothing on the product path links or loads this.
// The reference headers are included from where they lie (-I<reference>/CUDA);
// no reference source is copied into this repository.  The headers need their
// includes in a fixed order and use CUDA_CHECK / C_AIR without including the
// files that define them (CUDA/cusolver_utils.cuh:30, CUDA/constants.cuh:2).
//
// Exported (C linkage, defined by the reference):
//   esm   CUDA/esm.cuh:112     ibem  CUDA/ibem.cuh:424     invr  CUDA/invr.cuh:457
// Exported (C linkage, thin adapters defined here):
//   ref_sphere          -> sphere                CUDA/utils.cuh:384
//   ref_cart2sph        -> cartesian_2_spherical CUDA/utils.cuh:414
//   ref_geometry        -> geometry (gmsh v2.2)  CUDA/utils.cuh:291
//   ref_free            -> free() for the callee-malloc'd outputs
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <stdexcept>
#include <cuComplex.h>
#include <thrust/complex.h>
#include <cublas_v2.h>
#include <cusolverDn.h>

#include "cusolver_utils.cuh"
#include "constants.cuh"
#include "utils.cuh"
#include "esm.cuh"
#include "ibem.cuh"
#include "invr.cuh"

extern "C" void ref_sphere(double *r_ms, double *r_lh, cuDoubleComplex **p_s, cuDoubleComplex **p_h,
                           cuDoubleComplex **v_s, double k, double u, double a, int m, int l)
{
    sphere(r_ms, r_lh, p_s, p_h, v_s, k, u, a, m, l);
}

extern "C" void ref_cart2sph(int m, double *r_xx, double **azelr) { cartesian_2_spherical(m, r_xx, azelr); }

extern "C" void ref_geometry(const char *file, double k, double t, double **r_ms, double **r_lh, int **e_n, int *m,
                             int *l, int *n)
{
    geometry(r_ms, r_lh, e_n, k, t, m, l, n, const_cast<char *>(file));
}

extern "C" void ref_free(void *p) { free(p); }

extern "C" double ref_c_air(void) { return C_AIR; }
extern "C" double ref_rho_air(void) { return RHO_AIR; }
