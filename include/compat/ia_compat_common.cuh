// Shared glue of the drop-in headers in include/compat/: the reference's
// constant macros with their defaults (CUDA/constants.cuh:1-12, still
// overridable with -D), and the status -> exception mapping that mirrors the
// reference's CUDA_CHECK / CUSOLVER_CHECK behaviour (CUDA/cusolver_utils.cuh:30-58).
#pragma once
#include <cuComplex.h>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include "ia.h"

#ifndef C_AIR
#define C_AIR 343.5
#endif
#ifndef RHO_AIR
#define RHO_AIR 1.19
#endif
#ifndef MAX_LINE
#define MAX_LINE 4098
#endif
#ifndef BLOCK
#define BLOCK 512
#endif

static_assert(sizeof(ia_complex) == sizeof(cuDoubleComplex), "ia_complex must match cuDoubleComplex");

inline ia_config ia_compat_config()
{
    ia_config cfg;
    ia_config_default(&cfg);
    cfg.c = C_AIR;
    cfg.rho = RHO_AIR;
    return cfg;
}

inline void ia_compat_check(int status, const char *where)
{
    if (status != IA_OK) {
        std::printf("%s: %s (ia_status %d)\n", where, ia_status_string(status), status);
        throw std::runtime_error(where);
    }
}

// copy a device array to a new host buffer (for the *gpu entry points, whose
// coordinates live on the device)
template <class T>
inline T *ia_compat_to_host(const T *d, size_t count)
{
    T *h = (T *)std::malloc(sizeof(T) * (count ? count : 1));
    if (!h) throw std::runtime_error("malloc");
    if (cudaMemcpy(h, d, sizeof(T) * count, cudaMemcpyDeviceToHost) != cudaSuccess) {
        std::free(h);
        throw std::runtime_error("CUDA error");
    }
    return h;
}
