// Shared device helpers for the GB300 inverse-acoustics kernels.
//
// Complex numbers are double2 / float2 with (x = re, y = im), the same
// interleaved layout as the reference's cuDoubleComplex (CUDA/utils.cuh).
// Matrices are column-major; a batch of F matrices is stored back to back
// (frequency is the slowest index).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/ia.h"

#define IA_INV4PI 0.079577471545947667884

namespace ia {

// ---- debug builds: bounds checks on global-memory indexes ------------------
// Compiled with -DIA_DEBUG_BOUNDS (libia_debug.so), IA_IDX_OK(i, n) tests a
// global index against its buffer's extent before the access; the kernels
// skip an access whose test fails (a load then gives zero), and the first
// failing site of the translation unit (source line, index, extent) and the
// number of failures are recorded for ia_bounds_report().  A wrong index thus
// shows up as a report, not as a fault of a shared GPU.  In release builds
// IA_IDX_OK is the constant true and costs nothing.
struct IaBoundsSite {
    unsigned long long count;
    long long index, extent;
    int line, pad;
};
#ifdef IA_DEBUG_BOUNDS
static __device__ IaBoundsSite ia_tu_bounds;   // one per translation unit
__device__ __forceinline__ bool ia_idx_check(long long i, long long n, int line)
{
    if (i >= 0 && i < n) return true;
    if (atomicAdd(&ia_tu_bounds.count, 1ull) == 0ull) {
        ia_tu_bounds.index = i;
        ia_tu_bounds.extent = n;
        ia_tu_bounds.line = line;
    }
    return false;
}
#define IA_IDX_OK(i, n) (::ia::ia_idx_check((long long)(i), (long long)(n), __LINE__))
// reads (and clears) this translation unit's record
#define IA_BOUNDS_READER(fn)                                                                  \
    int fn(IaBoundsSite *out)                                                                 \
    {                                                                                         \
        IaBoundsSite z{};                                                                     \
        if (cudaMemcpyFromSymbol(out, ia_tu_bounds, sizeof(IaBoundsSite)) != cudaSuccess)    \
            return IA_ERR_CUDA;                                                               \
        if (cudaMemcpyToSymbol(ia_tu_bounds, &z, sizeof(IaBoundsSite)) != cudaSuccess)       \
            return IA_ERR_CUDA;                                                               \
        return IA_OK;                                                                         \
    }
#else
#define IA_IDX_OK(i, n) true
#define IA_BOUNDS_READER(fn)                                                                  \
    int fn(IaBoundsSite *out)                                                                 \
    {                                                                                         \
        *out = IaBoundsSite{};                                                                \
        return IA_OK;                                                                         \
    }
#endif

struct z64 { double re, im; };

__host__ __device__ __forceinline__ double2 zmake(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 zmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__host__ __device__ __forceinline__ double2 zmulc(double2 a, double2 b)
{
    return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// conj(a) * b
__host__ __device__ __forceinline__ double2 zcmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ double2 zscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ __forceinline__ double zabs2(double2 a) { return a.x * a.x + a.y * a.y; }
// acc += a * b
__device__ __forceinline__ void zfma(double2 &acc, double2 a, double2 b)
{
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
// acc -= a * b
__device__ __forceinline__ void zfms(double2 &acc, double2 a, double2 b)
{
    acc.x = fma(-a.x, b.x, acc.x);
    acc.x = fma(a.y, b.y, acc.x);
    acc.y = fma(-a.x, b.y, acc.y);
    acc.y = fma(-a.y, b.x, acc.y);
}
// acc += conj(a) * b
__device__ __forceinline__ void zcfma(double2 &acc, double2 a, double2 b)
{
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(-a.y, b.x, acc.y);
}
__device__ __forceinline__ double2 zdiv(double2 a, double2 b)
{
    // Smith-free scaled division; b is never tiny here (pivots, norms)
    double s = 1.0 / (b.x * b.x + b.y * b.y);
    return make_double2((a.x * b.x + a.y * b.y) * s, (a.y * b.x - a.x * b.y) * s);
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double2 warp_sum2(double2 v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// ---- single-precision complex (float2) overloads of the same helpers
__host__ __device__ __forceinline__ float2 zadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 zsub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 zmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 zscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ float2 zconj(float2 a) { return make_float2(a.x, -a.y); }
__host__ __device__ __forceinline__ float zabs2(float2 a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ void zfma(float2 &acc, float2 a, float2 b)
{
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(-a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(a.y, b.x, acc.y);
}
__device__ __forceinline__ void zfms(float2 &acc, float2 a, float2 b)
{
    acc.x = fmaf(-a.x, b.x, acc.x);
    acc.x = fmaf(a.y, b.y, acc.x);
    acc.y = fmaf(-a.x, b.y, acc.y);
    acc.y = fmaf(-a.y, b.x, acc.y);
}
__device__ __forceinline__ void zcfma(float2 &acc, float2 a, float2 b)
{
    acc.x = fmaf(a.x, b.x, acc.x);
    acc.x = fmaf(a.y, b.y, acc.x);
    acc.y = fmaf(a.x, b.y, acc.y);
    acc.y = fmaf(-a.y, b.x, acc.y);
}
__device__ __forceinline__ float2 zdiv(float2 a, float2 b)
{
    float s = 1.0f / (b.x * b.x + b.y * b.y);
    return make_float2((a.x * b.x + a.y * b.y) * s, (a.y * b.x - a.x * b.y) * s);
}
__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float2 warp_sum2(float2 v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
}

// complex element type -> real type, constructor
template <class T> struct ctraits;
template <> struct ctraits<double2> {
    typedef double R;
    __host__ __device__ static double2 make(double r, double i) { return make_double2(r, i); }
};
template <> struct ctraits<float2> {
    typedef float R;
    __host__ __device__ static float2 make(float r, float i) { return make_float2(r, i); }
};

// exp(i*t) / r
__device__ __forceinline__ double2 green(double kr, double invr)
{
    double s, c;
    sincos(kr, &s, &c);
    return make_double2(c * invr, s * invr);
}

}  // namespace ia
