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

// exp(i*t) / r
__device__ __forceinline__ double2 green(double kr, double invr)
{
    double s, c;
    sincos(kr, &s, &c);
    return make_double2(c * invr, s * invr);
}

}  // namespace ia
