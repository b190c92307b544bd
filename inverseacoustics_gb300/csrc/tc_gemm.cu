// Tensor-core complex GEMM at FP64-level accuracy: C = alpha op(A) op(B) +
// beta C on GB300's BF16 tcgen05 pipe, by the Ozaki scheme (Ozaki, Ogita,
// Oishi, Rump 2012: error-free splitting of the operands into slices whose
// products sum exactly in floating point).
//
// Slicing.  Each row of op(A) and each column of op(B) gets a power-of-two
// scale 2^e above its largest real or imaginary part; a value v becomes the
// integer X = rint(v 2^(5 - e + 6 (S - 1))), |X| < 2^(5 + 6 (S - 1)), written
// as S balanced base-64 digits d_0 .. d_{S-1} in [-32, 32] (most significant
// first).  Every digit is exact in BF16.  The complex product is carried as a
// real one: a row of A becomes [Re a_0, Im a_0, Re a_1, ...] (2K values), and
// complex column n of B becomes two real columns, [Re b, -Im b] (giving
// Re c) and [Im b, Re b] (giving Im c).
//
// Products.  For every slice pair (s, t) with s + t <= S - 1 the tensor core
// accumulates sum_k d_s(a) d_t(b) in FP32 into the TMEM accumulator of level
// L = s + t.  A level sums at most S products of |d d| <= 1024 over 2K terms:
// with S 1024 2K <= 2^24 every partial sum is an integer below 2^24, so the
// FP32 accumulation is exact whatever its rounding.  The epilogue combines
// the levels, sum_L 64^(S-1-L) lev_L, in 64-bit integers and scales the
// result by 2^(e_row + e_col - 10 - 6 (S - 1)).  The only errors are the
// rounding to S digits and the dropped pairs (s + t >= S): at most
// (4 S + 8) 2^(-6 S) of max|A_row| max|B_col| per product term, 8e-12 at
// S = 7 and 1.4e-13 at S = 8 (typical errors are far smaller) -- the
// double-float GEMM's level.
//
// Kernel.  One CTA per 128 output rows x 32 complex output columns of one
// batch entry; 128 threads.  Warp 0 (one lane) loads, per K step of 32 real
// values, all S slices of the A and B tiles with one 4-D TMA box each
// (64-byte swizzle) into a two-stage pipeline; warp 1 (one lane) issues the
// S (S + 1) / 2 pair MMAs (M = 128, N = 64, K = 16, two per stage) into S
// level accumulators of 64 TMEM columns each (512 columns at S = 8) and
// releases each stage with tcgen05.commit; then all four warps read the
// accumulators of their 32 rows (tcgen05.ld) and write C.  Every mbarrier
// wait is bounded; a wait that runs out sets IA_INFO_TIMEOUT in the batch
// entry's info word and the CTA skips its output.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <mutex>
#include "ia_common.cuh"
#include "ia_internal.h"
#include "tc_ptx.cuh"

namespace ia {

constexpr int TC_BM = 128;        // output rows per CTA (TMEM lanes)
constexpr int TC_BN = 64;         // real output columns per CTA (32 complex)
constexpr int TC_BK = 32;         // real K values per pipeline stage (64 bytes of BF16)
constexpr int TC_STAGES = 2;
constexpr int TC_THREADS = 128;
constexpr uint64_t TC_WAIT_NS = 2000000000ull;
constexpr uint32_t TC_A_SLICE = TC_BM * TC_BK * 2;   // bytes of one slice's A tile
constexpr uint32_t TC_B_SLICE = TC_BN * TC_BK * 2;

size_t tc_smem_bytes(int S) { return (size_t)TC_STAGES * S * (TC_A_SLICE + TC_B_SLICE) + 1024; }

// ---------------------------------------------------------------------------
// slicing
// ---------------------------------------------------------------------------
// largest |Re|, |Im| of an element as an order-preserving integer key, and the
// exponent e with max < 2^e from the largest key of a row
__device__ __forceinline__ unsigned long long abs_key(const double2 &v)
{
    const unsigned long long a = __double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFull;
    const unsigned long long b = __double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFull;
    return a > b ? a : b;
}
__device__ __forceinline__ unsigned long long abs_key(const float4 &v)
{
    // the high words carry the magnitude: |hi + lo| < 2^e whenever |hi| < 2^e
    const unsigned a = __float_as_uint(v.x) & 0x7FFFFFFFu, b = __float_as_uint(v.y) & 0x7FFFFFFFu;
    return a > b ? a : b;
}
__device__ __forceinline__ int key_exponent(unsigned long long k, const double2 *)
{
    return k ? (int)((k >> 52) & 0x7FF) - 1022 : 0;
}
__device__ __forceinline__ int key_exponent(unsigned long long k, const float4 *)
{
    return k ? (int)((k >> 23) & 0xFF) - 126 : 0;
}

// X = rint(v 2^q) for the real and imaginary parts (q: scale exponent)
__device__ __forceinline__ void to_fixed(const double2 &v, int q, long long &xr, long long &xi)
{
    const double sc = __longlong_as_double((long long)(q + 1023) << 52);
    xr = __double2ll_rn(v.x * sc);
    xi = __double2ll_rn(v.y * sc);
}
__device__ __forceinline__ void to_fixed(const float4 &v, int q, long long &xr, long long &xi)
{
    // (hi + lo) 2^q as rint(hi 2^q) + rint(lo 2^q): within one unit of the
    // fixed-point grid, with no FP64 instruction
    const float sc = __uint_as_float((unsigned)(q + 127) << 23);
    xr = __float2ll_rn(v.x * sc) + __float2ll_rn(v.z * sc);
    xi = __float2ll_rn(v.y * sc) + __float2ll_rn(v.w * sc);
}

__device__ __forceinline__ double2 load_conj(const double2 *X, size_t i, bool conj)
{
    double2 v = X[i];
    if (conj) v.y = -v.y;
    return v;
}
__device__ __forceinline__ float4 load_conj(const float4 *X, size_t i, bool conj)
{
    float4 v = X[i];
    if (conj) {
        v.y = -v.y;
        v.w = -v.w;
    }
    return v;
}

// balanced base-64 digits of X, most significant first
template <int S>
__device__ __forceinline__ void digits64(long long X, int (&d)[S])
{
#pragma unroll
    for (int s = S - 1; s >= 1; --s) {
        int r = (int)(X & 63);
        if (r > 32) r -= 64;
        d[s] = r;
        X = (X - r) >> 6;
    }
    d[0] = (int)X;
}

__device__ __forceinline__ __nv_bfloat162 bf2(int a, int b)
{
    return __floats2bfloat162_rn((float)a, (float)b);
}

// One CTA per 32 rows of the operand view V (R x K, element (r, k)); V is
// r-contiguous (V(r, k) = X[r + k ld]) or k-contiguous (X[k + r ld]), either
// optionally conjugated.  Writes planes [S][rows][Kp] (rows = R for the A
// role, 2 R for the B role) and e[r].  Two passes over the rows: the row
// maxima, then the digits (the second pass reads from L2).
constexpr int SL_ROWS = 32, SL_K = 64;

// One operand to slice (a launch can carry two, blockIdx.z picking one)
template <class Src>
struct SliceOp {
    const Src *X;
    int ld;
    long long sX;
    int R, conj, role_b, rcontig;
    __nv_bfloat16 *planes;
    int *exps;
};

template <class Src, int S>
__global__ void __launch_bounds__(256) tc_slice_kernel(SliceOp<Src> op0, SliceOp<Src> op1, int K, int Kp)
{
    __shared__ Src tile[SL_ROWS][SL_K + 1];
    const SliceOp<Src> &op = blockIdx.z ? op1 : op0;
    const int f = blockIdx.y, r0 = blockIdx.x * SL_ROWS, t = threadIdx.x;
    const int R = op.R, ld = op.ld, conj = op.conj, role_b = op.role_b;
    const bool RCONTIG = op.rcontig != 0;
    if (r0 >= R) return;   // the other operand's taller grid
    const Src *__restrict__ X = op.X + f * op.sX;
    __nv_bfloat16 *__restrict__ planes = op.planes;
    int *__restrict__ exps = op.exps;
    const int rows = role_b ? 2 * R : R;
    const size_t pstride = (size_t)rows * Kp;
    planes += (size_t)f * S * pstride;
    const int rr = t >> 3, kq = t & 7;
    const int Kh = Kp >> 1;   // complex columns of the padded planes
    auto load_tile = [&](int k0) {
        for (int e = t; e < SL_ROWS * SL_K; e += 256) {
            int r, kk;
            if (RCONTIG) {
                r = e & (SL_ROWS - 1);
                kk = e / SL_ROWS;
            } else {
                kk = e & (SL_K - 1);
                r = e / SL_K;
            }
            Src v = Src{};
            if (r0 + r < R && k0 + kk < K) {
                const size_t i = RCONTIG ? (size_t)(r0 + r) + (size_t)(k0 + kk) * ld
                                         : (size_t)(k0 + kk) + (size_t)(r0 + r) * ld;
                v = load_conj(X, i, conj != 0);
            }
            tile[r][kk] = v;
        }
    };
    unsigned long long key = 0;
    for (int k0 = 0; k0 < K; k0 += SL_K) {
        load_tile(k0);
        __syncthreads();
#pragma unroll
        for (int j = 0; j < SL_K / 8; ++j) {
            const unsigned long long kk = abs_key(tile[rr][kq + 8 * j]);
            key = kk > key ? kk : key;
        }
        __syncthreads();
    }
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
        key = ok > key ? ok : key;
    }
    const int e = key_exponent(key, (const Src *)nullptr);
    const int row = r0 + rr;
    if (kq == 0 && row < R) exps[(size_t)f * R + row] = e;
    const int q = 5 - e + 6 * (S - 1);
    for (int k0 = 0; k0 < Kh; k0 += SL_K) {
        load_tile(k0);
        __syncthreads();
        if (row < R) {
#pragma unroll 2
            for (int j = 0; j < SL_K / 8; ++j) {
                const int kk = kq + 8 * j, k = k0 + kk;
                if (k >= Kh) break;
                long long xr, xi;
                to_fixed(tile[rr][kk], q, xr, xi);
                int dr[S], di[S];
                digits64<S>(xr, dr);
                digits64<S>(xi, di);
#pragma unroll
                for (int s = 0; s < S; ++s) {
                    __nv_bfloat16 *P = planes + (size_t)s * pstride + 2 * (size_t)k;
                    if (!role_b) {
                        *reinterpret_cast<__nv_bfloat162 *>(P + (size_t)row * Kp) = bf2(dr[s], di[s]);
                    } else {
                        *reinterpret_cast<__nv_bfloat162 *>(P + (size_t)(2 * row) * Kp) = bf2(dr[s], -di[s]);
                        *reinterpret_cast<__nv_bfloat162 *>(P + (size_t)(2 * row + 1) * Kp) = bf2(di[s], dr[s]);
                    }
                }
            }
        }
        __syncthreads();
    }
}

// Single-pass form: SL1_RB rows of the view per CTA, their K values read from
// global memory once into a shared-memory strip; warp w then takes row w: the
// row maximum from the strip, then the digits of two complex values per lane
// (8-byte plane stores, 256 bytes per warp and plane).  The same digits and
// exponents as the two-pass kernel above, which re-reads the operand for the
// digits (from DRAM once the operand outgrows L2); that kernel remains for
// rows longer than the strip allows.
constexpr int SL1_RB = 8, SL1_THREADS = 256, SL1_UNROLL = 4;

__host__ __device__ constexpr int sl1_stride(int Kh) { return Kh + 1; }   // odd in 16-byte units: no bank conflicts

__device__ __forceinline__ unsigned bf2_bits(__nv_bfloat162 v)
{
    return (unsigned)__bfloat16_as_ushort(v.x) | ((unsigned)__bfloat16_as_ushort(v.y) << 16);
}

template <class Src, int S>
__global__ void __launch_bounds__(SL1_THREADS, 2) tc_slice1_kernel(SliceOp<Src> op0, SliceOp<Src> op1, int K, int Kp)
{
    extern __shared__ __align__(16) unsigned char sl1_smem[];
    Src *strip = reinterpret_cast<Src *>(sl1_smem);   // SL1_RB rows x sl1_stride(Kh)
    const SliceOp<Src> &op = blockIdx.z ? op1 : op0;
    const int f = blockIdx.y, r0 = blockIdx.x * SL1_RB, t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int R = op.R;
    if (r0 >= R) return;   // the other operand's taller grid
    const int Kh = Kp >> 1, ks = sl1_stride(Kh);
    const int nr = R - r0 < SL1_RB ? R - r0 : SL1_RB;
    const Src *__restrict__ X = op.X + f * op.sX;
    const bool conj = op.conj != 0;
    // extent of this entry's operand: K columns of ld (r-contiguous) or R rows of ld
    const long long xext = op.rcontig ? (long long)op.ld * K : (long long)op.ld * R;
    if (op.rcontig) {
        // V(r, k) = X[r + k ld]: the CTA's rows of one k are 8 contiguous
        // values; a warp covers 4 values of k per step
        const int r = lane & (SL1_RB - 1), kq = lane >> 3;
        for (int kb = 4 * w; kb < Kh; kb += 4 * (SL1_THREADS / 32) * SL1_UNROLL) {
            Src v[SL1_UNROLL];
#pragma unroll
            for (int u = 0; u < SL1_UNROLL; ++u) {
                const int k = kb + kq + 4 * (SL1_THREADS / 32) * u;
                v[u] = Src{};
                if (r < nr && k < K && IA_IDX_OK((r0 + r) + (long long)k * op.ld, xext))
                    v[u] = load_conj(X, (size_t)(r0 + r) + (size_t)k * op.ld, conj);
            }
#pragma unroll
            for (int u = 0; u < SL1_UNROLL; ++u) {
                const int k = kb + kq + 4 * (SL1_THREADS / 32) * u;
                if (k < Kh) strip[(size_t)r * ks + k] = v[u];
            }
        }
    } else {
        // V(r, k) = X[k + r ld]: a row is contiguous; warp w loads row w
        const Src *xr = X + (size_t)(r0 + w) * op.ld;
        for (int kb = lane; kb < Kh; kb += 32 * SL1_UNROLL) {
            Src v[SL1_UNROLL];
#pragma unroll
            for (int u = 0; u < SL1_UNROLL; ++u) {
                const int k = kb + 32 * u;
                v[u] = Src{};
                if (w < nr && k < K && IA_IDX_OK((long long)(r0 + w) * op.ld + k, xext))
                    v[u] = load_conj(xr, (size_t)k, conj);
            }
#pragma unroll
            for (int u = 0; u < SL1_UNROLL; ++u) {
                const int k = kb + 32 * u;
                if (k < Kh) strip[(size_t)w * ks + k] = v[u];
            }
        }
    }
    __syncthreads();
    if (w >= nr) return;
    const Src *srow = strip + (size_t)w * ks;
    unsigned long long key = 0;
    for (int k = lane; k < K; k += 32) {
        const unsigned long long kk = abs_key(srow[k]);
        key = kk > key ? kk : key;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
        key = ok > key ? ok : key;
    }
    const int e = key_exponent(key, (const Src *)nullptr);
    const int row = r0 + w;
    if (lane == 0) op.exps[(size_t)f * R + row] = e;
    const int q = 5 - e + 6 * (S - 1);
    const int rows = op.role_b ? 2 * R : R;
    const size_t pstride = (size_t)rows * Kp;
    __nv_bfloat16 *__restrict__ planes = op.planes + (size_t)f * S * pstride;
    for (int k = 2 * lane; k < Kh; k += 64) {
        // two complex values (k, k + 1); Kh is a multiple of 4
        long long x[4];
        to_fixed(srow[k], q, x[0], x[1]);
        to_fixed(srow[k + 1], q, x[2], x[3]);
        // digits least significant first (digits64's order), each plane
        // written as soon as its four digits exist
#pragma unroll
        for (int s = S - 1; s >= 0; --s) {
            int d[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (s > 0) {
                    int r = (int)(x[j] & 63);
                    if (r > 32) r -= 64;
                    d[j] = r;
                    x[j] = (x[j] - r) >> 6;
                } else {
                    d[j] = (int)x[j];
                }
            }
            __nv_bfloat16 *P = planes + (size_t)s * pstride + 2 * (size_t)k;
            const long long pext = (long long)S * pstride;   // this entry's planes
            if (!op.role_b) {
                uint2 u;
                u.x = bf2_bits(bf2(d[0], d[1]));
                u.y = bf2_bits(bf2(d[2], d[3]));
                if (IA_IDX_OK((long long)s * pstride + (long long)row * Kp + 2 * k + 3, pext))
                    *reinterpret_cast<uint2 *>(P + (size_t)row * Kp) = u;
            } else if (IA_IDX_OK((long long)s * pstride + (long long)(2 * row + 1) * Kp + 2 * k + 3, pext)) {
                uint2 u0, u1;
                u0.x = bf2_bits(bf2(d[0], -d[1]));
                u0.y = bf2_bits(bf2(d[2], -d[3]));
                u1.x = bf2_bits(bf2(d[1], d[0]));
                u1.y = bf2_bits(bf2(d[3], d[2]));
                *reinterpret_cast<uint2 *>(P + (size_t)(2 * row) * Kp) = u0;
                *reinterpret_cast<uint2 *>(P + (size_t)(2 * row + 1) * Kp) = u1;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// the tensor-core GEMM on slice planes
// ---------------------------------------------------------------------------
template <int S>
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N,
                   int Kp, const int *__restrict__ ea, const int *__restrict__ eb, double alpha, double beta,
                   double2 *__restrict__ C, int ldc, long long sC, int *info)
{
    static_assert(S * TC_BN <= 512, "the S level accumulators must fit the 512 TMEM columns");
    constexpr uint32_t STAGE = S * (TC_A_SLICE + TC_B_SLICE);
    extern __shared__ unsigned char tc_smem_raw[];
    __shared__ __align__(8) uint64_t bar_full[TC_STAGES], bar_empty[TC_STAGES], bar_done;
    __shared__ uint32_t s_tmem;
    __shared__ volatile int s_abort;
    __shared__ double s_colscale[TC_BN / 2];
    unsigned char *base = reinterpret_cast<unsigned char *>(((uintptr_t)tc_smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t base_u = tc::smem_u32(base);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int f = blockIdx.z, m0 = blockIdx.y * TC_BM, c0 = blockIdx.x * TC_BN;
    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; ++s) {
            tc::mbar_init(tc::smem_u32(&bar_full[s]), 1);
            tc::mbar_init(tc::smem_u32(&bar_empty[s]), 1);
        }
        tc::mbar_init(tc::smem_u32(&bar_done), 1);
        s_abort = 0;
        tc::mbar_fence_init();
        tc::prefetch_tmap(&tmA);
        tc::prefetch_tmap(&tmB);
    }
    if (warp == 2) tc::tmem_alloc(tc::smem_u32(&s_tmem), 512);
    if (threadIdx.x < TC_BN / 2) {
        const int n = c0 / 2 + threadIdx.x;
        s_colscale[threadIdx.x] = n < N ? ldexp(1.0, eb[(size_t)f * N + n]) : 0.0;
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = s_tmem;
    const int nkb = (Kp + TC_BK - 1) / TC_BK;

    if (warp == 0 && lane == 0) {
        // producer: all S slices of the A and B tiles of one K step per stage
        int issued = 0;
        for (int kb = 0; kb < nkb && !s_abort; ++kb) {
            const int s = kb % TC_STAGES;
            const uint32_t ph = (uint32_t)(kb / TC_STAGES) & 1u;
            if (kb >= TC_STAGES && !tc::mbar_wait(tc::smem_u32(&bar_empty[s]), ph ^ 1u, TC_WAIT_NS)) {
                s_abort = 1;
                break;
            }
            const uint32_t full = tc::smem_u32(&bar_full[s]);
            tc::mbar_arrive_expect_tx(full, STAGE);
            const uint32_t a = base_u + (uint32_t)s * STAGE;
            tc::tma_load_4d(a, &tmA, kb * TC_BK, m0, 0, f, full);
            tc::tma_load_4d(a + S * TC_A_SLICE, &tmB, kb * TC_BK, c0, 0, f, full);
            issued = kb + 1;
        }
        if (s_abort) {
            // let this CTA's copies in flight land before the CTA ends
            for (int kb = issued - TC_STAGES > 0 ? issued - TC_STAGES : 0; kb < issued; ++kb)
                tc::mbar_wait(tc::smem_u32(&bar_full[kb % TC_STAGES]), (uint32_t)(kb / TC_STAGES) & 1u, TC_WAIT_NS);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: level L = s + t accumulates in TMEM columns [64 L, 64 L + 64)
        constexpr uint32_t idesc = tc::idesc_bf16_f32(TC_BM, TC_BN);
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % TC_STAGES;
            const uint32_t ph = (uint32_t)(kb / TC_STAGES) & 1u;
            if (s_abort || !tc::mbar_wait(tc::smem_u32(&bar_full[s]), ph, TC_WAIT_NS)) {
                s_abort = 1;
                break;
            }
            tc::tc_fence_after();
            const uint32_t a = base_u + (uint32_t)s * STAGE, b = a + S * TC_A_SLICE;
#pragma unroll
            for (int kk = 0; kk < TC_BK / 16; ++kk) {
#pragma unroll
                for (int i = 0; i < S; ++i) {
                    const uint64_t ad = tc::sdesc(a + i * TC_A_SLICE + kk * 32, 512, 4);
#pragma unroll
                    for (int j = 0; j + i < S; ++j) {
                        const uint64_t bd = tc::sdesc(b + j * TC_B_SLICE + kk * 32, 512, 4);
                        tc::mma_bf16(tmem + (uint32_t)((i + j) * TC_BN), ad, bd, idesc,
                                     (kb | kk | i) != 0 ? 1u : 0u);
                    }
                }
            }
            tc::mma_commit(tc::smem_u32(&bar_empty[s]));
        }
        tc::mma_commit(tc::smem_u32(&bar_done));
    }
    __syncwarp();
    const bool done = tc::mbar_wait(tc::smem_u32(&bar_done), 0, 2 * TC_WAIT_NS);
    __syncwarp();
    tc::tc_fence_after();
    const bool ok = done && !s_abort;
    if (!ok && threadIdx.x == 0 && info) atomicOr(info + f, IA_INFO_TIMEOUT);

    // epilogue: this thread's row, 16 real columns (8 complex) at a time
    const int row = m0 + warp * 32 + lane;
    const double rs = row < M ? ldexp(alpha, ea[(size_t)f * M + row] - 10 - 6 * (S - 1)) : 0.0;
    constexpr double TOP = (double)(1ll << (6 * (S - 1)));
    double2 *Cf = C + f * sC;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int ch = 0; ch < TC_BN / 16; ++ch) {
        uint32_t v[S][16];
#pragma unroll
        for (int L = 0; L < S; ++L) tc::tmem_ld16(lane_base + (uint32_t)(L * TC_BN + ch * 16), v[L]);
        tc::tmem_wait_ld();
        if (!ok || row >= M) continue;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int n = c0 / 2 + ch * 8 + q;
            if (n >= N) break;
            double part[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int j = 2 * q + h;
                long long acc = 0;
#pragma unroll
                for (int L = 1; L < S; ++L) acc = acc * 64 + (long long)__float2int_rn(__uint_as_float(v[L][j]));
                part[h] = fma((double)__float2int_rn(__uint_as_float(v[0][j])), TOP, (double)acc);
            }
            const double sc = rs * s_colscale[ch * 8 + q];
            double2 out = make_double2(part[0] * sc, part[1] * sc);
            double2 *p = Cf + row + (size_t)n * ldc;
            if (beta != 0.0) {
                const double2 old = *p;
                out.x = fma(beta, old.x, out.x);
                out.y = fma(beta, old.y, out.y);
            }
            *p = out;
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 2) tc::tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_encode_once;
cudaError_t g_encode_err = cudaSuccess;

int encode_fn(PFN_cuTensorMapEncodeTiled_v12000 *out)
{
    std::call_once(g_encode_once, [] {
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        g_encode_err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (g_encode_err == cudaSuccess && q != cudaDriverEntryPointSuccess) g_encode_err = cudaErrorNotSupported;
        g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    if (g_encode_err != cudaSuccess || !g_encode) return cuda_status(g_encode_err ? g_encode_err : cudaErrorNotSupported);
    *out = g_encode;
    return IA_OK;
}

// 4-D map over planes [batch][S][rows][Kp] (BF16), box (32, box_rows, S, 1),
// 64-byte swizzle
int make_tmap(CUtensorMap *tm, const __nv_bfloat16 *planes, int Kp, int rows, int S, int batch, int box_rows)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc;
    int st = encode_fn(&enc);
    if (st) return st;
    const cuuint64_t dims[4] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)S, (cuuint64_t)batch};
    const cuuint64_t strides[3] = {(cuuint64_t)Kp * 2, (cuuint64_t)rows * Kp * 2, (cuuint64_t)S * rows * Kp * 2};
    const cuuint32_t box[4] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows, (cuuint32_t)S, 1};
    const cuuint32_t es[4] = {1, 1, 1, 1};
    CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16 *>(planes), dims, strides, box,
                     es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? IA_OK : IA_ERR_CUDA;
}

template <int S>
int gemm_launch(ia_context *ctx, const CUtensorMap &ta, const CUtensorMap &tb, const TcPlanes &A, const TcPlanes &B,
                int M, int N, double alpha, double beta, double2 *C, int ldc, long long sC, int batch, int *info)
{
    const size_t smem = tc_smem_bytes(S);
    IA_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((2 * N + TC_BN - 1) / TC_BN, (M + TC_BM - 1) / TC_BM, batch);
    tc_gemm_kernel<S><<<grid, TC_THREADS, smem, ctx->stream>>>(ta, tb, M, N, A.Kp, A.e, B.e, alpha, beta, C, ldc, sC,
                                                                info);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

template <class Src, int S>
int slice_launch(ia_context *ctx, const SliceOp<Src> &a, const SliceOp<Src> *b, int K, int Kp, int batch)
{
    const int rmax = b && b->R > a.R ? b->R : a.R;
    const size_t smem1 = sizeof(Src) * SL1_RB * (size_t)sl1_stride(Kp >> 1);
    if (smem1 <= 200 * 1024) {
        if (smem1 > 48 * 1024)
            IA_CUDA_TRY(cudaFuncSetAttribute(tc_slice1_kernel<Src, S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem1));
        dim3 grid((rmax + SL1_RB - 1) / SL1_RB, batch, b ? 2 : 1);
        tc_slice1_kernel<Src, S><<<grid, SL1_THREADS, smem1, ctx->stream>>>(a, b ? *b : a, K, Kp);
        IA_LAUNCH_CHECK(ctx);
        return IA_OK;
    }
    dim3 grid((rmax + SL_ROWS - 1) / SL_ROWS, batch, b ? 2 : 1);
    tc_slice_kernel<Src, S><<<grid, 256, 0, ctx->stream>>>(a, b ? *b : a, K, Kp);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

// the operand descriptor and plane allocation of one operand
template <class Src>
int slice_prepare(bool role_b, Op op, const Src *X, int ld, long long sX, int R, int K, int S, int batch,
                  TcPlanes &out, WsCursor &cur, SliceOp<Src> &d)
{
    if (R < 1 || K < 1 || batch < 1 || S < TC_SLICES_MIN || S > TC_SLICES_MAX) return IA_ERR_ARG;
    const int Kp = (2 * K + 7) & ~7;
    if ((long long)S * 1024 * Kp > (1ll << 24)) return IA_ERR_TOO_LARGE;   // level sums would leave FP32's exact range
    const int rows = role_b ? 2 * R : R;
    out.R = R;
    out.rows = rows;
    out.Kp = Kp;
    out.S = S;
    out.p = cur.take<__nv_bfloat16>((size_t)batch * S * rows * Kp);
    out.e = cur.take<int>((size_t)batch * R);
    if (cur.off > cur.cap) return IA_ERR_ALLOC;
    // view V(r, k): the A role reads rows of op(A), the B role columns of op(B)
    d = SliceOp<Src>{X, ld, sX, R, op == OP_C ? 1 : 0, role_b ? 1 : 0, (role_b ? op != OP_N : op == OP_N) ? 1 : 0,
                     out.p, out.e};
    return IA_OK;
}

template <class Src>
int slice_dispatch(ia_context *ctx, int S, const SliceOp<Src> &a, const SliceOp<Src> *b, int K, int Kp, int batch)
{
    switch (S) {
    case 6: return slice_launch<Src, 6>(ctx, a, b, K, Kp, batch);
    case 7: return slice_launch<Src, 7>(ctx, a, b, K, Kp, batch);
    default: return slice_launch<Src, 8>(ctx, a, b, K, Kp, batch);
    }
}

template <class Src>
int slice_any(ia_context *ctx, bool role_b, Op op, const Src *X, int ld, long long sX, int R, int K, int S, int batch,
              TcPlanes &out, WsCursor &cur)
{
    SliceOp<Src> d;
    const int st = slice_prepare<Src>(role_b, op, X, ld, sX, R, K, S, batch, out, cur, d);
    if (st) return st;
    return slice_dispatch<Src>(ctx, S, d, nullptr, K, out.Kp, batch);
}

}  // namespace

size_t tc_planes_bytes(int R, int K, int S, bool role_b, int batch)
{
    const size_t Kp = (size_t)((2 * K + 7) & ~7), rows = role_b ? 2 * (size_t)R : (size_t)R;
    return ws_round(2 * (size_t)batch * S * rows * Kp) + ws_round(4 * (size_t)batch * R);
}

int tc_slice(ia_context *ctx, bool role_b, Op op, const double2 *X, int ld, long long sX, int R, int K, int S,
             int batch, TcPlanes &out, WsCursor &cur)
{
    return slice_any<double2>(ctx, role_b, op, X, ld, sX, R, K, S, batch, out, cur);
}

int tc_slice(ia_context *ctx, bool role_b, Op op, const float4 *X, int ld, long long sX, int R, int K, int S,
             int batch, TcPlanes &out, WsCursor &cur)
{
    return slice_any<float4>(ctx, role_b, op, X, ld, sX, R, K, S, batch, out, cur);
}

int tc_slice_pair(ia_context *ctx, Op opa, const double2 *A, int lda, long long sA, int M, Op opb, const double2 *B,
                  int ldb, long long sB, int N, int K, int S, int batch, TcPlanes &pa, TcPlanes &pb, WsCursor &cur)
{
    SliceOp<double2> da, db;
    int st = slice_prepare<double2>(false, opa, A, lda, sA, M, K, S, batch, pa, cur, da);
    if (!st) st = slice_prepare<double2>(true, opb, B, ldb, sB, N, K, S, batch, pb, cur, db);
    if (st) return st;
    return slice_dispatch<double2>(ctx, S, da, &db, K, pa.Kp, batch);
}

int tc_gemm(ia_context *ctx, const TcPlanes &A, const TcPlanes &B, int M, int N, double alpha, double beta,
            double2 *C, int ldc, long long sC, int batch, int *info)
{
    if (M <= 0 || N <= 0 || batch <= 0) return IA_OK;
    if (A.S != B.S || A.Kp != B.Kp || A.R != M || B.R != N || A.rows != M || B.rows != 2 * N) return IA_ERR_ARG;
    CUtensorMap ta, tb;
    int st = make_tmap(&ta, A.p, A.Kp, A.rows, A.S, batch, TC_BM);
    if (!st) st = make_tmap(&tb, B.p, B.Kp, B.rows, B.S, batch, TC_BN);
    if (st) return st;
    switch (A.S) {
    case 6: return gemm_launch<6>(ctx, ta, tb, A, B, M, N, alpha, beta, C, ldc, sC, batch, info);
    case 7: return gemm_launch<7>(ctx, ta, tb, A, B, M, N, alpha, beta, C, ldc, sC, batch, info);
    case 8: return gemm_launch<8>(ctx, ta, tb, A, B, M, N, alpha, beta, C, ldc, sC, batch, info);
    default: return IA_ERR_ARG;
    }
}

IA_BOUNDS_READER(bounds_read_tc)

}  // namespace ia

using namespace ia;

// Batched complex GEMM with FP64 operands and output (the reference's
// cublasZgemm, CUDA/ibem.cuh:398): IA_PREC_FP64 runs the FP64 CUDA-core GEMM,
// IA_PREC_MIXED the sliced tensor-core GEMM with `slices` BF16 slices per
// operand (0: the default).  Workspace from the context.
extern "C" int ia_zgemm_batch(ia_context *ctx, int opa, int opb, int M, int N, int K, double alpha,
                              const ia_complex *d_A, int lda, long long sA, const ia_complex *d_B, int ldb,
                              long long sB, double beta, ia_complex *d_C, int ldc, long long sC, int batch,
                              int precision, int slices, int *d_info)
{
    if (!ctx || M < 1 || N < 1 || K < 1 || batch < 1 || !d_A || !d_B || !d_C) return IA_ERR_ARG;
    if (opa < OP_N || opa > OP_C || opb < OP_N || opb > OP_C) return IA_ERR_ARG;
    if (precision == IA_PREC_FP64) {
        return zgemm_batched(ctx, (Op)opa, (Op)opb, M, N, K, make_double2(alpha, 0.0), (const double2 *)d_A, lda, sA,
                             (const double2 *)d_B, ldb, sB, make_double2(beta, 0.0), (double2 *)d_C, ldc, sC, batch);
    }
    if (precision != IA_PREC_MIXED) return IA_ERR_ARG;
    const int S = slices ? slices : TC_SLICES_DEFAULT;
    if (S < TC_SLICES_MIN || S > TC_SLICES_MAX) return IA_ERR_ARG;
    const size_t need = tc_planes_bytes(M, K, S, false, batch) + tc_planes_bytes(N, K, S, true, batch) + 1024;
    int st = ws_reserve(ctx, need);
    if (st) return st;
    WsCursor cur{(char *)ctx->ws, 0, ctx->ws_bytes};
    TcPlanes A, B;
    if ((st = tc_slice(ctx, false, (Op)opa, (const double2 *)d_A, lda, sA, M, K, S, batch, A, cur))) return st;
    if ((st = tc_slice(ctx, true, (Op)opb, (const double2 *)d_B, ldb, sB, N, K, S, batch, B, cur))) return st;
    return tc_gemm(ctx, A, B, M, N, alpha, beta, (double2 *)d_C, ldc, sC, batch, d_info);
}
