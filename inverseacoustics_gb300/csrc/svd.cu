// Batched one-sided (Hestenes) Jacobi SVD, one CTA per frequency, templated
// on the element type (double2 for the FP64 path, float2 for the mixed path).
//
// Replaces cusolverDnZgesvd in csvd() (CUDA/tsvd.cuh:39,93) and the MATLAB
// svd() behind csvdG.m:17-24.  The columns of Y (M x N, M >= N) are
// orthogonalised pairwise with complex plane rotations; a round-robin
// (circle-method) ordering makes the N/2 pairs of a round disjoint, so each
// warp rotates one pair with no synchronisation inside a round.  Column dot
// products are warp-shuffle reductions in a fixed order, so repeated runs
// give identical results.  A pair is rotated while
// |y_i^H y_j| > sqrt(Mdot) eps ||y_i|| ||y_j||; the sweep loop ends after a
// sweep without rotations or at the sweep cap (IA_INFO_NOCONV).
//
// Only the first Mdot rows enter the dot products; rows Mdot..M-1 are rotated
// along (the pipeline keeps conj(b)^T there, so U^H b falls out of the
// rotations without forming U).
#include <cooperative_groups.h>
#include "ia_common.cuh"
#include "ia_internal.h"

namespace ia {

namespace cg = cooperative_groups;

constexpr int SVD_MAX_WARPS = 16;

__device__ __forceinline__ void rr_pair(int N2, int round, int k, int &i, int &j)
{
    if (k == 0) {
        i = round;
        j = N2 - 1;
    } else {
        // (round + k) mod (N2 - 1) and (round - k + N2 - 1) mod (N2 - 1):
        // both operands lie in [0, 2 (N2 - 1)), so one conditional
        // subtraction replaces the integer division
        i = round + k;
        if (i >= N2 - 1) i -= N2 - 1;
        j = round - k + N2 - 1;
        if (j >= N2 - 1) j -= N2 - 1;
    }
    if (i > j) { int t = i; i = j; j = t; }
}

// Rotation that zeroes y_i^H y_j for column norms a, b and product g.
template <class T, class R>
__device__ __forceinline__ bool jacobi_rotation(R a, R b, T g, R tol, R &c, T &sp, R *rel = nullptr)
{
    R gm = sqrt(g.x * g.x + g.y * g.y);
    const R sa = sqrt(a), sb = sqrt(b);
    if (!(gm > tol * sa * sb) || gm == 0) return false;
    if (rel) *rel = gm / (sa * sb);   // the relative coupling |y_i^H y_j| / (|y_i||y_j|)
    R zeta = (b - a) / (2 * gm);
    R t;
    if (fabs(zeta) > (R)1e30) t = (R)0.5 / zeta;
    else t = (zeta >= 0 ? (R)1 : (R)-1) / (fabs(zeta) + sqrt(1 + zeta * zeta));
    c = 1 / sqrt(1 + t * t);
    R s = t * c;
    sp = ctraits<T>::make(s * g.x / gm, s * g.y / gm);   // s' = s e^{i arg gamma}
    return true;
}

template <class T>
__device__ __forceinline__ void rotate_pair(T &u, T &v, typename ctraits<T>::R c, T sp)
{
    T nu = zscale(u, c), nv = zscale(v, c);
    zfms(nu, zconj(sp), v);
    zfma(nv, sp, u);
    u = nu;
    v = nv;
}

// KPL > 0: rows cached in registers (M <= 32*KPL); KPL == 0: streamed.
template <class T, int KPL>
__global__ void __launch_bounds__(SVD_MAX_WARPS * 32) jacobi_kernel(int M, int Mdot, int N, T *Y, long long sY, T *V,
                                                                      long long sV, int max_sweeps,
                                                                      typename ctraits<T>::R tol, int *info)
{
    typedef typename ctraits<T>::R R;
    __shared__ int s_rot;
    const int f = blockIdx.x;
    Y += f * sY;
    if (V) V += f * sV;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int N2 = N + (N & 1);
    const T zero = ctraits<T>::make(0, 0);
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        if (threadIdx.x == 0) s_rot = 0;
        __syncthreads();
        int rot_local = 0;
        for (int round = 0; round < N2 - 1; ++round) {
            for (int k = wid; k < N2 / 2; k += nw) {
                int i, j;
                rr_pair(N2, round, k, i, j);
                if (j >= N) continue;
                T *yi = Y + (size_t)i * M, *yj = Y + (size_t)j * M;
                R a = 0, b = 0, c;
                T g = zero, sp;
                if (KPL > 0) {
                    T ui[KPL > 0 ? KPL : 1], vj[KPL > 0 ? KPL : 1];
#pragma unroll
                    for (int t = 0; t < KPL; ++t) {
                        int r = lane + 32 * t;
                        ui[t] = r < M ? yi[r] : zero;
                        vj[t] = r < M ? yj[r] : zero;
                        if (r < Mdot) {
                            a += zabs2(ui[t]);
                            b += zabs2(vj[t]);
                            zcfma(g, ui[t], vj[t]);
                        }
                    }
                    a = warp_sum(a);
                    b = warp_sum(b);
                    g = warp_sum2(g);
                    if (!jacobi_rotation(a, b, g, tol, c, sp)) continue;
#pragma unroll
                    for (int t = 0; t < KPL; ++t) {
                        int r = lane + 32 * t;
                        if (r < M) {
                            rotate_pair(ui[t], vj[t], c, sp);
                            yi[r] = ui[t];
                            yj[r] = vj[t];
                        }
                    }
                } else {
                    for (int r = lane; r < Mdot; r += 32) {
                        T u = yi[r], v = yj[r];
                        a += zabs2(u);
                        b += zabs2(v);
                        zcfma(g, u, v);
                    }
                    a = warp_sum(a);
                    b = warp_sum(b);
                    g = warp_sum2(g);
                    if (!jacobi_rotation(a, b, g, tol, c, sp)) continue;
                    for (int r = lane; r < M; r += 32) {
                        T u = yi[r], v = yj[r];
                        rotate_pair(u, v, c, sp);
                        yi[r] = u;
                        yj[r] = v;
                    }
                }
                if (V) {
                    T *vi = V + (size_t)i * N, *vjp = V + (size_t)j * N;
                    for (int r = lane; r < N; r += 32) {
                        T u = vi[r], v = vjp[r];
                        rotate_pair(u, v, c, sp);
                        vi[r] = u;
                        vjp[r] = v;
                    }
                }
                rot_local++;
            }
            __syncthreads();
        }
        if (lane == 0 && rot_local) atomicAdd(&s_rot, rot_local);
        __syncthreads();
        int total = s_rot;
        __syncthreads();
        if (total == 0) break;
    }
    if (threadIdx.x == 0 && sweep >= max_sweeps && info) atomicOr(&info[f], IA_INFO_NOCONV);
}

// Same iteration with Y held in shared memory for the whole run (M x N small
// enough); V, when accumulated, stays in global memory and its two columns
// are fetched before the dot products so their latency overlaps them.
template <class T, int KPL>
__global__ void __launch_bounds__(sizeof(T) <= 8 ? 2 * SVD_MAX_WARPS * 32 : SVD_MAX_WARPS * 32)
    jacobi_smem_kernel(int M, int Mdot, int N, T *Yg, long long sY,
                                                                           T *V, long long sV, int max_sweeps,
                                                                           typename ctraits<T>::R tol, int *info)
{
    typedef typename ctraits<T>::R R;
    extern __shared__ __align__(16) unsigned char smraw[];
    T *Y = reinterpret_cast<T *>(smraw);
    __shared__ int s_rot;
    const int f = blockIdx.x;
    Yg += f * sY;
    if (V) V += f * sV;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int N2 = N + (N & 1);
    const T zero = ctraits<T>::make(0, 0);
    for (int e = threadIdx.x; e < M * N; e += blockDim.x) Y[e] = Yg[e];
    __syncthreads();
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        if (threadIdx.x == 0) s_rot = 0;
        __syncthreads();
        int rot_local = 0;
        for (int round = 0; round < N2 - 1; ++round) {
            for (int k = wid; k < N2 / 2; k += nw) {
                int i, j;
                rr_pair(N2, round, k, i, j);
                if (j >= N) continue;
                T vi[KPL], vj[KPL];
                T *gvi = V ? V + (size_t)i * N : nullptr, *gvj = V ? V + (size_t)j * N : nullptr;
                if (V) {
#pragma unroll
                    for (int t = 0; t < KPL; ++t) {
                        int r = lane + 32 * t;
                        vi[t] = r < N ? gvi[r] : zero;
                        vj[t] = r < N ? gvj[r] : zero;
                    }
                }
                T *yi = Y + (size_t)i * M, *yj = Y + (size_t)j * M;
                R a = 0, b = 0, c;
                T g = zero, sp;
                T ui[KPL], uj[KPL];
#pragma unroll
                for (int t = 0; t < KPL; ++t) {
                    int r = lane + 32 * t;
                    ui[t] = r < M ? yi[r] : zero;
                    uj[t] = r < M ? yj[r] : zero;
                    if (r < Mdot) {
                        a += zabs2(ui[t]);
                        b += zabs2(uj[t]);
                        zcfma(g, ui[t], uj[t]);
                    }
                }
                a = warp_sum(a);
                b = warp_sum(b);
                g = warp_sum2(g);
                if (!jacobi_rotation(a, b, g, tol, c, sp)) continue;
#pragma unroll
                for (int t = 0; t < KPL; ++t) {
                    int r = lane + 32 * t;
                    if (r < M) {
                        rotate_pair(ui[t], uj[t], c, sp);
                        yi[r] = ui[t];
                        yj[r] = uj[t];
                    }
                }
                if (V) {
#pragma unroll
                    for (int t = 0; t < KPL; ++t) {
                        int r = lane + 32 * t;
                        if (r < N) {
                            rotate_pair(vi[t], vj[t], c, sp);
                            gvi[r] = vi[t];
                            gvj[r] = vj[t];
                        }
                    }
                }
                rot_local++;
            }
            __syncthreads();
        }
        if (lane == 0 && rot_local) atomicAdd(&s_rot, rot_local);
        __syncthreads();
        int total = s_rot;
        __syncthreads();
        if (total == 0) break;
    }
    for (int e = threadIdx.x; e < M * N; e += blockDim.x) Yg[e] = Y[e];
    if (threadIdx.x == 0 && sweep >= max_sweeps && info) atomicOr(&info[f], IA_INFO_NOCONV);
}

// The shared-memory iteration with a half-warp per pair (M, N <= 128): each
// lane holds 8 rows of both columns, the sums reduce over 16 lanes, and a
// 32-warp CTA works all 64 pairs of a round at once instead of two pairs per
// warp one after the other.  Same rotation order as jacobi_smem_kernel.
template <class T>
__device__ __forceinline__ typename ctraits<T>::R half_sum(typename ctraits<T>::R v, unsigned mask)
{
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
    return v;
}

template <class T>
__global__ void __launch_bounds__(sizeof(T) <= 8 ? 1024 : 512)
    jacobi_half_kernel(int M, int Mdot, int N, T *Yg, long long sY, int max_sweeps, typename ctraits<T>::R tol,
                       int *info)
{
    typedef typename ctraits<T>::R R;
    constexpr int KPL = 8;
    extern __shared__ __align__(16) unsigned char smraw[];
    T *Y = reinterpret_cast<T *>(smraw);
    __shared__ int s_rot;
    __shared__ unsigned s_maxrel;   // largest |y_i^H y_j| / (|y_i||y_j|) rotated in the sweep (float bits)
    const int f = blockIdx.x;
    Yg += f * sY;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int half = lane >> 4, hl = lane & 15;
    const unsigned mask = half ? 0xffff0000u : 0x0000ffffu;
    const int N2 = N + (N & 1);
    const T zero = ctraits<T>::make(0, 0);
    for (int e = threadIdx.x; e < M * N; e += blockDim.x) Y[e] = Yg[e];
    __syncthreads();
    int sweep = 0;
    for (; sweep < max_sweeps; ++sweep) {
        if (threadIdx.x == 0) {
            s_rot = 0;
            s_maxrel = 0u;
        }
        __syncthreads();
        int rot_local = 0;
        float relmax = 0.f;
        for (int round = 0; round < N2 - 1; ++round) {
            for (int k = 2 * wid + half; k < N2 / 2; k += 2 * nw) {
                int i, j;
                rr_pair(N2, round, k, i, j);
                if (j >= N) continue;
                T *yi = Y + (size_t)i * M, *yj = Y + (size_t)j * M;
                R a = 0, b = 0, c;
                T g = zero, sp;
                T ui[KPL], uj[KPL];
#pragma unroll
                for (int t = 0; t < KPL; ++t) {
                    int r = hl + 16 * t;
                    ui[t] = r < M ? yi[r] : zero;
                    uj[t] = r < M ? yj[r] : zero;
                    if (r < Mdot) {
                        a += zabs2(ui[t]);
                        b += zabs2(uj[t]);
                        zcfma(g, ui[t], uj[t]);
                    }
                }
                a = half_sum<T>(a, mask);
                b = half_sum<T>(b, mask);
                g.x = half_sum<T>(g.x, mask);
                g.y = half_sum<T>(g.y, mask);
                R rel = 0;
                if (!jacobi_rotation(a, b, g, tol, c, sp, sizeof(R) == 4 ? &rel : nullptr)) continue;
                relmax = fmaxf(relmax, (float)rel);
#pragma unroll
                for (int t = 0; t < KPL; ++t) {
                    int r = hl + 16 * t;
                    if (r < M) {
                        rotate_pair(ui[t], uj[t], c, sp);
                        yi[r] = ui[t];
                        yj[r] = uj[t];
                    }
                }
                rot_local++;
            }
            __syncthreads();
        }
        if (hl == 0 && rot_local) {
            atomicAdd(&s_rot, rot_local);
            if (sizeof(R) == 4) atomicMax(&s_maxrel, __float_as_uint(relmax));
        }
        __syncthreads();
        const int total = s_rot;
        const float maxrel = __uint_as_float(s_maxrel);
        __syncthreads();
        if (total == 0) break;
        // FP32 (a start for the FP64-level refinement that follows): when the
        // largest rotated coupling of the sweep was below sqrt(tol) / 2, the
        // next sweep's couplings are below tol (quadratic convergence) and
        // would only confirm it -- skip that sweep.  FP64 runs to the test.
        if (sizeof(R) == 4 && maxrel < 0.5f * sqrtf((float)tol)) break;
    }
    for (int e = threadIdx.x; e < M * N; e += blockDim.x) Yg[e] = Y[e];
    if (threadIdx.x == 0 && sweep >= max_sweeps && info) atomicOr(&info[f], IA_INFO_NOCONV);
}

// The same iteration over a cluster of CS CTAs per bin (no accumulator).
// FP32: for latency, in small batches and the last part of a staggered
// pipeline, whose chain ends the pass.  FP64 (bound by the FP64 pipe of its
// SM): whenever the batch leaves SMs idle, CS = 2 or 4 CTAs per bin.  CTA q owns the pair slots
// [q P, (q + 1) P) of the circle ordering (P = N2 / 2 / JC_CS).  From one
// round to the next the ordering moves every "upper" column (slot k holds
// columns (r + k) and (r - k) mod (N2 - 1), column N2 - 1 fixed in slot 0)
// one slot down and every "lower" column one slot up; so a CTA keeps its
// columns in two rings of P + 1 entries indexed by slot +/- round, and per
// round only two columns cross to a neighbour CTA, written straight into its
// ring's free entry through distributed shared memory (slot 0's upper column
// turns into slot 1's lower one in CTA 0, the top slot's lower into its upper
// one in the last CTA).  One cluster barrier per round.  Per pair the
// arithmetic is jacobi_half_kernel's (a half-warp per pair, the same
// reductions, rotation and stopping rule; the sweep's rotation count and
// largest coupling are combined over the cluster), so the factors are
// bitwise the same.
template <class T, int JC_CS, int KPL = 8>
__global__ void __launch_bounds__(KPL <= 8 ? 512 : 256)
    jacobi_cluster_kernel(int M, int Mdot, int N, T *Yg, long long sY, int max_sweeps, typename ctraits<T>::R tol,
                          int *info)
{
    typedef typename ctraits<T>::R R;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int f = blockIdx.x / JC_CS;
    const int N2 = N + (N & 1), NR = N2 - 1, P = N2 / 2 / JC_CS, RING = P + 1, k0 = rank * P;
    extern __shared__ __align__(16) unsigned char jc_raw[];
    T *up = reinterpret_cast<T *>(jc_raw);   // RING x M: upper columns, entry (slot + t) mod RING
    T *lo = up + (size_t)RING * M;           // RING x M: lower columns, entry (slot - t) mod RING
    T *fixc = lo + (size_t)RING * M;         // M: column N2 - 1 (CTA 0)
    __shared__ int s_rot[2];
    __shared__ unsigned s_rel[2];
    Yg += f * sY;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int half = lane >> 4, hl = lane & 15, hw = 2 * wid + half;
    const unsigned mask = half ? 0xffff0000u : 0x0000ffffu;
    const T zero = ctraits<T>::make(0, 0);
    // columns of slot k at round r (k0 = 0 .. NP - 1)
    auto col_up = [&](int k, int r) { int c = r + k; return c >= NR ? c - NR : c; };
    auto col_lo = [&](int k, int r) { if (k == 0) return N2 - 1; int c = r - k; return c < 0 ? c + NR : c; };
    const long long yext = (long long)M * N;
    auto load_col = [&](T *dst, int c) {
        for (int i = threadIdx.x; i < M; i += blockDim.x)
            dst[i] = c < N && IA_IDX_OK((long long)c * M + i, yext) ? Yg[(size_t)c * M + i] : zero;
    };
    // round 0: slot k holds columns k and N2 - 1 - k (N2 - 1 in slot 0)
    for (int s = 0; s < P; ++s) {
        const int k = k0 + s;
        load_col(up + (size_t)s * M, col_up(k, 0));
        if (k == 0) load_col(fixc, N2 - 1);
        else load_col(lo + (size_t)s * M, col_lo(k, 0));
    }
    if (threadIdx.x == 0) {
        s_rot[0] = s_rot[1] = 0;
        s_rel[0] = s_rel[1] = 0u;
    }
    cluster.sync();
    int r = 0, t = 0, par = 0, sweep = 0;   // round mod NR, round mod RING
    for (; sweep < max_sweeps; ++sweep) {
        int rot_local = 0;
        float relmax = 0.f;
        for (int round = 0; round < NR; ++round) {
            const int tn = t + 1 == RING ? 0 : t + 1;
            for (int s = hw; s < P; s += 2 * nw) {
                const int k = k0 + s;
                const int cu = col_up(k, r), cl = col_lo(k, r);
                int eu = s + t;
                if (eu >= RING) eu -= RING;
                int el = s - t;
                if (el < 0) el += RING;
                T *pu = up + (size_t)eu * M, *pl = k == 0 ? fixc : lo + (size_t)el * M;
                const bool uf = cu < cl;   // the upper column is y_i
                T *yi = uf ? pu : pl, *yj = uf ? pl : pu;
                const int j = uf ? cl : cu;
                T ui[KPL], uj[KPL];
#pragma unroll
                for (int q = 0; q < KPL; ++q) {
                    const int rr = hl + 16 * q;
                    ui[q] = rr < M ? yi[rr] : zero;
                    uj[q] = rr < M ? yj[rr] : zero;
                }
                if (j < N) {
                    R a = 0, b = 0, c;
                    T g = zero, sp;
#pragma unroll
                    for (int q = 0; q < KPL; ++q) {
                        if (hl + 16 * q < Mdot) {
                            a += zabs2(ui[q]);
                            b += zabs2(uj[q]);
                            zcfma(g, ui[q], uj[q]);
                        }
                    }
                    a = half_sum<T>(a, mask);
                    b = half_sum<T>(b, mask);
                    g.x = half_sum<T>(g.x, mask);
                    g.y = half_sum<T>(g.y, mask);
                    R rel = 0;
                    if (jacobi_rotation(a, b, g, tol, c, sp, sizeof(R) == 4 ? &rel : nullptr)) {
                        relmax = fmaxf(relmax, (float)rel);
#pragma unroll
                        for (int q = 0; q < KPL; ++q) {
                            const int rr = hl + 16 * q;
                            if (rr < M) {
                                rotate_pair(ui[q], uj[q], c, sp);
                                yi[rr] = ui[q];
                                yj[rr] = uj[q];
                            }
                        }
                        rot_local++;
                    }
                }
                // the columns that leave this CTA's rings for the next round
                const T *vu = uf ? ui : uj, *vl = uf ? uj : ui;   // registers of the upper / lower column
                if (s == 0) {
                    T *dst;
                    if (rank > 0) {
                        int e = P - 1 + tn;
                        if (e >= RING) e -= RING;
                        dst = cluster.map_shared_rank(up, rank - 1) + (size_t)e * M;
                    } else {
                        int e = 1 - tn;
                        if (e < 0) e += RING;
                        dst = lo + (size_t)e * M;
                    }
#pragma unroll
                    for (int q = 0; q < KPL; ++q)
                        if (hl + 16 * q < M) dst[hl + 16 * q] = vu[q];
                }
                if (s == P - 1) {
                    T *dst;
                    if (rank < JC_CS - 1) {
                        int e = -tn;
                        if (e < 0) e += RING;
                        dst = cluster.map_shared_rank(lo, rank + 1) + (size_t)e * M;
                    } else {
                        int e = P - 1 + tn;
                        if (e >= RING) e -= RING;
                        dst = up + (size_t)e * M;
                    }
#pragma unroll
                    for (int q = 0; q < KPL; ++q)
                        if (hl + 16 * q < M) dst[hl + 16 * q] = vl[q];
                }
            }
            cluster.sync();
            t = tn;
            r = r + 1 == NR ? 0 : r + 1;
        }
        if (hl == 0 && rot_local) {
            atomicAdd(&s_rot[par], rot_local);
            if (sizeof(R) == 4) atomicMax(&s_rel[par], __float_as_uint(relmax));
        }
        cluster.sync();
        int total = 0;
        unsigned mr = 0u;
        for (int q = 0; q < JC_CS; ++q) {
            total += *cluster.map_shared_rank(&s_rot[par], q);
            const unsigned v = *cluster.map_shared_rank(&s_rel[par], q);
            mr = v > mr ? v : mr;
        }
        if (threadIdx.x == 0) {
            s_rot[par ^ 1] = 0;
            s_rel[par ^ 1] = 0u;
        }
        par ^= 1;
        if (total == 0) break;
        if (sizeof(R) == 4 && __uint_as_float(mr) < 0.5f * sqrtf((float)tol)) break;
    }
    cluster.sync();   // every CTA has read the others' counters
    // r is back at 0 after whole sweeps: the round-0 layout, entries shifted by t
    for (int s = 0; s < P; ++s) {
        const int k = k0 + s;
        int eu = s + t;
        if (eu >= RING) eu -= RING;
        int el = s - t;
        if (el < 0) el += RING;
        const int cu = col_up(k, r), cl = col_lo(k, r);
        const T *pu = up + (size_t)eu * M, *pl = k == 0 ? fixc : lo + (size_t)el * M;
        for (int i = threadIdx.x; i < M; i += blockDim.x) {
            if (cu < N && IA_IDX_OK((long long)cu * M + i, yext)) Yg[(size_t)cu * M + i] = pu[i];
            if (cl < N && IA_IDX_OK((long long)cl * M + i, yext)) Yg[(size_t)cl * M + i] = pl[i];
        }
    }
    if (rank == 0 && threadIdx.x == 0 && sweep >= max_sweeps && info) atomicOr(&info[f], IA_INFO_NOCONV);
}

template <class T>
__global__ void identity_kernel(int N, T *V, long long sV)
{
    const int f = blockIdx.y;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < N * N; e += gridDim.x * blockDim.x) {
        int r = e % N, c = e / N;
        V[f * sV + e] = ctraits<T>::make(r == c ? 1 : 0, 0);
    }
}

// ---- GPU-wide Jacobi for large systems (M > 256) ------------------------
// One launch per round of the circle ordering, one CTA per (pair, bin), so a
// few large systems (the 642 x 642 G Z of the drop-in invr() with n_am = m)
// spread over every SM instead of holding one SM each through ~10 sweeps of
// 641 rounds.  A bin's CTAs skip the rounds of a sweep once its previous sweep
// rotated nothing; the host reads the per-sweep total after each sweep (one
// synchronisation per sweep) and stops when every bin is done.  Same
// rotations, tolerance and ordering as the one-CTA kernels; the column dot
// products reduce over the CTA in a fixed order.
constexpr int WIDE_THREADS = 256;

template <class T>
__global__ void __launch_bounds__(WIDE_THREADS)
    jacobi_round_kernel(int M, int Mdot, int N, T *Y, long long sY, T *V, long long sV, int round,
                        typename ctraits<T>::R tol, const int *__restrict__ active, int *__restrict__ rot)
{
    typedef typename ctraits<T>::R R;
    __shared__ R red[4][WIDE_THREADS / 32];
    __shared__ R s_c;
    __shared__ T s_sp;
    __shared__ int s_do;
    const int f = blockIdx.y;
    if (!active[f]) return;
    const int N2 = N + (N & 1);
    int i, j;
    rr_pair(N2, round, blockIdx.x, i, j);
    if (j >= N) return;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    T *yi = Y + f * sY + (size_t)i * M, *yj = Y + f * sY + (size_t)j * M;
    R a = 0, b = 0;
    T g = ctraits<T>::make(0, 0);
    for (int r = tid; r < Mdot; r += WIDE_THREADS) {
        const T u = yi[r], v = yj[r];
        a += zabs2(u);
        b += zabs2(v);
        zcfma(g, u, v);
    }
    a = warp_sum(a);
    b = warp_sum(b);
    g.x = warp_sum(g.x);
    g.y = warp_sum(g.y);
    if (lane == 0) {
        red[0][wid] = a;
        red[1][wid] = b;
        red[2][wid] = g.x;
        red[3][wid] = g.y;
    }
    __syncthreads();
    if (tid == 0) {
        a = red[0][0];
        b = red[1][0];
        g = ctraits<T>::make(red[2][0], red[3][0]);
        for (int w = 1; w < WIDE_THREADS / 32; ++w) {
            a += red[0][w];
            b += red[1][w];
            g.x += red[2][w];
            g.y += red[3][w];
        }
        R c;
        T sp;
        s_do = jacobi_rotation(a, b, g, tol, c, sp) ? 1 : 0;
        s_c = c;
        s_sp = sp;
        if (s_do) atomicAdd(&rot[f], 1);
    }
    __syncthreads();
    if (!s_do) return;
    const R c = s_c;
    const T sp = s_sp;
    for (int r = tid; r < M; r += WIDE_THREADS) {
        T u = yi[r], v = yj[r];
        rotate_pair(u, v, c, sp);
        yi[r] = u;
        yj[r] = v;
    }
    if (V) {
        T *vi = V + f * sV + (size_t)i * N, *vj = V + f * sV + (size_t)j * N;
        for (int r = tid; r < N; r += WIDE_THREADS) {
            T u = vi[r], v = vj[r];
            rotate_pair(u, v, c, sp);
            vi[r] = u;
            vj[r] = v;
        }
    }
}

// counters: active[batch], rot[batch], total.  reset: every bin active.
__global__ void jacobi_wide_reset_kernel(int batch, int *cnt)
{
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < batch; f += gridDim.x * blockDim.x) {
        cnt[f] = 1;
        cnt[batch + f] = 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt[2 * batch] = 0;
}

// end of a sweep: a bin stays active while it rotated; total = active bins
__global__ void jacobi_wide_sweep_kernel(int batch, int *cnt)
{
    __shared__ int s_tot;
    if (threadIdx.x == 0) s_tot = 0;
    __syncthreads();
    int n = 0;
    for (int f = threadIdx.x; f < batch; f += blockDim.x) {
        const int act = cnt[f] && cnt[batch + f] > 0;
        cnt[f] = act;
        cnt[batch + f] = 0;
        n += act;
    }
    atomicAdd(&s_tot, n);
    __syncthreads();
    if (threadIdx.x == 0) cnt[2 * batch] = s_tot;
}

__global__ void jacobi_wide_flag_kernel(int batch, const int *cnt, int *info)
{
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < batch; f += gridDim.x * blockDim.x)
        if (cnt[f] && info) atomicOr(&info[f], IA_INFO_NOCONV);
}

template <class T>
static int jacobi_wide(ia_context *ctx, int M, int Mdot, int N, T *Y, long long sY, T *V, long long sV, int batch,
                       int max_sweeps, typename ctraits<T>::R tol, int *info)
{
    const size_t need = 2 * (size_t)batch + 1;
    if (ctx->dcount_n < need) {
        if (ctx->dcount) IA_CUDA_TRY(cudaFree(ctx->dcount));
        ctx->dcount = nullptr;
        ctx->dcount_n = 0;
        IA_CUDA_TRY(cudaMalloc((void **)&ctx->dcount, sizeof(int) * need));
        ctx->dcount_n = need;
    }
    int *cnt = ctx->dcount;
    jacobi_wide_reset_kernel<<<(batch + 255) / 256, 256, 0, ctx->stream>>>(batch, cnt);
    IA_LAUNCH_CHECK(ctx);
    const int N2 = N + (N & 1), pairs = N2 / 2;
    int total = batch;
    int sweep = 0;
    for (; sweep < max_sweeps && total > 0; ++sweep) {
        for (int round = 0; round < N2 - 1; ++round) {
            jacobi_round_kernel<T><<<dim3(pairs, batch), WIDE_THREADS, 0, ctx->stream>>>(M, Mdot, N, Y, sY, V, sV,
                                                                                         round, tol, cnt, cnt + batch);
            IA_LAUNCH_CHECK(ctx);
        }
        jacobi_wide_sweep_kernel<<<1, 256, 0, ctx->stream>>>(batch, cnt);
        IA_LAUNCH_CHECK(ctx);
        IA_CUDA_TRY(cudaMemcpyAsync(&total, cnt + 2 * batch, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        IA_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    }
    if (total > 0) {
        jacobi_wide_flag_kernel<<<(batch + 255) / 256, 256, 0, ctx->stream>>>(batch, cnt, info);
        IA_LAUNCH_CHECK(ctx);
    }
    return IA_OK;
}

template <class T>
int jacobi_rows_batched(ia_context *ctx, int M, int Mdot, int N, T *Y, T *V, int batch, int max_sweeps, int *info)
{
    typedef typename ctraits<T>::R R;
    if (V) {
        dim3 g((N * N + 255) / 256 < 256 ? (N * N + 255) / 256 : 256, batch);
        identity_kernel<T><<<g, 256, 0, ctx->stream>>>(N, V, (long long)N * N);
        IA_LAUNCH_CHECK(ctx);
    }
    int nw = (N + 1) / 2;
    if (nw > SVD_MAX_WARPS) nw = SVD_MAX_WARPS;
    if (nw < 1) nw = 1;
    // FP64: rotate while |y_i^H y_j| > sqrt(Mdot) eps |y_i||y_j|.  FP32 (the
    // mixed path, always followed by FP64 eigen-refinement): 8x that, above
    // the rounding noise of FP32 dot products.  A looser start (64x) cut the
    // FP32 sweeps but left more coupled pairs for the FP64 Jacobi on X^H E X
    // and made the whole solve slower.
    const double eps = sizeof(R) == 8 ? 2.220446049250313e-16 : 8.0 * 1.1920928955078125e-07;
    const R tol = (R)(sqrt((double)Mdot) * eps);
    const long long sY = (long long)M * N, sV = (long long)N * N;
    const size_t smem = sizeof(T) * (size_t)M * N;
    // without accumulator: a half-warp per pair (FP32: every pair of a round at
    // once in 32 warps; FP64: 16 warps, the 128-register budget), Y in shared
    // memory up to the per-CTA limit (an FP64 121 x 120 system fits)
    const size_t half_smem_max = sizeof(T) <= 8 ? 200 * 1024 : 227 * 1024 - 64;   // 16 B static besides
    {
        // over a cluster per bin: FP32 for batches that leave most of the GPU
        // idle and for the last part of a staggered pipeline (4x the SMs for
        // ~0.7x the time per bin); FP64 whenever 2 or 4 CTAs per bin fit on
        // the SMs (the FP64 pipe of more SMs per bin).  Systems of 129-272 rows
        // (12 or 17 rows per lane) take 8-CTA clusters in as many waves as
        // needed: their alternative is a one-CTA kernel on global memory.
        const int np = (N + (N & 1)) / 2;
        int cs = 0, kpl = 8;
        if (!V && M <= 128 && N <= 128) {
            if (sizeof(T) == 8) {
                if (np % 4 == 0 && np / 4 >= 2 && (16 * batch <= ctx->sm_count || ctx->tail_part)) cs = 4;
            } else {
                for (int c : {4, 2})
                    if (!cs && np % c == 0 && np / c >= 2 && c * batch <= ctx->sm_count) cs = c;
            }
        } else if (!V && M <= 272 && N <= 272 && M > 128 && np % 8 == 0 && np / 8 >= 2) {
            cs = 8;
            kpl = M <= 192 ? 12 : 17;
        }
        if (cs) {
            const int P = np / cs;
            const size_t csm = sizeof(T) * ((size_t)2 * (P + 1) * M + M);
            const int nwc = (P + 1) / 2;
            cudaLaunchConfig_t lc = {};
            lc.gridDim = dim3((unsigned)(cs * batch));
            lc.blockDim = dim3((unsigned)(32 * nwc));
            lc.dynamicSmemBytes = csm;
            lc.stream = ctx->stream;
            cudaLaunchAttribute at[1];
            at[0].id = cudaLaunchAttributeClusterDimension;
            at[0].val.clusterDim.x = cs;
            at[0].val.clusterDim.y = 1;
            at[0].val.clusterDim.z = 1;
            lc.attrs = at;
            lc.numAttrs = 1;
            auto kern = kpl == 17   ? jacobi_cluster_kernel<T, 8, 17>
                        : kpl == 12 ? jacobi_cluster_kernel<T, 8, 12>
                        : (cs == 4 ? jacobi_cluster_kernel<T, 4> : jacobi_cluster_kernel<T, 2>);
            if (csm > 48 * 1024)
                IA_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)csm));
            IA_CUDA_TRY(cudaLaunchKernelEx(&lc, kern, M, Mdot, N, Y, sY, max_sweeps, tol, info));
            IA_LAUNCH_CHECK(ctx);
            return IA_OK;
        }
    }
    if (!V && M <= 128 && N <= 128 && smem <= half_smem_max) {
        const int pairs = (N + (N & 1)) / 2;
        const int wcap = sizeof(T) <= 8 ? 32 : 16;
        int nws = (pairs + 1) / 2;
        if (nws > wcap) nws = wcap;
        if (nws < 1) nws = 1;
        IA_CUDA_TRY(cudaFuncSetAttribute(jacobi_half_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)half_smem_max));
        jacobi_half_kernel<T><<<batch, nws * 32, smem, ctx->stream>>>(M, Mdot, N, Y, sY, max_sweeps, tol, info);
    } else if (M <= 128 && N <= 128 && smem <= 200 * 1024) {
        const int wmax = sizeof(T) <= 8 ? 2 * SVD_MAX_WARPS : SVD_MAX_WARPS;
        int nws = (N + 1) / 2 < wmax ? (N + 1) / 2 : wmax;
        if (nws < 1) nws = 1;
        IA_CUDA_TRY(cudaFuncSetAttribute(jacobi_smem_kernel<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024));
        jacobi_smem_kernel<T, 4><<<batch, nws * 32, smem, ctx->stream>>>(M, Mdot, N, Y, sY, V, sV, max_sweeps, tol,
                                                                         info);
    } else if (M <= 128)
        jacobi_kernel<T, 4><<<batch, nw * 32, 0, ctx->stream>>>(M, Mdot, N, Y, sY, V, sV, max_sweeps, tol, info);
    else if (M <= 256)
        jacobi_kernel<T, 8><<<batch, nw * 32, 0, ctx->stream>>>(M, Mdot, N, Y, sY, V, sV, max_sweeps, tol, info);
    else {
        // large systems, few of them (one CTA per bin would leave most SMs
        // idle): over the whole GPU, round by round, where the host may
        // synchronise (not under stream capture).  With a bin per SM or more
        // the one-CTA kernel is faster (the 512-bin order-15 HELS solve: 3.1 s
        // against 4.6 s round by round).
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        IA_CUDA_TRY(cudaStreamIsCapturing(ctx->stream, &cs));
        if (cs == cudaStreamCaptureStatusNone && !ctx->capturing && 2 * batch <= ctx->sm_count)
            return jacobi_wide<T>(ctx, M, Mdot, N, Y, sY, V, sV, batch, max_sweeps, tol, info);
        jacobi_kernel<T, 0><<<batch, nw * 32, 0, ctx->stream>>>(M, Mdot, N, Y, sY, V, sV, max_sweeps, tol, info);
    }
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}
template int jacobi_rows_batched<double2>(ia_context *, int, int, int, double2 *, double2 *, int, int, int *);
template int jacobi_rows_batched<float2>(ia_context *, int, int, int, float2 *, float2 *, int, int, int *);

int jacobi_svd_batched(ia_context *ctx, int M, int N, double2 *Y, double2 *V, int batch, int max_sweeps, int *info)
{
    return jacobi_rows_batched<double2>(ctx, M, M, N, Y, V, batch, max_sweeps, info);
}

// sigma_j = ||y_j||, descending order (ties by index), U = Y/sigma, V permuted.
__global__ void svd_finalize_kernel(int M, int N, const double2 *Y, const double2 *V, double *s, double2 *Uy,
                                    double2 *Vs, int *info)
{
    extern __shared__ double sm[];
    double *sig = sm;                              // N
    int *rank = reinterpret_cast<int *>(sm + N);   // N
    const int f = blockIdx.x;
    Y += (size_t)f * M * N;
    if (V) V += (size_t)f * N * N;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = wid; j < N; j += nw) {
        double a = 0.0;
        for (int r = lane; r < M; r += 32) {
            double2 u = Y[r + (size_t)j * M];
            a = fma(u.x, u.x, fma(u.y, u.y, a));
        }
        a = warp_sum(a);
        if (lane == 0) sig[j] = sqrt(a);
    }
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        double sj = sig[j];
        int rk = 0;
        for (int i = 0; i < N; ++i) {
            double si = sig[i];
            if (si > sj || (si == sj && i < j)) rk++;
        }
        rank[j] = rk;
        if (s) s[(size_t)f * N + rk] = sj;
        if (info && (!(sj == sj) || isinf(sj))) atomicOr(&info[f], IA_INFO_NONFINITE);
    }
    __syncthreads();
    if (Uy) {
        for (int j = wid; j < N; j += nw) {
            double inv = sig[j] > 0.0 ? 1.0 / sig[j] : 0.0;
            double2 *dst = Uy + (size_t)f * M * N + (size_t)rank[j] * M;
            for (int r = lane; r < M; r += 32) dst[r] = zscale(Y[r + (size_t)j * M], inv);
        }
    }
    if (Vs && V) {
        for (int j = wid; j < N; j += nw) {
            double2 *dst = Vs + (size_t)f * N * N + (size_t)rank[j] * N;
            for (int r = lane; r < N; r += 32) dst[r] = V[r + (size_t)j * N];
        }
    }
}

int svd_finalize_batched(ia_context *ctx, int M, int N, const double2 *Y, const double2 *V, double *s, double2 *Uy,
                         double2 *Vs, int batch, int *info)
{
    size_t smem = (size_t)N * (sizeof(double) + sizeof(int));
    svd_finalize_kernel<<<batch, 256, smem, ctx->stream>>>(M, N, Y, V, s, Uy, Vs, info);
    IA_LAUNCH_CHECK(ctx);
    return IA_OK;
}

size_t svd_workspace_bytes(int m, int n, int batch)
{
    int M = m >= n ? m : n, N = m >= n ? n : m;
    return ws_round(sizeof(double2) * (size_t)M * N * batch) + ws_round(sizeof(double2) * (size_t)N * N * batch) +
           512;
}

int svd_batched(ia_context *ctx, int m, int n, const double2 *A, bool transposed_input, double2 *U, double *s,
                double2 *V, int batch, int max_sweeps, int *info, double2 *Y, double2 *Vacc)
{
    const bool tall = m >= n;
    const int M = tall ? m : n, N = tall ? n : m;
    int st = IA_OK;
    const long long sA = (long long)m * n;
    if (tall) {
        // Y = A (m x n)
        if (!transposed_input) st = zcopy2d_batched(ctx, m, n, A, m, sA, Y, M, (long long)M * N, false, batch);
        else st = ztranspose_batched(ctx, n, m, A, n, sA, Y, M, (long long)M * N, false, batch);
    } else {
        // Y = A^H (n x m)
        if (!transposed_input) st = ztranspose_batched(ctx, m, n, A, m, sA, Y, M, (long long)M * N, true, batch);
        else st = zcopy2d_batched(ctx, n, m, A, n, sA, Y, M, (long long)M * N, true, batch);
    }
    if (st) return st;
    st = jacobi_svd_batched(ctx, M, N, Y, Vacc, batch, max_sweeps, info);
    if (st) return st;
    // tall:  A = Uy S Vacc^H        -> U = Uy,   V = Vacc
    // wide:  A^H = Uy S Vacc^H      -> U = Vacc, V = Uy
    if (tall) return svd_finalize_batched(ctx, M, N, Y, Vacc, s, U, V, batch, info);
    return svd_finalize_batched(ctx, M, N, Y, Vacc, s, V, U, batch, info);
}

IA_BOUNDS_READER(bounds_read_svd)

}  // namespace ia
