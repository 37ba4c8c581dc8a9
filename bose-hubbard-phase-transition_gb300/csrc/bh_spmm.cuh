// bh_spmm.cuh -- the sparse products Y = H X of the solver (CSR and
// matrix-free), included by one translation unit per element type.
#pragma once

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <type_traits>

#include "bh_krylov.cuh"

namespace bh {

// Explicitly rounded products and fused multiply-adds for the products below:
// the compiler neither contracts nor splits them, so every launch shape (a
// different instantiation of the same loops) rounds every entry of Y the
// same way.  Accumulation: acc = fma(v, x, acc) per entry in storage order;
// epilogue: y = fma(J, acc, fma(U, d, shift) * x).
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

// Y = H X for ncols columns; column t belongs to solve t / group with
// prm[3 s + 0..2] = (J, U, shift).  L lanes per row, lanes over columns.
// DP > 0 (= group, one pass over the row's columns): the product also yields
// the partial sums of X_s^T Y_s (the block-Lanczos coefficient A = V_j^T H V_j
// of every solve): lane t holds Y[r][t] and receives X[r][s DP + q] from the
// neighbouring lanes by shuffles; FP32 sums over 16 rows, then FP64 slots in
// shared memory, reduced per CTA into dpart[(cta DP + q) ncols + t].
template <class T, int L, int CW, int DP>
__global__ void __launch_bounds__(256)
k_spmm(OpView<T> A, int ncols, int group, const double* __restrict__ prm,
       const T* __restrict__ X, T* __restrict__ Y, double* __restrict__ dpart) {
    extern __shared__ double s_dot[];
    const int gl = threadIdx.x % L;
    const int lane = threadIdx.x & 31;
    const unsigned seg = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << (lane & ~(L - 1)));
    const int rows_per_block = blockDim.x / L;
    const int cpl = ncols / L;
    constexpr int NDP = DP > 0 ? DP : 1;
    T dacc[CW][NDP];
    int drows = 0;
    if constexpr (DP > 0) {
#pragma unroll
        for (int u = 0; u < CW; ++u)
#pragma unroll
            for (int q = 0; q < NDP; ++q) {
                dacc[u][q] = T(0);
                s_dot[(size_t)(u * NDP + q) * blockDim.x + threadIdx.x] = 0.0;
            }
    }
    for (int64_t r = (int64_t)blockIdx.x * rows_per_block + threadIdx.x / L; r < A.D;
         r += (int64_t)gridDim.x * rows_per_block) {
        const int64_t e0 = A.rp[r], e1 = A.rp[r + 1];
        const T d = A.vd ? A.vd[r] : T(0);
        for (int c0 = 0; c0 < cpl; c0 += CW) {
            T acc[CW];
#pragma unroll
            for (int u = 0; u < CW; ++u) acc[u] = T(0);
            const int nc = min(CW, cpl - c0);
            // four entries per step: their X rows are all requested before the
            // first product (the summation order per column is unchanged)
            int64_t e = e0;
            for (; e + 4 <= e1; e += 4) {
                int64_t cc[4];
                T vv[4], xv[4][CW];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    cc[k] = A.ci[e + k];
                    vv[k] = A.tv[e + k];
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const T* xr = X + cc[k] * ncols + gl + c0 * L;
#pragma unroll
                    for (int u = 0; u < CW; ++u)
                        if (u < nc) xv[k][u] = xr[u * L];
                }
#pragma unroll
                for (int k = 0; k < 4; ++k)
#pragma unroll
                    for (int u = 0; u < CW; ++u)
                        if (u < nc) acc[u] = fma_rn(vv[k], xv[k][u], acc[u]);
            }
            for (; e < e1; ++e) {
                const int64_t col = A.ci[e];
                const T v = A.tv[e];
                const T* xr = X + col * ncols + gl + c0 * L;
#pragma unroll
                for (int u = 0; u < CW; ++u)
                    if (u < nc) acc[u] = fma_rn(v, xr[u * L], acc[u]);
            }
            T xself[CW], yv[CW];
#pragma unroll
            for (int u = 0; u < CW; ++u) {
                xself[u] = T(0);
                yv[u] = T(0);
                if (u < nc) {
                    const int t = gl + (c0 + u) * L;
                    const int s = t / group;
                    const T Jc = (T)prm[3 * s], Uc = (T)prm[3 * s + 1], sh = (T)prm[3 * s + 2];
                    xself[u] = X[r * ncols + t];
                    yv[u] = fma_rn(Jc, acc[u], mul_rn(fma_rn(Uc, d, sh), xself[u]));
                    Y[r * ncols + t] = yv[u];
                }
            }
            if constexpr (DP > 0) {
                const int qo = gl % DP;  // this lane's column within its solve
#pragma unroll
                for (int u = 0; u < CW; ++u)
#pragma unroll
                    for (int q = 0; q < DP; ++q) {
                        const T xq = __shfl_sync(seg, xself[u], gl - qo + q, L);
                        dacc[u][q] += xq * yv[u];
                    }
            }
        }
        if constexpr (DP > 0) {
            if (++drows == 16) {
                drows = 0;
#pragma unroll
                for (int u = 0; u < CW; ++u)
#pragma unroll
                    for (int q = 0; q < NDP; ++q) {
                        s_dot[(size_t)(u * NDP + q) * blockDim.x + threadIdx.x] += (double)dacc[u][q];
                        dacc[u][q] = T(0);
                    }
            }
        }
    }
    if constexpr (DP > 0) {
#pragma unroll
        for (int u = 0; u < CW; ++u)
#pragma unroll
            for (int q = 0; q < NDP; ++q)
                s_dot[(size_t)(u * NDP + q) * blockDim.x + threadIdx.x] += (double)dacc[u][q];
        __syncthreads();
        // one thread per (column t, q): sum over the CTA's row slots in order
        for (int e = threadIdx.x; e < ncols * DP; e += blockDim.x) {
            const int t = e / DP, q = e % DP;
            const int u = t / L, g = t % L;
            double sum = 0.0;
            for (int ro = 0; ro < rows_per_block; ++ro)
                sum += s_dot[(size_t)(u * NDP + q) * blockDim.x + ro * L + g];
            dpart[((size_t)blockIdx.x * DP + q) * ncols + t] = sum;
        }
    }
}

// Contiguous VW-column vectors of a row (16-byte aligned when the row's
// offset is a multiple of VW columns and VW * sizeof(T) >= 16, else 8-byte).
template <class T, int VW>
struct SpVec {
    T v[VW];
};
template <class T, int VW>
__device__ __forceinline__ SpVec<T, VW> sp_ldv(const T* __restrict__ p) {
    SpVec<T, VW> o;
    if constexpr (std::is_same<T, float>::value && VW == 4) {
        const float4 x = *reinterpret_cast<const float4*>(p);
        o.v[0] = x.x, o.v[1] = x.y, o.v[2] = x.z, o.v[3] = x.w;
    } else if constexpr (std::is_same<T, float>::value && VW == 2) {
        const float2 x = *reinterpret_cast<const float2*>(p);
        o.v[0] = x.x, o.v[1] = x.y;
    } else {
#pragma unroll
        for (int q = 0; q < VW; q += 2) {
            const double2 x = *reinterpret_cast<const double2*>(p + q);
            o.v[q] = x.x, o.v[q + 1] = x.y;
        }
    }
    return o;
}
template <class T, int VW>
__device__ __forceinline__ void sp_stv(T* __restrict__ p, const SpVec<T, VW>& o) {
    if constexpr (std::is_same<T, float>::value && VW == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(o.v[0], o.v[1], o.v[2], o.v[3]);
    } else if constexpr (std::is_same<T, float>::value && VW == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(o.v[0], o.v[1]);
    } else {
#pragma unroll
        for (int q = 0; q < VW; q += 2) *reinterpret_cast<double2*>(p + q) = make_double2(o.v[q], o.v[q + 1]);
    }
}

// CSR product with contiguous column vectors: VL lanes per row, lane l
// computes the VW adjacent columns t = VW (l + VL u) (u = pass; masked by
// t < ncols, ncols a multiple of VW), so every gathered X row is read with
// VW-wide vector loads and a warp's loads of one entry cover VL * VW
// contiguous values.  Each column's sum is the same chain of fma_rn over the
// row's entries in storage order as in k_spmm (four entries' rows requested
// before their products), and the epilogue is the same: Y equals k_spmm's
// bit for bit.  DP > 0 (block size, DP dividing VW, one pass over the row):
// the lane's VW columns hold whole solves, so the partials of X_s^T Y_s need
// no data from other lanes; FP32 sums over 16 rows, then FP64 slots in shared
// memory, reduced per CTA into dpart[(cta DP + q) ncols + t] like k_spmm.
template <class T, int VL, int VW, int DP>
__global__ void __launch_bounds__(256)
k_spmm_v(OpView<T> A, int ncols, int group, const double* __restrict__ prm,
         const T* __restrict__ X, T* __restrict__ Y, double* __restrict__ dpart) {
    extern __shared__ double s_dot[];
    const int gl = threadIdx.x % VL;
    const int rows_per_block = blockDim.x / VL;
    const int npass = (ncols + VL * VW - 1) / (VL * VW);
    constexpr int NDP = DP > 0 ? DP : 1;
    T dacc[VW][NDP];
    int drows = 0;
    if constexpr (DP > 0) {
#pragma unroll
        for (int v = 0; v < VW; ++v)
#pragma unroll
            for (int q = 0; q < NDP; ++q) {
                dacc[v][q] = T(0);
                s_dot[(size_t)(v * NDP + q) * blockDim.x + threadIdx.x] = 0.0;
            }
    }
    for (int64_t r = (int64_t)blockIdx.x * rows_per_block + threadIdx.x / VL; r < A.D;
         r += (int64_t)gridDim.x * rows_per_block) {
        const int64_t e0 = A.rp[r], e1 = A.rp[r + 1];
        const T d = A.vd ? A.vd[r] : T(0);
        for (int u = 0; u < npass; ++u) {
            const int t0 = (gl + VL * u) * VW;
            const bool on = t0 < ncols;
            T acc[VW];
#pragma unroll
            for (int v = 0; v < VW; ++v) acc[v] = T(0);
            int64_t e = e0;
            // UE entries per step: their X rows are all requested before the
            // first product (the summation order per column is unchanged)
            constexpr int UE = 4;  // 8 measured 6% slower at m=13 (48 registers, fewer warps)
            for (; e + UE <= e1; e += UE) {
                int cc[UE];
                T vv[UE];
                SpVec<T, VW> xv[UE];
#pragma unroll
                for (int k = 0; k < UE; ++k) {
                    cc[k] = A.ci[e + k];
                    vv[k] = A.tv[e + k];
                }
                if (on) {
#pragma unroll
                    for (int k = 0; k < UE; ++k) xv[k] = sp_ldv<T, VW>(X + (int64_t)cc[k] * ncols + t0);
#pragma unroll
                    for (int k = 0; k < UE; ++k)
#pragma unroll
                        for (int v = 0; v < VW; ++v) acc[v] = fma_rn(vv[k], xv[k].v[v], acc[v]);
                }
            }
            for (; e < e1; ++e) {
                const int64_t col = A.ci[e];
                const T w = A.tv[e];
                if (on) {
                    const SpVec<T, VW> x = sp_ldv<T, VW>(X + col * ncols + t0);
#pragma unroll
                    for (int v = 0; v < VW; ++v) acc[v] = fma_rn(w, x.v[v], acc[v]);
                }
            }
            if (!on) continue;
            const SpVec<T, VW> xs = sp_ldv<T, VW>(X + r * ncols + t0);
            SpVec<T, VW> yv;
#pragma unroll
            for (int v = 0; v < VW; ++v) {
                const int s = (t0 + v) / group;
                const T Jc = (T)prm[3 * s], Uc = (T)prm[3 * s + 1], sh = (T)prm[3 * s + 2];
                yv.v[v] = fma_rn(Jc, acc[v], mul_rn(fma_rn(Uc, d, sh), xs.v[v]));
            }
            sp_stv<T, VW>(Y + r * ncols + t0, yv);
            if constexpr (DP > 0) {
#pragma unroll
                for (int v = 0; v < VW; ++v)
#pragma unroll
                    for (int q = 0; q < DP; ++q) dacc[v][q] += xs.v[(v / DP) * DP + q] * yv.v[v];
            }
        }
        if constexpr (DP > 0) {
            if (++drows == 16) {
                drows = 0;
#pragma unroll
                for (int v = 0; v < VW; ++v)
#pragma unroll
                    for (int q = 0; q < NDP; ++q) {
                        s_dot[(size_t)(v * NDP + q) * blockDim.x + threadIdx.x] += (double)dacc[v][q];
                        dacc[v][q] = T(0);
                    }
            }
        }
    }
    if constexpr (DP > 0) {
#pragma unroll
        for (int v = 0; v < VW; ++v)
#pragma unroll
            for (int q = 0; q < NDP; ++q)
                s_dot[(size_t)(v * NDP + q) * blockDim.x + threadIdx.x] += (double)dacc[v][q];
        __syncthreads();
        for (int e = threadIdx.x; e < ncols * DP; e += blockDim.x) {
            const int t = e / DP, q = e % DP;
            const int g = t / VW, v = t % VW;
            double sum = 0.0;
            for (int ro = 0; ro < rows_per_block; ++ro)
                sum += s_dot[(size_t)(v * NDP + q) * blockDim.x + ro * VL + g];
            dpart[((size_t)blockIdx.x * DP + q) * ncols + t] = sum;
        }
    }
}

// Target index and amplitude of directed bond k of the state with index r,
// occupations w and packed suffix sums sufp; c = -1 if site i is empty.
template <class T>
__device__ __forceinline__ void mf_hop(int k, uint64_t w, uint64_t sufp, int64_t r, int bits,
                                       uint64_t mask, int n, const uint8_t* s_bd,
                                       const uint32_t* s_rt, const T* s_sq, int64_t& c, T& v) {
    const int i = s_bd[2 * k], j = s_bd[2 * k + 1];
    const int ni = (int)((w >> (bits * i)) & mask);
    c = -1;
    v = T(0);
    if (ni < 1) return;
    const int nj = (int)((w >> (bits * j)) & mask);
    int64_t rr = r;
    if (i < j) {
        for (int t = i; t < j; ++t) {
            const int st = (int)((sufp >> (bits * t)) & mask);
            rr += (int64_t)s_rt[t * (n + 1) + st + 1] - (int64_t)s_rt[t * (n + 1) + st];
        }
    } else {
        for (int t = j; t < i; ++t) {
            const int st = (int)((sufp >> (bits * t)) & mask);
            rr -= (int64_t)s_rt[t * (n + 1) + st] - (int64_t)s_rt[t * (n + 1) + st - 1];
        }
    }
    c = rr;
    v = s_sq[ni * (nj + 1)];
}

template <class T, int L, int CW>
__global__ void __launch_bounds__(256)
k_spmm_mf(OpView<T> A, int ncols, int group, const double* __restrict__ prm,
          const T* __restrict__ X, T* __restrict__ Y) {
    constexpr int SLOTS = L >= 4 ? 128 / L : 1;
    extern __shared__ __align__(16) unsigned char s_raw[];
    const int m = A.m, n = A.n, nb = A.nbonds, bits = A.bits;
    const int nrt = (m - 1) * (n + 1), nsq = n * (n + 1) + 1;
    T* s_sq = reinterpret_cast<T*>(s_raw);
    uint32_t* s_rt = reinterpret_cast<uint32_t*>(s_raw + (((size_t)nsq * sizeof(T) + 15) & ~(size_t)15));
    uint8_t* s_bd = reinterpret_cast<uint8_t*>(s_rt + nrt);
    // per-row hop lists (L >= 4): target index and amplitude of every bond
    const size_t hop_off = (((size_t)nsq * sizeof(T) + 15) & ~(size_t)15) + (size_t)nrt * 4 + 2 * (size_t)nb;
    int32_t* s_hc = reinterpret_cast<int32_t*>(s_raw + ((hop_off + 15) & ~(size_t)15));
    T* s_hv = reinterpret_cast<T*>(s_hc + (blockDim.x / L) * nb + ((blockDim.x / L) * nb & 1));
    for (int i = threadIdx.x; i < nsq; i += blockDim.x) s_sq[i] = A.sq[i];
    for (int i = threadIdx.x; i < nrt; i += blockDim.x) s_rt[i] = A.rt[i];
    for (int i = threadIdx.x; i < 2 * nb; i += blockDim.x) s_bd[i] = A.bonds[i];
    __syncthreads();
    const uint64_t mask = (1ull << bits) - 1ull;
    const int lane = threadIdx.x & 31;
    const int gl = threadIdx.x % L;
    const unsigned seg = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << (lane & ~(L - 1)));
    const int rows_per_block = blockDim.x / L;
    const int cpl = ncols / L;
    int32_t* hc = s_hc + (threadIdx.x / L) * nb;
    T* hv = s_hv + (threadIdx.x / L) * nb;
    for (int64_t r = (int64_t)blockIdx.x * rows_per_block + threadIdx.x / L; r < A.D;
         r += (int64_t)gridDim.x * rows_per_block) {
        const uint64_t w = A.occ[r];
        // suffix sums suf_t (t <= m - 2), packed like the occupations
        uint64_t sufp = 0;
        int suf = 0, v2 = 0;
        for (int t = m - 1; t >= 0; --t) {
            const int nt = (int)((w >> (bits * t)) & mask);
            v2 += nt * (nt - 1);
            if (t < m - 1) sufp |= (uint64_t)suf << (bits * t);
            suf += nt;
        }
        const T d = (T)(0.5 * (double)v2);
        if constexpr (L >= 4) {
            // the row's lanes split the bonds, then share them through shared memory
#pragma unroll
            for (int sl = 0; sl < SLOTS; ++sl) {
                const int k = sl * L + gl;
                if (k < nb) {
                    int64_t c;
                    T v;
                    mf_hop<T>(k, w, sufp, r, bits, mask, n, s_bd, s_rt, s_sq, c, v);
                    hc[k] = (int32_t)c;
                    hv[k] = v;
                }
            }
            __syncwarp(seg);
        }
        for (int c0 = 0; c0 < cpl; c0 += CW) {
            T acc[CW];
#pragma unroll
            for (int u = 0; u < CW; ++u) acc[u] = T(0);
            const int nc = min(CW, cpl - c0);
            if constexpr (L >= 4) {
                // bonds in order, four per step: the four X rows are requested
                // before the first product
                for (int k0 = 0; k0 < nb; k0 += 4) {
                    int32_t cc[4];
                    T vv[4], xv[4][CW];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        cc[k] = k0 + k < nb ? hc[k0 + k] : -1;
                        vv[k] = k0 + k < nb ? hv[k0 + k] : T(0);
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        if (cc[k] < 0) continue;
                        const T* xr = X + (int64_t)cc[k] * ncols + gl + c0 * L;
#pragma unroll
                        for (int u = 0; u < CW; ++u)
                            if (u < nc) xv[k][u] = xr[u * L];
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        if (cc[k] < 0) continue;
#pragma unroll
                        for (int u = 0; u < CW; ++u)
                            if (u < nc) acc[u] = fma_rn(vv[k], xv[k][u], acc[u]);
                    }
                }
            } else {
                // one or two lanes per row: each lane evaluates every bond
                for (int k = 0; k < nb; ++k) {
                    int64_t c;
                    T v;
                    mf_hop<T>(k, w, sufp, r, bits, mask, n, s_bd, s_rt, s_sq, c, v);
                    if (c < 0) continue;
                    const T* xr = X + c * ncols + gl + c0 * L;
#pragma unroll
                    for (int u = 0; u < CW; ++u)
                        if (u < nc) acc[u] = fma_rn(v, xr[u * L], acc[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < CW; ++u) {
                if (u < nc) {
                    const int t = gl + (c0 + u) * L;
                    const int s = t / group;
                    const T Jc = (T)prm[3 * s], Uc = (T)prm[3 * s + 1], sh = (T)prm[3 * s + 2];
                    const T xv = X[r * ncols + t];
                    Y[r * ncols + t] = fma_rn(Jc, acc[u], mul_rn(fma_rn(Uc, d, sh), xv));
                }
            }
        }
        if constexpr (L >= 4) __syncwarp(seg);  // the next row overwrites the hop list
    }
}

// Four consecutive hop values of a row's list (16-byte aligned).
__device__ __forceinline__ void load4(const float* p, float (&v)[4]) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x;
    v[1] = q.y;
    v[2] = q.z;
    v[3] = q.w;
}
__device__ __forceinline__ void load4(const double* p, double (&v)[4]) {
    const double2 a = *reinterpret_cast<const double2*>(p);
    const double2 b = *reinterpret_cast<const double2*>(p + 2);
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
}

// Matrix-free product with one warp per row (8 rows per CTA), for any ncols:
// lane l computes columns t = l + 32 u (u < CW per pass, t < ncols).  The
// row's integer work is spread over the lanes (m <= 32 sites): lane t
// extracts n_t, the suffix sums s_t = sum_{u > t} n_u and the interaction
// sum come from warp scans, and the rank of the state after a hop i -> j is
//   r + (P_a[j] - P_a[i])   (i < j),   r - (P_b[i] - P_b[j])   (i > j),
// with exclusive prefix sums over sites of the rank increments
//   a_t = RT[t][s_t + 1] - RT[t][s_t],   b_t = RT[t][s_t] - RT[t][s_t - 1]
// (one boson crossing the cut after site t raises or lowers s_t by one; sums
// modulo 2^32, the true difference is below D in magnitude), so a bond costs
// a few shuffles instead of |i - j| rank-table lookups.  The valid hops
// (n_i >= 1) are compacted in bond order into the warp's shared-memory list
// and summed in that order, as the other matrix-free paths do: Y is the same
// bit for bit.
template <class T, int CW>
__global__ void __launch_bounds__(256)
k_spmm_mf_warp(OpView<T> A, int ncols, int group, const double* __restrict__ prm,
               const T* __restrict__ X, T* __restrict__ Y) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    constexpr unsigned FULL = 0xffffffffu;
    const int m = A.m, n = A.n, nb = A.nbonds, bits = A.bits;
    const int nrt = (m - 1) * (n + 1), nsq = n * (n + 1) + 1;
    const int nbp = (nb + 3) & ~3;
    T* s_sq = reinterpret_cast<T*>(s_raw);
    uint32_t* s_rt = reinterpret_cast<uint32_t*>(s_raw + (((size_t)nsq * sizeof(T) + 15) & ~(size_t)15));
    uint8_t* s_bd = reinterpret_cast<uint8_t*>(s_rt + nrt);
    const size_t hop_off =
        ((((size_t)nsq * sizeof(T) + 15) & ~(size_t)15) + (size_t)nrt * 4 + 2 * (size_t)nb + 15) & ~(size_t)15;
    int32_t* s_hc = reinterpret_cast<int32_t*>(s_raw + hop_off);
    T* s_hv = reinterpret_cast<T*>(s_raw + hop_off + (size_t)8 * nbp * sizeof(int32_t));
    for (int i = threadIdx.x; i < nsq; i += blockDim.x) s_sq[i] = A.sq[i];
    for (int i = threadIdx.x; i < nrt; i += blockDim.x) s_rt[i] = A.rt[i];
    for (int i = threadIdx.x; i < 2 * nb; i += blockDim.x) s_bd[i] = A.bonds[i];
    __syncthreads();
    const uint64_t mask = (1ull << bits) - 1ull;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t* hc = s_hc + warp * nbp;
    T* hv = s_hv + warp * nbp;
    const int cpl = (ncols + 31) >> 5;
    // every lane of a warp walks the same rows: the shuffles below are uniform
    for (int64_t r = (int64_t)blockIdx.x * 8 + warp; r < A.D; r += (int64_t)gridDim.x * 8) {
        const uint64_t w = A.occ[r];
        const int nt = lane < m ? (int)((w >> (bits * lane)) & mask) : 0;
        int suf = nt;  // inclusive suffix sum over lanes >= this one
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_down_sync(FULL, suf, o);
            if (lane + o < 32) suf += v;
        }
        const int st = suf - nt;
        int v2 = nt * (nt - 1);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v2 += __shfl_xor_sync(FULL, v2, o);
        const T d = (T)(0.5 * (double)v2);
        uint32_t a = 0, b = 0;
        if (lane < m - 1) {
            const uint32_t* rt = s_rt + lane * (n + 1);
            if (st < n) a = rt[st + 1] - rt[st];
            if (st > 0) b = rt[st] - rt[st - 1];
        }
        uint32_t pa = a, pb = b;  // inclusive prefix sums, then exclusive
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t ua = __shfl_up_sync(FULL, pa, o), ub = __shfl_up_sync(FULL, pb, o);
            if (lane >= o) {
                pa += ua;
                pb += ub;
            }
        }
        pa -= a;
        pb -= b;
        // hop list of the row: bonds k = k0 + lane, valid ones compacted in order
        int cnt = 0;
        for (int k0 = 0; k0 < nb; k0 += 32) {
            const int k = k0 + lane;
            int i = 0, j = 0;
            if (k < nb) {
                i = s_bd[2 * k];
                j = s_bd[2 * k + 1];
            }
            const int ni = __shfl_sync(FULL, nt, i), nj = __shfl_sync(FULL, nt, j);
            const uint32_t pai = __shfl_sync(FULL, pa, i), paj = __shfl_sync(FULL, pa, j);
            const uint32_t pbi = __shfl_sync(FULL, pb, i), pbj = __shfl_sync(FULL, pb, j);
            const bool ok = k < nb && ni >= 1;
            const unsigned bal = __ballot_sync(FULL, ok);
            if (ok) {
                const int32_t dr = i < j ? (int32_t)(paj - pai) : -(int32_t)(pbi - pbj);
                const int pos = cnt + __popc(bal & ((1u << lane) - 1u));
                hc[pos] = (int32_t)r + dr;
                hv[pos] = s_sq[ni * (nj + 1)];
            }
            cnt += __popc(bal);
        }
        __syncwarp();
        for (int c0 = 0; c0 < cpl; c0 += CW) {
            T acc[CW];
            bool on[CW];
#pragma unroll
            for (int u = 0; u < CW; ++u) {
                acc[u] = T(0);
                on[u] = c0 + u < cpl && lane + 32 * (c0 + u) < ncols;
            }
            // bonds in order, four per step: the four X rows are requested
            // before the first product
            for (int e = 0; e < cnt; e += 4) {
                const int4 c4 = *reinterpret_cast<const int4*>(hc + e);
                const int cc[4] = {c4.x, c4.y, c4.z, c4.w};
                T vv[4], xv[4][CW];
                load4(hv + e, vv);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (e + k >= cnt) continue;
                    const T* xr = X + (int64_t)cc[k] * ncols + lane + 32 * c0;
#pragma unroll
                    for (int u = 0; u < CW; ++u)
                        if (on[u]) xv[k][u] = xr[32 * u];
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (e + k >= cnt) continue;
#pragma unroll
                    for (int u = 0; u < CW; ++u)
                        if (on[u]) acc[u] = fma_rn(vv[k], xv[k][u], acc[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < CW; ++u) {
                if (on[u]) {
                    const int t = lane + 32 * (c0 + u);
                    const int s = t / group;
                    const T Jc = (T)prm[3 * s], Uc = (T)prm[3 * s + 1], sh = (T)prm[3 * s + 2];
                    const T xv = X[r * ncols + t];
                    Y[r * ncols + t] = fma_rn(Jc, acc[u], mul_rn(fma_rn(Uc, d, sh), xv));
                }
            }
        }
        __syncwarp();  // the next row overwrites the hop list
    }
}

// Resident CTAs per SM of the fused CSR product (found once per instance).
template <class T, int L, int CW, int DP>
int spmm_fused_per_sm() {
    static std::atomic<int> occ{0};
    int n = occ.load(std::memory_order_relaxed);
    if (n == 0) {
        n = std::max(1, resident_ctas(k_spmm<T, L, CW, DP>, 256, (size_t)256 * CW * DP * sizeof(double)));
        occ.store(n, std::memory_order_relaxed);
    }
    return n;
}

// Resident CTAs per SM of the fused contiguous-column product (found once per instance).
template <class T, int VL, int VW, int DP>
int spmm_fused_v_per_sm() {
    static std::atomic<int> occ{0};
    int n = occ.load(std::memory_order_relaxed);
    if (n == 0) {
        n = std::max(1, resident_ctas(k_spmm_v<T, VL, VW, DP>, 256, (size_t)256 * VW * DP * sizeof(double)));
        occ.store(n, std::memory_order_relaxed);
    }
    return n;
}

// Dynamic shared memory of the matrix-free product at L lanes per row: the
// -sqrt table, the rank table and the bonds, plus (L >= 4) the hop lists of
// the CTA's rows ((256 / L) rows x nbonds x (int32 + T), 16-byte aligned parts).
template <class T>
size_t spmm_mf_smem(const OpView<T>& op, int L) {
    const int nsq = op.n * (op.n + 1) + 1;
    size_t smem = (((size_t)nsq * sizeof(T) + 15) & ~(size_t)15) +
                  (size_t)(op.m - 1) * (op.n + 1) * sizeof(uint32_t) + 2 * (size_t)op.nbonds;
    if (L >= 4) {
        const size_t nh = (size_t)(256 / L) * op.nbonds;
        smem = ((smem + 15) & ~(size_t)15) + (nh + (nh & 1)) * 4 + nh * sizeof(T);
    }
    return smem;
}

// Dynamic shared memory of the warp-per-row matrix-free product: the same
// tables, then the hop lists of its 8 rows, padded to 4 entries (int32 row
// indices, then the values).
template <class T>
size_t spmm_mf_warp_smem(const OpView<T>& op) {
    const int nsq = op.n * (op.n + 1) + 1;
    const size_t nbp = ((size_t)op.nbonds + 3) & ~(size_t)3;
    size_t smem = (((size_t)nsq * sizeof(T) + 15) & ~(size_t)15) +
                  (size_t)(op.m - 1) * (op.n + 1) * sizeof(uint32_t) + 2 * (size_t)op.nbonds;
    smem = (smem + 15) & ~(size_t)15;
    return smem + 8 * nbp * (sizeof(int32_t) + sizeof(T));
}

// Algorithmic bytes of one product: the operator's stream (CSR pattern,
// values and diagonal, or the packed occupations) plus X read and Y written once.
template <class T, bool MF>
double spmm_bytes(const OpView<T>& op, int ncols) {
    const double D = (double)op.D;
    if (MF) return D * 8.0 + 2.0 * D * ncols * sizeof(T);
    const double nnz = (double)op.rp_nnz;
    return nnz * (4.0 + sizeof(T)) + (D + 1.0) * 8.0 + (op.vd ? D * sizeof(T) : 0.0) +
           2.0 * D * ncols * sizeof(T);
}

// Calls f(L, CW) as compile-time constants for the instantiated shapes:
// CW in {1, 4} for L < 32 (1 when cw == 1, else 4), {1, 2, 4} for L = 32.
template <class F>
void by_shape(int L, int cw, F&& f) {
    auto narrow_or_wide = [&](auto lc) {
        if (cw == 1) f(lc, std::integral_constant<int, 1>());
        else f(lc, std::integral_constant<int, 4>());
    };
    switch (L) {
        case 1: narrow_or_wide(std::integral_constant<int, 1>()); break;
        case 2: narrow_or_wide(std::integral_constant<int, 2>()); break;
        case 4: narrow_or_wide(std::integral_constant<int, 4>()); break;
        case 8: narrow_or_wide(std::integral_constant<int, 8>()); break;
        case 16: narrow_or_wide(std::integral_constant<int, 16>()); break;
        default:
            if (cw == 1) f(std::integral_constant<int, 32>(), std::integral_constant<int, 1>());
            else if (cw == 2) f(std::integral_constant<int, 32>(), std::integral_constant<int, 2>());
            else f(std::integral_constant<int, 32>(), std::integral_constant<int, 4>());
            break;
    }
}

// Calls f(VL, VW) as compile-time constants: VL in {2, 4, 8, 16, 32}, VW in {2, 4}.
template <class F>
void by_vshape(int VL, int VW, F&& f) {
    auto w = [&](auto lc) {
        if (VW == 2) f(lc, std::integral_constant<int, 2>());
        else f(lc, std::integral_constant<int, 4>());
    };
    switch (VL) {
        case 2: w(std::integral_constant<int, 2>()); break;
        case 4: w(std::integral_constant<int, 4>()); break;
        case 8: w(std::integral_constant<int, 8>()); break;
        case 16: w(std::integral_constant<int, 16>()); break;
        default: w(std::integral_constant<int, 32>()); break;
    }
}

// The product without the fused partials, with shape s (L, CW from the
// instantiated set: CW in {1, 4} for L < 32, {1, 2, 4} for L = 32; or the
// contiguous-column product when s.VW > 0).
template <class T, bool MF>
void spmm_launch_plain(const OpView<T>& op, int ncols, int group, const double* prm, const T* X, T* Y,
                       cudaStream_t st, const SpmmShape& s) {
    if constexpr (!MF) {
        if (s.VW > 0) {
            const int64_t rows = (op.D + (256 / s.L) - 1) / (256 / s.L);
            auto go = [&](auto lc, auto wc) {
                constexpr int VL = decltype(lc)::value, VW = decltype(wc)::value;
                auto kern = k_spmm_v<T, VL, VW, 0>;
                int64_t g = s.grid;
                if (g == 0) g = std::min<int64_t>(rows, (int64_t)sm_count() * 16);
                else if (g < 0) g = std::min<int64_t>(rows, (int64_t)sm_count() * std::max(1, resident_ctas(kern, 256, 0)));
                g = std::max<int64_t>(1, std::min<int64_t>(g, 0x7fffffff));
                kern<<<(unsigned)g, 256, 0, st>>>(op, ncols, group, prm, X, Y, nullptr);
            };
            by_vshape(s.L, s.VW, go);
            return;
        }
    }
    const int64_t rows = (op.D + (256 / s.L) - 1) / (256 / s.L);
    size_t smem = 0;
    if (MF) {
        BH_REQUIRE(op.nbonds <= 128, "matrix-free product: at most 128 directed bonds");
        BH_REQUIRE(op.m <= 32, "matrix-free product: at most 32 sites");
        smem = s.L == 32 ? spmm_mf_warp_smem(op) : spmm_mf_smem(op, s.L);
    }
    auto go = [&](auto lc, auto cwc) {
        constexpr int LL = decltype(lc)::value, CC = decltype(cwc)::value;
        auto launch = [&](auto kern) {
            allow_large_smem(kern, smem);
            int64_t g = s.grid;
            if (g == 0) g = std::min<int64_t>(rows, (int64_t)sm_count() * 16);
            else if (g < 0) g = std::min<int64_t>(rows, (int64_t)sm_count() * std::max(1, resident_ctas(kern, 256, smem)));
            g = std::max<int64_t>(1, std::min<int64_t>(g, 0x7fffffff));
            if constexpr (MF) kern<<<(unsigned)g, 256, smem, st>>>(op, ncols, group, prm, X, Y);
            else kern<<<(unsigned)g, 256, 0, st>>>(op, ncols, group, prm, X, Y, nullptr);
        };
        if constexpr (MF && LL == 32) launch(k_spmm_mf_warp<T, CC>);
        else if constexpr (MF) launch(k_spmm_mf<T, LL, CC>);
        else launch(k_spmm<T, LL, CC, 0>);
    };
    by_shape(s.L, s.CW, go);
}

// Launch of Y = H X on a CSR (MF = false) or matrix-free (MF = true)
// operator.  Default shape: L lanes per row over the columns (the largest
// power of two <= 32 dividing ncols), CW columns per lane per pass (1 or 2
// when that covers the row's share, else 4 with further passes); a product
// that does not fuse the local coefficient takes the tuning table's shape
// instead when `tuned` and the table has one.  Returns the algorithmic bytes.
template <class T, bool MF>
double launch_spmm_kind(const OpView<T>& op, int ncols, int group, const double* prm, const T* X,
                        T* Y, cudaStream_t st, double* dpart, int* dparts, bool tuned) {
    const int64_t D = op.D;
    const SpmmShape def = spmm_resolve(SpmmChoice{}, ncols, MF);
    const int L = def.L, CW = def.CW;
    if (dparts) *dparts = 0;
    if (!MF && dpart != nullptr && (group == 2 || group == 4) && spmm_fuses_vec(ncols, group)) {
        // fused X^T Y partials on the contiguous-column product (every lane
        // holds whole solves), one resident wave
        const SpmmShape v = spmm_resolve(SpmmChoice{0, 0, 0, 1}, ncols, false);
        const int rpb = 256 / v.L;
        const int64_t g = std::max<int64_t>(1, std::min<int64_t>((D + rpb - 1) / rpb, (int64_t)sm_count() * 16));
        auto go = [&](auto lc, auto wc) {
            constexpr int VL = decltype(lc)::value, VW = decltype(wc)::value;
            auto fused = [&](auto dpc) {
                constexpr int DPP = decltype(dpc)::value;
                if constexpr (VW % DPP == 0) {
                    auto kern = k_spmm_v<T, VL, VW, DPP>;
                    const size_t smem = (size_t)256 * VW * DPP * sizeof(double);
                    const int per_sm = std::min(4, spmm_fused_v_per_sm<T, VL, VW, DPP>());
                    const int64_t gf = std::min<int64_t>(g, (int64_t)sm_count() * per_sm);
                    if (dparts) *dparts = (int)gf;
                    allow_large_smem(kern, smem);
                    kern<<<(unsigned)gf, 256, smem, st>>>(op, ncols, group, prm, X, Y, dpart);
                }
            };
            if (group == 2) fused(std::integral_constant<int, 2>());
            else fused(std::integral_constant<int, 4>());
        };
        if constexpr (!MF) by_vshape(v.L, v.VW, go);
        return spmm_bytes<T, MF>(op, ncols);
    }
    if (spmm_fuses(MF, dpart != nullptr, ncols, group)) {
        // fused X^T Y partials (CSR, one pass over the columns, block size 2
        // or 4) on one resident wave (fewer partial rows to reduce, no tail wave)
        const int rpb = 256 / L;
        const int64_t g = std::max<int64_t>(1, std::min<int64_t>((D + rpb - 1) / rpb, (int64_t)sm_count() * 16));
        auto go = [&](auto lc, auto cwc) {
            constexpr int LL = decltype(lc)::value, CC = decltype(cwc)::value;
            auto fused = [&](auto dpc) {
                constexpr int DPP = decltype(dpc)::value;
                const int per_sm = std::min(4, spmm_fused_per_sm<T, LL, CC, DPP>());
                const int64_t gf = std::min<int64_t>(g, (int64_t)sm_count() * per_sm);
                if (dparts) *dparts = (int)gf;
                k_spmm<T, LL, CC, DPP><<<(unsigned)gf, 256, 256 * CC * DPP * sizeof(double), st>>>(
                    op, ncols, group, prm, X, Y, dpart);
            };
            if (group == 2) fused(std::integral_constant<int, 2>());
            else fused(std::integral_constant<int, 4>());
        };
        if constexpr (!MF) by_shape(L, CW, go);
        return spmm_bytes<T, MF>(op, ncols);
    }
    SpmmShape s = def;
    SpmmChoice c;
    if (tuned && tune_lookup(tune_key(op, ncols), &c)) s = spmm_resolve(c, ncols, MF);
    spmm_launch_plain<T, MF>(op, ncols, group, prm, X, Y, st, s);
    return spmm_bytes<T, MF>(op, ncols);
}

template <class T, bool MF>
double launch_spmm_shape_kind(const OpView<T>& op, int ncols, int group, const double* prm,
                              const T* X, T* Y, cudaStream_t st, const SpmmShape& s) {
    BH_REQUIRE(spmm_shape_valid(s, ncols, MF),
               "launch shape: lanes must be a power of two <= 32 dividing the column count "
               "(32 at any count for the matrix-free product), columns per lane 1 or 4 (or 2 "
               "with 32 lanes), grid >= -1");
    spmm_launch_plain<T, MF>(op, ncols, group, prm, X, Y, st, s);
    return spmm_bytes<T, MF>(op, ncols);
}

// Event pair that is destroyed with its scope.
struct TimerPair {
    cudaEvent_t a = nullptr, b = nullptr;
    TimerPair() {
        BH_CUDA(cudaEventCreate(&a));
        BH_CUDA(cudaEventCreate(&b));
    }
    ~TimerPair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

template <class T, bool MF>
int tune_spmm_kind(const OpView<T>& op, int ncols, int group, const double* prm, const T* X, T* Y,
                   cudaStream_t st, bool has_dpart, bool force, TuneEntry* out) {
    if (!force && !autotune_on()) return 0;
    if (op.D < 1 || spmm_fuses(MF, has_dpart, ncols, group)) return 0;
    const TuneKey key = tune_key(op, ncols);
    if (!force && tune_lookup(key, nullptr)) return 0;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    BH_CUDA(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone) return 0;

    const std::vector<SpmmChoice> cands = spmm_candidates(ncols, MF);
    int launches = 0;
    // each candidate's kernel once on the first rows only (module loading and
    // first-launch costs stay out of the timings); rows below 256 of Y get
    // the values of the full product
    OpView<T> head = op;
    head.D = std::min<int64_t>(op.D, 256);
    for (const SpmmChoice& c : cands) {
        spmm_launch_plain<T, MF>(head, ncols, group, prm, X, Y, st, spmm_resolve(c, ncols, MF));
        ++launches;
    }
    BH_CUDA(cudaGetLastError());
    TimerPair ev;
    // the fastest of `reps` separately timed launches (products of other
    // streams running at the same time only ever lengthen a launch)
    auto time_ms = [&](const SpmmShape& s, int reps) {
        float best = 0.f;
        for (int i = 0; i < reps; ++i) {
            BH_CUDA(cudaEventRecord(ev.a, st));
            spmm_launch_plain<T, MF>(op, ncols, group, prm, X, Y, st, s);
            BH_CUDA(cudaEventRecord(ev.b, st));
            BH_CUDA(cudaGetLastError());
            BH_CUDA(cudaEventSynchronize(ev.b));
            float ms = 0.f;
            BH_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
            best = i == 0 ? ms : std::min(best, ms);
        }
        launches += reps;
        return best;
    };
    // the default first; products above 0.25 ms are timed once per shape,
    // and above 2 ms only the default, one step fewer lanes and one wave run
    float t_def = time_ms(spmm_resolve(cands[0], ncols, MF), 1);
    const int reps = t_def < 0.25f ? 3 : 1;
    if (reps > 1) t_def = std::min(t_def, time_ms(spmm_resolve(cands[0], ncols, MF), reps));
    const bool expensive = t_def > 2.0f;
    size_t best = 0;
    float t_best = t_def;
    int timed = 1;
    for (size_t i = 1; i < cands.size(); ++i) {
        const SpmmChoice& c = cands[i];
        if (expensive && (c.narrow || c.dl > 1 || (c.dl == 1 && c.wave))) continue;
        const float t = time_ms(spmm_resolve(c, ncols, MF), reps);
        ++timed;
        if (t < t_best) {
            t_best = t;
            best = i;
        }
    }
    // keep the default unless another shape is clearly faster (3%)
    if (best != 0 && t_best > 0.97f * t_def) {
        best = 0;
        t_best = t_def;
    }
    TuneEntry e;
    e.choice = cands[best];
    e.ncols = ncols;
    e.shape = spmm_resolve(cands[best], ncols, MF);
    e.ms = t_best;
    e.ms_default = t_def;
    e.candidates = timed;
    tune_store(key, e);
    if (out) *out = e;
    return launches;
}

}  // namespace bh
