// bh_krylov.cu -- device-resident block thick-restart Lanczos, batched.
//
// Replaces Op::IRLM_eigen (src/operator.cpp:22-33), i.e. Spectra's
// implicitly restarted Arnoldi (GenEigsBase.h:417-441, Arnoldi.h:183-280), and
// the per-point OpenMP loop around it (src/analysis.cpp:302-314).
//
// S independent solves that share one sparsity pattern (the (J, U, mu) points
// of a phase-diagram grid: H = J T + U V - mu N) run in lock-step as one
// batch.  Every Krylov block of the batch is one row-major D x (S p) array, so
// one SpMM streams T once per step for all S p vectors and every gathered row
// of X is a contiguous S p-vector.  Per block step j:
//     W  = H V_j                                         k_spmm
//     A  = V_j^T W;  W -= V_j A + V_{j-1} R_{j-1}^T      k_dot + k_local_coef + k_update
//          (after a thick restart: + V_keep S^T, the arrowhead coupling)
//     C  = [V_0..V_j]^T W;  W -= [V_0..V_j] C            k_dot + k_dot_finalize + k_update
//          (one full classical Gram-Schmidt re-orthogonalisation pass; the
//           Gram matrix W^T W is accumulated in the same pass)
//     W  = V_{j+1} R  (Cholesky QR)                      k_qr_finalize + k_normalize
// The projected matrix T (FP64) is assembled on the device from A, R and C;
// the host reads it only at a restart, solves the small eigenproblems in FP64,
// and sends back the Ritz rotation applied by k_rotate.  At each restart the
// solves that have converged are retired (their Ritz vectors are rotated out)
// and the remaining ones are compacted into a narrower batch.
//
// Vectors are FP64 (plain method) or FP32 (mixed); the coefficients A, C, R
// and all reductions are FP64 (FP32 partial sums over at most 32 rows are
// folded into FP64 accumulators).  A final FP64 Rayleigh-Ritz on the Ritz
// vectors (FP64 SpMM, FP64 Gram matrices, FP64 generalised eigensolve) gives
// the returned eigenvalues and their true FP64 residuals.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <numeric>
#include <thread>
#include <type_traits>

#include "bh_krylov.cuh"

namespace bh {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// Partial sums of C_s[(j p + q)][q'] = sum_r V_j[r][s p + q] W[r][s p + q'] over
// one chunk of rows (blockIdx.x) and JT blocks j (blockIdx.y).
// part layout: [chunk][c < kcap][ncols]  (row c, column s p + q').
template <class T, int PMAX, int JT>
__global__ void __launch_bounds__(512)
k_dot(int64_t D, int ncols, int ld, int p, int nblk, int64_t bstride, const T* __restrict__ V,
      const T* __restrict__ W, int64_t rows_per_chunk, int kcap, double* __restrict__ part) {
    extern __shared__ double s_red[];
    const int t = threadIdx.x % ncols, ro = threadIdx.x / ncols, R = blockDim.x / ncols;
    const int s = t / p, q = t % p;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t r1 = min(D, r0 + rows_per_chunk);
    const int j0 = blockIdx.y * JT;
    const int nj = min(JT, nblk - j0);
    double accd[JT][PMAX];
    T accf[JT][PMAX];
#pragma unroll
    for (int a = 0; a < JT; ++a)
#pragma unroll
        for (int b = 0; b < PMAX; ++b) {
            accd[a][b] = 0.0;
            accf[a][b] = T(0);
        }
    int cnt = 0;
    for (int64_t r = r0 + ro; r < r1; r += R) {
        const T* wr = W + r * ld + s * p;
        T w[PMAX];
#pragma unroll
        for (int b = 0; b < PMAX; ++b) w[b] = b < p ? wr[b] : T(0);
#pragma unroll
        for (int a = 0; a < JT; ++a) {
            if (a < nj) {
                const T v = V[(int64_t)(j0 + a) * bstride + r * ld + t];
#pragma unroll
                for (int b = 0; b < PMAX; ++b) accf[a][b] += v * w[b];
            }
        }
        if (++cnt == 32) {
            cnt = 0;
#pragma unroll
            for (int a = 0; a < JT; ++a)
#pragma unroll
                for (int b = 0; b < PMAX; ++b) {
                    accd[a][b] += (double)accf[a][b];
                    accf[a][b] = T(0);
                }
        }
    }
#pragma unroll
    for (int a = 0; a < JT; ++a)
#pragma unroll
        for (int b = 0; b < PMAX; ++b) s_red[(size_t)threadIdx.x * (JT * PMAX) + a * PMAX + b] =
            accd[a][b] + (double)accf[a][b];
    __syncthreads();
    if (ro == 0) {
        for (int a = 0; a < nj; ++a)
            for (int b = 0; b < p; ++b) {
                double sum = 0.0;
                for (int u = 0; u < R; ++u)
                    sum += s_red[(size_t)(u * ncols + t) * (JT * PMAX) + a * PMAX + b];
                part[((size_t)blockIdx.x * kcap + (size_t)(j0 + a) * p + q) * ncols + s * p + b] = sum;
            }
    }
}

// Sum of one coefficient's chunk partials by one warp (lanes stride over the
// chunks, then a fixed-order shuffle tree): the result is deterministic.
__device__ __forceinline__ double warp_sum_chunks(const double* __restrict__ part, int nchunks,
                                                  size_t chunk_stride, size_t offset) {
    const int lane = threadIdx.x & 31;
    // four independent partial sums per lane (chunks lane + 32 (4 i + k)), so
    // that four loads are in flight; fixed order, so the result is deterministic
    double v0 = 0.0, v1 = 0.0, v2 = 0.0, v3 = 0.0;
    int ch = lane;
    for (; ch + 96 < nchunks; ch += 128) {
        v0 += part[(size_t)ch * chunk_stride + offset];
        v1 += part[(size_t)(ch + 32) * chunk_stride + offset];
        v2 += part[(size_t)(ch + 64) * chunk_stride + offset];
        v3 += part[(size_t)(ch + 96) * chunk_stride + offset];
    }
    for (; ch < nchunks; ch += 32) v0 += part[(size_t)ch * chunk_stride + offset];
    double v = (v0 + v1) + (v2 + v3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// C = sum over chunks; Cf = (T)C; optionally T_s[c][jcol p + q'] += C.
// One warp per coefficient.
template <class T>
__global__ void k_dot_finalize(int nchunks, int kc, int ncols, int ldC, int p, int kcap,
                               const double* __restrict__ part, double* __restrict__ C,
                               T* __restrict__ Cf, double* __restrict__ Tm, int Tdim, int jcol) {
    const int total = kc * ncols;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int idx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; idx < total; idx += warps) {
        const int c = idx / ncols, t = idx % ncols;
        const double sum = warp_sum_chunks(part, nchunks, (size_t)kcap * ncols, (size_t)c * ncols + t);
        if ((threadIdx.x & 31) != 0) continue;
        if (C) C[(size_t)c * ldC + t] = sum;
        if (Cf) Cf[(size_t)c * ldC + t] = (T)sum;
        if (Tm) {
            const int s = t / p, q = t % p;
            Tm[(size_t)s * Tdim * Tdim + (size_t)(jcol * p + q) * Tdim + c] += sum;
        }
    }
}

// Coefficients of the local block-Lanczos step for column block j, rows
// c in [c_lo, (j+1) p):
//   rows of block j      : A = V_j^T W (from the chunk partials of a 1-block k_dot)
//   rows below block j   : the known couplings of the new block with the
//                          earlier columns, T_s[j p + q'][c] (lower part:
//                          R_{j-1} from the previous QR, or the arrowhead rows
//                          written at a thick restart)
// Cf[(c - c_lo)][s p + q'] receives them, and T_s[c][j p + q'] += them.
template <class T>
__global__ void k_local_coef(int nchunks, int j, int c_lo, int ncols, int p, int kcap,
                             const double* __restrict__ part, double* __restrict__ Tm, int Tdim,
                             T* __restrict__ Cf) {
    const int rows = (j + 1) * p - c_lo;
    const int total = rows * ncols;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int idx = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; idx < total; idx += warps) {
        const int cr = idx / ncols, t = idx % ncols;
        const int c = c_lo + cr;
        const int s = t / p, q = t % p;
        double* Ts = Tm + (size_t)s * Tdim * Tdim;
        double v;
        if (c >= j * p)
            v = warp_sum_chunks(part, nchunks, (size_t)kcap * ncols, (size_t)(c - j * p) * ncols + t);
        else
            v = Ts[(size_t)c * Tdim + j * p + q];
        if ((threadIdx.x & 31) != 0) continue;
        Cf[(size_t)cr * ncols + t] = (T)v;
        Ts[(size_t)(j * p + q) * Tdim + c] += v;
    }
}

// W[r][s p + q'] -= sum_{c < kc} V_{c/p}[r][s p + c%p] Cf[c][s p + q'], then
// (optionally) Gram partials G_s[q][q'] = sum_r W[r][s p + q] W[r][s p + q'].
// Two rows per iteration and four columns of C per inner step keep eight
// independent loads in flight per thread.
template <class T, int PMAX>
__global__ void __launch_bounds__(256)
k_update(int64_t D, int ncols, int p, int lp, int kc, int64_t bstride, const T* __restrict__ V,
         const T* __restrict__ Cf, T* __restrict__ W, int64_t rows_per_cta, int do_gram,
         double* __restrict__ gpart) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    T* sC = reinterpret_cast<T*>(s_raw);
    double* sG = reinterpret_cast<double*>(s_raw + (((size_t)kc * ncols * sizeof(T) + 15) & ~(size_t)15));
    for (int i = threadIdx.x; i < kc * ncols; i += blockDim.x) sC[i] = Cf[i];
    __syncthreads();
    const int t = threadIdx.x % ncols, ro = threadIdx.x / ncols, R = blockDim.x / ncols;
    const int s = t / p, q = t % p, pm = p - 1;
    const int lane = threadIdx.x & 31;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per_cta;
    const int64_t r1 = min(D, r0 + rows_per_cta);
    double gd[PMAX];
    T gf[PMAX];
#pragma unroll
    for (int b = 0; b < PMAX; ++b) {
        gd[b] = 0.0;
        gf[b] = T(0);
    }
    int cnt = 0;
    for (int64_t base = r0; base < r1; base += 2 * R) {
        const int64_t rA = base + ro, rB = rA + R;
        const bool vA = rA < r1, vB = rB < r1;
        T wA = vA ? W[rA * ncols + t] : T(0);
        T wB = vB ? W[rB * ncols + t] : T(0);
        if (kc > 0 && (vA || vB)) {
            const T* pA = V + (vA ? rA : r0) * ncols + s * p;
            const T* pB = V + (vB ? rB : r0) * ncols + s * p;
            T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
            T b0 = T(0), b1 = T(0), b2 = T(0), b3 = T(0);
            int c = 0;
            for (; c + 3 < kc; c += 4) {
                const int64_t o0 = (int64_t)(c >> lp) * bstride + (c & pm);
                const int64_t o1 = (int64_t)((c + 1) >> lp) * bstride + ((c + 1) & pm);
                const int64_t o2 = (int64_t)((c + 2) >> lp) * bstride + ((c + 2) & pm);
                const int64_t o3 = (int64_t)((c + 3) >> lp) * bstride + ((c + 3) & pm);
                const T x0 = pA[o0], x1 = pA[o1], x2 = pA[o2], x3 = pA[o3];
                const T y0 = pB[o0], y1 = pB[o1], y2 = pB[o2], y3 = pB[o3];
                const T k0 = sC[c * ncols + t], k1 = sC[(c + 1) * ncols + t];
                const T k2 = sC[(c + 2) * ncols + t], k3 = sC[(c + 3) * ncols + t];
                a0 += x0 * k0;
                a1 += x1 * k1;
                a2 += x2 * k2;
                a3 += x3 * k3;
                b0 += y0 * k0;
                b1 += y1 * k1;
                b2 += y2 * k2;
                b3 += y3 * k3;
            }
            for (; c < kc; ++c) {
                const int64_t o0 = (int64_t)(c >> lp) * bstride + (c & pm);
                const T k0 = sC[c * ncols + t];
                a0 += pA[o0] * k0;
                b0 += pB[o0] * k0;
            }
            // rows past the chunk end read a valid row but must stay zero
            wA = vA ? wA - ((a0 + a1) + (a2 + a3)) : T(0);
            wB = vB ? wB - ((b0 + b1) + (b2 + b3)) : T(0);
            if (vA) W[rA * ncols + t] = wA;
            if (vB) W[rB * ncols + t] = wB;
        }
        if (do_gram) {
#pragma unroll
            for (int b = 0; b < PMAX; ++b) {
                if (b < p) {
                    const T xa = __shfl_sync(0xffffffffu, wA, lane - q + b);
                    const T xb = __shfl_sync(0xffffffffu, wB, lane - q + b);
                    gf[b] += xa * wA + xb * wB;
                }
            }
            if (++cnt == 16) {
                cnt = 0;
#pragma unroll
                for (int b = 0; b < PMAX; ++b) {
                    gd[b] += (double)gf[b];
                    gf[b] = T(0);
                }
            }
        }
    }
    if (do_gram) {
#pragma unroll
        for (int b = 0; b < PMAX; ++b) sG[(size_t)threadIdx.x * PMAX + b] = gd[b] + (double)gf[b];
        __syncthreads();
        if (ro == 0)
            for (int b = 0; b < p; ++b) {
                double sum = 0.0;
                for (int u = 0; u < R; ++u) sum += sG[(size_t)(u * ncols + t) * PMAX + b];
                gpart[((size_t)blockIdx.x * p + b) * ncols + t] = sum;  // G_s[b][q] at column t
            }
    }
}

// ---- per-solve vector kernels for block sizes P = 1, 2, 4 ----
// A thread owns all P columns of one solve in a row: loads are P-wide vectors
// (a warp reads 32 solves x P contiguous values), and the P x P products of a
// block need no data from other lanes.
template <class T, int P>
struct Vec {
    T v[P];
};

template <class T, int P>
__device__ __forceinline__ Vec<T, P> ldv(const T* __restrict__ p) {
    Vec<T, P> o;
    if constexpr (P == 1) {
        o.v[0] = p[0];
    } else if constexpr (std::is_same<T, float>::value && P == 2) {
        const float2 x = *reinterpret_cast<const float2*>(p);
        o.v[0] = x.x;
        o.v[1] = x.y;
    } else if constexpr (std::is_same<T, float>::value && P == 4) {
        const float4 x = *reinterpret_cast<const float4*>(p);
        o.v[0] = x.x;
        o.v[1] = x.y;
        o.v[2] = x.z;
        o.v[3] = x.w;
    } else {
#pragma unroll
        for (int q = 0; q < P; q += 2) {
            const double2 x = *reinterpret_cast<const double2*>(p + q);
            o.v[q] = x.x;
            o.v[q + 1] = x.y;
        }
    }
    return o;
}

template <class T, int P>
__device__ __forceinline__ void stv(T* __restrict__ p, const Vec<T, P>& o) {
    if constexpr (P == 1) {
        p[0] = o.v[0];
    } else if constexpr (std::is_same<T, float>::value && P == 2) {
        *reinterpret_cast<float2*>(p) = make_float2(o.v[0], o.v[1]);
    } else if constexpr (std::is_same<T, float>::value && P == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(o.v[0], o.v[1], o.v[2], o.v[3]);
    } else {
#pragma unroll
        for (int q = 0; q < P; q += 2) *reinterpret_cast<double2*>(p + q) = make_double2(o.v[q], o.v[q + 1]);
    }
}

// Partial sums of C_s[(j P + q)][q'] = sum_r V_j[r][s P + q] W[r][s P + q']
// over one chunk of rows (blockIdx.y) and JT blocks (tile blockIdx.x: the
// tiles of one chunk run side by side, so W's chunk is read from DRAM once).
// Thread = (solve s, row group ro); the loads of RU rows (JT + 1 vectors
// each) are issued before their products.  Products are summed in T per
// thread and flushed every 32 rows into the thread's own FP64 slots in shared
// memory (s_red[val NT + tid]), which the CTA then sums over the row groups
// in a fixed order.  part layout as k_dot.
template <class T, int P, int JT, int RU>
__global__ void __launch_bounds__(128)
k_dotv(int64_t D, int S, int nblk, int64_t bstride, const T* __restrict__ V,
       const T* __restrict__ W, int64_t rows_per_chunk, int kcap, double* __restrict__ part) {
    extern __shared__ double s_red[];
    constexpr int NV = JT * P * P;
    const int NT = blockDim.x;
    const int ncols = S * P;
    const int s = threadIdx.x % S, ro = threadIdx.x / S, R = NT / S;
    const int64_t r0 = (int64_t)blockIdx.y * rows_per_chunk;
    const int64_t r1 = min(D, r0 + rows_per_chunk);
    const int j0 = blockIdx.x * JT;
    const int nj = min(JT, nblk - j0);
    double* mine = s_red + threadIdx.x;
#pragma unroll
    for (int v = 0; v < NV; ++v) mine[(size_t)v * NT] = 0.0;
    T acc[JT][P][P];
#pragma unroll
    for (int a = 0; a < JT; ++a)
#pragma unroll
        for (int q = 0; q < P; ++q)
#pragma unroll
            for (int b = 0; b < P; ++b) acc[a][q][b] = T(0);
    const T* Vb = V + (int64_t)j0 * bstride + s * P;
    const T* Wb = W + s * P;
    int cnt = 0;
    for (int64_t base = r0 + ro; base < r1; base += RU * R) {
        Vec<T, P> w[RU], x[RU][JT];
#pragma unroll
        for (int u = 0; u < RU; ++u) {
            const int64_t r = base + (int64_t)u * R;
            const int64_t rr = r < r1 ? r : base;  // a valid row; its products are dropped
            w[u] = ldv<T, P>(Wb + rr * ncols);
#pragma unroll
            for (int a = 0; a < JT; ++a)
                if (a < nj) x[u][a] = ldv<T, P>(Vb + (int64_t)a * bstride + rr * ncols);
            if (r >= r1)
#pragma unroll
                for (int b = 0; b < P; ++b) w[u].v[b] = T(0);
        }
#pragma unroll
        for (int u = 0; u < RU; ++u)
#pragma unroll
            for (int a = 0; a < JT; ++a)
                if (a < nj)
#pragma unroll
                    for (int q = 0; q < P; ++q)
#pragma unroll
                        for (int b = 0; b < P; ++b) acc[a][q][b] += x[u][a].v[q] * w[u].v[b];
        cnt += RU;
        if (cnt >= 32) {
            cnt = 0;
#pragma unroll
            for (int a = 0; a < JT; ++a)
#pragma unroll
                for (int q = 0; q < P; ++q)
#pragma unroll
                    for (int b = 0; b < P; ++b) {
                        mine[(size_t)((a * P + q) * P + b) * NT] += (double)acc[a][q][b];
                        acc[a][q][b] = T(0);
                    }
        }
    }
#pragma unroll
    for (int a = 0; a < JT; ++a)
#pragma unroll
        for (int q = 0; q < P; ++q)
#pragma unroll
            for (int b = 0; b < P; ++b) mine[(size_t)((a * P + q) * P + b) * NT] += (double)acc[a][q][b];
    __syncthreads();
    // one thread per (value, solve) sums the R row groups in order
    for (int e = threadIdx.x; e < NV * S; e += NT) {
        const int val = e / S, ss = e % S;
        const int a = val / (P * P), q = (val / P) % P, b = val % P;
        if (a >= nj) continue;
        double sum = 0.0;
        for (int u = 0; u < R; ++u) sum += s_red[(size_t)val * NT + u * S + ss];
        part[((size_t)blockIdx.y * kcap + (size_t)(j0 + a) * P + q) * ncols + ss * P + b] = sum;
    }
}

// W[r][s P + q'] -= sum_{c < kc} V_{c/P}[r][s P + c%P] Cf[c][s P + q'], then
// (optionally) Gram partials G_s[q][q'] = sum_r W[r][s P + q] W[r][s P + q']
// written as gpart[(cta P + q) ncols + s P + q'] (the k_update layout).
// Two rows per iteration; the inner step issues the loads of several basis
// blocks before using them.
template <class T, int P>
__global__ void __launch_bounds__(256)
k_updatev(int64_t D, int S, int nblk, int64_t bstride, const T* __restrict__ V,
          const T* __restrict__ Cf, T* __restrict__ W, int64_t rows_per_cta, int do_gram,
          double* __restrict__ gpart) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    const int ncols = S * P;
    const int kc = nblk * P;
    T* sC = reinterpret_cast<T*>(s_raw);
    double* sG = reinterpret_cast<double*>(s_raw + (((size_t)kc * ncols * sizeof(T) + 15) & ~(size_t)15));
    for (int i = threadIdx.x; i < kc * ncols; i += blockDim.x) sC[i] = Cf[i];
    __syncthreads();
    const int s = threadIdx.x % S, ro = threadIdx.x / S, R = blockDim.x / S;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per_cta;
    const int64_t r1 = min(D, r0 + rows_per_cta);
    double gd[P][P];
    T gf[P][P];
#pragma unroll
    for (int q = 0; q < P; ++q)
#pragma unroll
        for (int b = 0; b < P; ++b) {
            gd[q][b] = 0.0;
            gf[q][b] = T(0);
        }
    int cnt = 0;
    const T* Vs = V + s * P;
    for (int64_t base = r0; base < r1; base += 2 * R) {
        const int64_t rA = base + ro, rB = rA + R;
        const bool vA = rA < r1, vB = rB < r1;
        Vec<T, P> wA, wB;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            wA.v[q] = T(0);
            wB.v[q] = T(0);
        }
        if (vA) wA = ldv<T, P>(W + rA * ncols + s * P);
        if (vB) wB = ldv<T, P>(W + rB * ncols + s * P);
        if (nblk > 0 && vA) {
            const T* pA = Vs + rA * ncols;
            const T* pB = Vs + (vB ? rB : rA) * ncols;
            T aA[P], aB[P];
#pragma unroll
            for (int q = 0; q < P; ++q) {
                aA[q] = T(0);
                aB[q] = T(0);
            }
            constexpr int U = P >= 4 ? 4 : 8;  // blocks per inner step: 2 U vector loads in flight
            int j = 0;
            for (; j + U - 1 < nblk; j += U) {
                Vec<T, P> x[U], y[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    x[u] = ldv<T, P>(pA + (int64_t)(j + u) * bstride);
                    y[u] = ldv<T, P>(pB + (int64_t)(j + u) * bstride);
                }
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int q = 0; q < P; ++q) {
                        const Vec<T, P> c = ldv<T, P>(sC + (size_t)((j + u) * P + q) * ncols + s * P);
#pragma unroll
                        for (int b = 0; b < P; ++b) {
                            aA[b] += x[u].v[q] * c.v[b];
                            aB[b] += y[u].v[q] * c.v[b];
                        }
                    }
            }
            for (; j < nblk; ++j) {
                const Vec<T, P> x0 = ldv<T, P>(pA + (int64_t)j * bstride);
                const Vec<T, P> y0 = ldv<T, P>(pB + (int64_t)j * bstride);
#pragma unroll
                for (int q = 0; q < P; ++q) {
                    const Vec<T, P> c = ldv<T, P>(sC + (size_t)(j * P + q) * ncols + s * P);
#pragma unroll
                    for (int b = 0; b < P; ++b) {
                        aA[b] += x0.v[q] * c.v[b];
                        aB[b] += y0.v[q] * c.v[b];
                    }
                }
            }
#pragma unroll
            for (int b = 0; b < P; ++b) {
                wA.v[b] -= aA[b];
                wB.v[b] = vB ? wB.v[b] - aB[b] : T(0);
            }
            stv<T, P>(W + rA * ncols + s * P, wA);
            if (vB) stv<T, P>(W + rB * ncols + s * P, wB);
        }
        if (do_gram) {
#pragma unroll
            for (int q = 0; q < P; ++q)
#pragma unroll
                for (int b = 0; b < P; ++b) gf[q][b] += wA.v[q] * wA.v[b] + wB.v[q] * wB.v[b];
            if (++cnt == 16) {
                cnt = 0;
#pragma unroll
                for (int q = 0; q < P; ++q)
#pragma unroll
                    for (int b = 0; b < P; ++b) {
                        gd[q][b] += (double)gf[q][b];
                        gf[q][b] = T(0);
                    }
            }
        }
    }
    if (do_gram) {
#pragma unroll
        for (int q = 0; q < P; ++q)
#pragma unroll
            for (int b = 0; b < P; ++b) sG[(size_t)(q * P + b) * blockDim.x + threadIdx.x] = gd[q][b] + (double)gf[q][b];
        __syncthreads();
        for (int e = threadIdx.x; e < P * P * S; e += blockDim.x) {
            const int val = e / S, ss = e % S;
            const int q = val / P, b = val % P;
            double sum = 0.0;
            for (int u = 0; u < R; ++u) sum += sG[(size_t)val * blockDim.x + u * S + ss];
            gpart[((size_t)blockIdx.x * P + q) * ncols + ss * P + b] = sum;
        }
    }
}

// One CTA per solve: G = sum of the Gram partials (fixed-order tree
// reduction), then one pass of the block orthonormalisation W = Q R:
//   mode 0  shifted Cholesky  G + s I = R^T R, s = shift_rel * max_i G_ii,
//           which always exists and bounds cond(W R^{-1}); Racc <- R
//   mode 1  Cholesky G = R^T R;  Racc <- R Racc
//   mode 2  Cholesky G = R^T R;  Rtot = R Racc is the block coupling,
//           written to T_s[(jrow p + a)][(jrow - 1) p + b]  (final pass)
// (shifted CholQR3: the product of the three factors is exact, and the
// last two passes restore orthonormality to working precision).  For p = 1
// a single mode-2 pass normalises the vector.  In the final pass a
// direction whose norm |Rtot_ii| is below kill_abs * (its norm before
// orthogonalisation) is numerically inside the span of the basis: it is
// dropped (zero column of Rinv, zero row of the coupling, dead flag set).
// The norm before orthogonalisation is sqrt(sum_c T[c][col]^2 + |Rtot_.i|^2)
// with col = (jrow - 1) p + i, the coefficients of H v_col in the basis.
constexpr int QR_THREADS = 128;
// The serial part of k_qr_finalize (thread 0 of a solve's CTA): the p x p
// Cholesky factor of G (shifted in mode 0), the accumulated factor, the
// dropped directions, the inverse on the kept ones, and the writes.  PM is
// the block capacity: PM <= 4 unrolls every loop so the factors stay in
// registers; larger blocks run the same loops with the factors in local memory.
template <int PM>
__device__ __forceinline__ void qr_factor(int p, int s, int mode, double shift_rel, const double (*G)[16],
                                          const double* s_pre, const double* sRa, bool final_check,
                                          double* __restrict__ Racc,
                                          double* __restrict__ Rinv, double* __restrict__ Tm, int Tdim, int jrow,
                                          double kill_abs, unsigned char* __restrict__ dead,
                                          int* __restrict__ need3) {
    if constexpr (PM <= 4) {
    // the p x p factors in registers: every loop below runs to the capacity
        // PM (unrolled for PM <= 4, so the arrays are indexed by constants) and
        // stops at p; larger blocks keep them in local memory
        double R[PM][PM], Ri[PM][PM], Rt[PM][PM];
#pragma unroll
        for (int a = 0; a < PM; ++a)
#pragma unroll
            for (int b = 0; b < PM; ++b) {
                R[a][b] = 0.0;
                Ri[a][b] = 0.0;
                Rt[a][b] = 0.0;
            }
        double* Ra = Racc + (size_t)s * p * p;
        auto cholesky = [&](double shift) {
            double dmin = INFINITY;
#pragma unroll
            for (int i = 0; i < PM; ++i) {
                if (i >= p) break;
                double d = G[i][i] + shift;
#pragma unroll
                for (int k = 0; k < i; ++k) d -= R[k][i] * R[k][i];
                dmin = fmin(dmin, d);
                R[i][i] = 0.0;
#pragma unroll
                for (int j = i + 1; j < PM; ++j) R[i][j] = 0.0;
                if (!(d > 0.0)) continue;  // zero column (already dropped) stays zero
                const double rii = sqrt(d);
                R[i][i] = rii;
#pragma unroll
                for (int j = i + 1; j < PM; ++j) {
                    if (j >= p) break;
                    double v = 0.5 * (G[i][j] + G[j][i]);
#pragma unroll
                    for (int k = 0; k < i; ++k) v -= R[k][i] * R[k][j];
                    R[i][j] = v / rii;
                }
            }
            return dmin;
        };
        if (mode == 0) {
            double gmax = 0.0;
            for (int i = 0; i < p; ++i) gmax = fmax(gmax, G[i][i]);
            // well conditioned (every pivot >= 1e-4 of the largest diagonal
            // entry, i.e. cond(W)^2 <= 1e4): plain Cholesky, and two passes
            // (CholQR2) orthonormalise to working precision.  Otherwise the
            // shifted first pass, and the step needs all three.
            bool plain = need3 != nullptr && gmax > 0.0;
            if (plain) plain = cholesky(0.0) >= 1e-4 * gmax;
            if (!plain) {
                cholesky(shift_rel * gmax);
                if (need3) atomicAdd(need3, 1);
            }
        } else {
            cholesky(0.0);
        }
        // accumulated factor Rt = R * Racc (upper triangular products)
#pragma unroll
        for (int a = 0; a < PM; ++a) {
            if (a >= p) break;
#pragma unroll
            for (int b = 0; b < PM; ++b) {
                if (b >= p) break;
                if (mode == 0 || p == 1) {
                    Rt[a][b] = R[a][b];
                } else {
                    double v = 0.0;
#pragma unroll
                    for (int k = a; k <= b; ++k) v += R[a][k] * sRa[k * p + b];
                    Rt[a][b] = v;
                }
            }
        }
        const bool final_pass = mode == 2;
        bool drop[PM];
#pragma unroll
        for (int i = 0; i < PM; ++i) drop[i] = i < p && R[i][i] == 0.0;
        if (final_check) {
#pragma unroll
            for (int i = 0; i < PM; ++i) {
                if (i >= p) break;
                double own = 0.0;
#pragma unroll
                for (int k = 0; k <= i; ++k) own += Rt[k][i] * Rt[k][i];
                if (!(fabs(Rt[i][i]) > kill_abs * sqrt(s_pre[i] + own))) drop[i] = true;
            }
        }
        // inverse of this pass's R on the kept directions
#pragma unroll
        for (int j = 0; j < PM; ++j) {
            if (j >= p) break;
            if (drop[j] && final_pass) continue;
            if (R[j][j] == 0.0) continue;
            Ri[j][j] = 1.0 / R[j][j];
#pragma unroll
            for (int i = j - 1; i >= 0; --i) {
                if (R[i][i] == 0.0) continue;
                double v = 0.0;
#pragma unroll
                for (int k = i + 1; k <= j; ++k) v += R[i][k] * Ri[k][j];
                Ri[i][j] = -v / R[i][i];
            }
        }
#pragma unroll
        for (int a = 0; a < PM; ++a) {
            if (a >= p) break;
#pragma unroll
            for (int b = 0; b < PM; ++b) {
                if (b >= p) break;
                Rinv[(size_t)s * p * p + a * p + b] = Ri[a][b];
                Ra[a * p + b] = (final_pass && drop[a]) ? 0.0 : Rt[a][b];
            }
        }
        if (!final_pass) return;
        if (Tm && jrow > 0) {
            double* Tw = Tm + (size_t)s * Tdim * Tdim;
#pragma unroll
            for (int a = 0; a < PM; ++a) {
                if (a >= p) break;
#pragma unroll
                for (int b = 0; b < PM; ++b) {
                    if (b >= p) break;
                    Tw[(size_t)((jrow - 1) * p + b) * Tdim + jrow * p + a] = drop[a] ? 0.0 : Rt[a][b];
                }
            }
            if (dead)
#pragma unroll
                for (int a = 0; a < PM; ++a)
                    if (a < p) dead[(size_t)s * Tdim + jrow * p + a] = drop[a] ? 1 : 0;
        }
    } else {
    // the p x p factors in registers: every loop below runs to the capacity
        // PM (unrolled for PM <= 4, so the arrays are indexed by constants) and
        // stops at p; larger blocks keep them in local memory
        double R[PM][PM], Ri[PM][PM], Rt[PM][PM];
#pragma unroll 1
        for (int a = 0; a < PM; ++a)
#pragma unroll 1
            for (int b = 0; b < PM; ++b) {
                R[a][b] = 0.0;
                Ri[a][b] = 0.0;
                Rt[a][b] = 0.0;
            }
        double* Ra = Racc + (size_t)s * p * p;
        auto cholesky = [&](double shift) {
            double dmin = INFINITY;
#pragma unroll 1
            for (int i = 0; i < PM; ++i) {
                if (i >= p) break;
                double d = G[i][i] + shift;
#pragma unroll 1
                for (int k = 0; k < i; ++k) d -= R[k][i] * R[k][i];
                dmin = fmin(dmin, d);
                R[i][i] = 0.0;
#pragma unroll 1
                for (int j = i + 1; j < PM; ++j) R[i][j] = 0.0;
                if (!(d > 0.0)) continue;  // zero column (already dropped) stays zero
                const double rii = sqrt(d);
                R[i][i] = rii;
#pragma unroll 1
                for (int j = i + 1; j < PM; ++j) {
                    if (j >= p) break;
                    double v = 0.5 * (G[i][j] + G[j][i]);
#pragma unroll 1
                    for (int k = 0; k < i; ++k) v -= R[k][i] * R[k][j];
                    R[i][j] = v / rii;
                }
            }
            return dmin;
        };
        if (mode == 0) {
            double gmax = 0.0;
            for (int i = 0; i < p; ++i) gmax = fmax(gmax, G[i][i]);
            // well conditioned (every pivot >= 1e-4 of the largest diagonal
            // entry, i.e. cond(W)^2 <= 1e4): plain Cholesky, and two passes
            // (CholQR2) orthonormalise to working precision.  Otherwise the
            // shifted first pass, and the step needs all three.
            bool plain = need3 != nullptr && gmax > 0.0;
            if (plain) plain = cholesky(0.0) >= 1e-4 * gmax;
            if (!plain) {
                cholesky(shift_rel * gmax);
                if (need3) atomicAdd(need3, 1);
            }
        } else {
            cholesky(0.0);
        }
        // accumulated factor Rt = R * Racc (upper triangular products)
#pragma unroll 1
        for (int a = 0; a < PM; ++a) {
            if (a >= p) break;
#pragma unroll 1
            for (int b = 0; b < PM; ++b) {
                if (b >= p) break;
                if (mode == 0 || p == 1) {
                    Rt[a][b] = R[a][b];
                } else {
                    double v = 0.0;
#pragma unroll 1
                    for (int k = a; k <= b; ++k) v += R[a][k] * sRa[k * p + b];
                    Rt[a][b] = v;
                }
            }
        }
        const bool final_pass = mode == 2;
        bool drop[PM];
#pragma unroll 1
        for (int i = 0; i < PM; ++i) drop[i] = i < p && R[i][i] == 0.0;
        if (final_check) {
#pragma unroll 1
            for (int i = 0; i < PM; ++i) {
                if (i >= p) break;
                double own = 0.0;
#pragma unroll 1
                for (int k = 0; k <= i; ++k) own += Rt[k][i] * Rt[k][i];
                if (!(fabs(Rt[i][i]) > kill_abs * sqrt(s_pre[i] + own))) drop[i] = true;
            }
        }
        // inverse of this pass's R on the kept directions
#pragma unroll 1
        for (int j = 0; j < PM; ++j) {
            if (j >= p) break;
            if (drop[j] && final_pass) continue;
            if (R[j][j] == 0.0) continue;
            Ri[j][j] = 1.0 / R[j][j];
#pragma unroll 1
            for (int i = j - 1; i >= 0; --i) {
                if (R[i][i] == 0.0) continue;
                double v = 0.0;
#pragma unroll 1
                for (int k = i + 1; k <= j; ++k) v += R[i][k] * Ri[k][j];
                Ri[i][j] = -v / R[i][i];
            }
        }
#pragma unroll 1
        for (int a = 0; a < PM; ++a) {
            if (a >= p) break;
#pragma unroll 1
            for (int b = 0; b < PM; ++b) {
                if (b >= p) break;
                Rinv[(size_t)s * p * p + a * p + b] = Ri[a][b];
                Ra[a * p + b] = (final_pass && drop[a]) ? 0.0 : Rt[a][b];
            }
        }
        if (!final_pass) return;
        if (Tm && jrow > 0) {
            double* Tw = Tm + (size_t)s * Tdim * Tdim;
#pragma unroll 1
            for (int a = 0; a < PM; ++a) {
                if (a >= p) break;
#pragma unroll 1
                for (int b = 0; b < PM; ++b) {
                    if (b >= p) break;
                    Tw[(size_t)((jrow - 1) * p + b) * Tdim + jrow * p + a] = drop[a] ? 0.0 : Rt[a][b];
                }
            }
            if (dead)
#pragma unroll 1
                for (int a = 0; a < PM; ++a)
                    if (a < p) dead[(size_t)s * Tdim + jrow * p + a] = drop[a] ? 1 : 0;
        }
    }
}

template <int PM>
__global__ void __launch_bounds__(QR_THREADS)
k_qr_finalize(int p, int nchunks, int ncols, const double* __restrict__ gpart, int mode,
              double shift_rel, double* __restrict__ Racc, double* __restrict__ Rinv,
              double* __restrict__ Tm, int Tdim, int jrow, double kill_abs,
              unsigned char* __restrict__ dead, int* __restrict__ need3) {
    // entries of G reduced per pass: the whole p x p block for p <= 4
    constexpr int NE = PM * PM < 16 ? PM * PM : 16;
    __shared__ double G[16][16];
    __shared__ double red[QR_THREADS / 32][16];
    __shared__ double red_pre[QR_THREADS / 32][PM];
    __shared__ double s_pre[16];
    __shared__ double s_ra[PM * PM];
    const int s = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // The kernel is a chain of dependent L2 round trips for one CTA per solve,
    // so every global load is issued up front: the skip flag, the chunk
    // partials of G, the coefficient rows of the final check and the
    // accumulated factor all go out before the first reduction waits on them.
    //
    // Final pass of a step whose blocks were all well conditioned: the middle
    // Gram pass was skipped and the block is already orthonormal (G = I).  The
    // partials are read either way (a live buffer; the values are then unused).
    const int n3 = (mode == 2 && need3) ? *need3 : 1;
    // accumulated factor of the earlier passes, read by the serial part
    if (mode != 0 && p > 1)
        for (int e = threadIdx.x; e < p * p; e += QR_THREADS) s_ra[e] = Racc[(size_t)s * p * p + e];
    // final pass: the squared norms of the new directions' coefficients in the
    // basis, sum_c T[col][c]^2 (col = (jrow - 1) p + i), summed by every thread
    const bool final_check = mode == 2 && Tm && jrow > 0;
    double pre[PM];
#pragma unroll
    for (int i = 0; i < PM; ++i) pre[i] = 0.0;
    if (final_check) {
        const double* Ts = Tm + (size_t)s * Tdim * Tdim + (size_t)(jrow - 1) * p * Tdim;
        for (int c = threadIdx.x; c < jrow * p; c += QR_THREADS)
#pragma unroll
            for (int i = 0; i < PM; ++i)
                if (i < p) {
                    const double t = Ts[(size_t)i * Tdim + c];
                    pre[i] += t * t;
                }
    }
    // G = sum of the chunk partials: every thread sums the chunks
    // tid, tid + QR_THREADS, ... of each entry (independent loads in flight),
    // then a fixed-order reduction over the lanes and the warps
    for (int e0 = 0; e0 < p * p; e0 += NE) {
        const int ne = min(NE, p * p - e0);
        double acc[NE];
        int off[NE];
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            acc[k] = 0.0;
            const int e = min(e0 + k, p * p - 1), a = e / p, b = e % p;
            off[k] = a * ncols + s * p + b;
        }
#pragma unroll 4
        for (int ch = threadIdx.x; ch < nchunks; ch += QR_THREADS) {
            const double* gp = gpart + (size_t)ch * p * ncols;
#pragma unroll
            for (int k = 0; k < NE; ++k)
                if (k < ne) acc[k] += gp[off[k]];
        }
#pragma unroll
        for (int k = 0; k < NE; ++k) {
            double v = acc[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) red[warp][k] = v;
        }
        if (e0 == 0 && final_check) {
#pragma unroll
            for (int i = 0; i < PM; ++i) {
                double v = pre[i];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == 0) red_pre[warp][i] = v;
            }
        }
        __syncthreads();
        if (threadIdx.x < ne) {
            const int e = e0 + threadIdx.x, a = e / p, b = e % p;
            double v = 0.0;
            for (int w = 0; w < QR_THREADS / 32; ++w) v += red[w][threadIdx.x];
            G[a][b] = n3 == 0 ? (a == b ? 1.0 : 0.0) : v;
        }
        if (e0 == 0 && final_check && threadIdx.x >= 32 && threadIdx.x < 32 + p) {
            const int i = threadIdx.x - 32;
            double v = 0.0;
            for (int w = 0; w < QR_THREADS / 32; ++w) v += red_pre[w][i];
            s_pre[i] = v;
        }
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    qr_factor<PM>(p, s, mode, shift_rel, G, s_pre, s_ra, final_check, Racc, Rinv, Tm, Tdim, jrow, kill_abs, dead, need3);
}

// V[r][s p + q'] = sum_{q <= q'} W[r][s p + q] Rinv_s[q][q']
template <class T>
__global__ void k_normalize(int64_t D, int ncols, int p, const double* __restrict__ Rinv,
                            const T* __restrict__ W, T* __restrict__ Vout) {
    const int64_t total = D * ncols;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / ncols;
        const int t = (int)(idx - r * ncols);
        const int s = t / p, q = t % p;
        const T* wr = W + r * ncols + s * p;
        const double* ri = Rinv + (size_t)s * p * p;
        T acc = T(0);
        for (int b = 0; b <= q; ++b) acc += wr[b] * (T)ri[b * p + q];
        Vout[idx] = acc;
    }
}

// CholQR passes without materialised intermediates: w = W[r][s P ..] times
// the nR upper-triangular factors Rinv_k (k < nR, slot k at Rinv + k rstride,
// solve s at s P P, entry [b][q] at b P + q), each applied in T exactly as a
// separate normalisation would; Vout (if not null) receives the result, and
// with do_gram the Gram partials of the result go to gpart in the k_update
// layout.  Four rows per iteration keep four loads in flight per thread.
template <class T, int P>
__global__ void __launch_bounds__(256)
k_normgram(int64_t D, int S, int nR, const double* __restrict__ Rinv, int64_t rstride,
           const T* __restrict__ W, T* __restrict__ Vout, int64_t rows_per_cta, int do_gram,
           double* __restrict__ gpart, const int* __restrict__ skip_if_zero, int* __restrict__ reset) {
    extern __shared__ double sG[];
    // a pass the step does not need (all blocks well conditioned) does nothing
    if (skip_if_zero && *skip_if_zero == 0) return;
    if (reset && blockIdx.x == 0 && threadIdx.x == 0) *reset = 0;
    constexpr int RU = 4;
    const int ncols = S * P;
    const int s = threadIdx.x % S, ro = threadIdx.x / S, R = blockDim.x / S;
    T rm[3][P][P];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int b = 0; b < P; ++b)
#pragma unroll
            for (int q = 0; q < P; ++q)
                rm[k][b][q] = k < nR ? (T)Rinv[(size_t)k * rstride + (size_t)s * P * P + b * P + q] : T(0);
    const int64_t r0 = (int64_t)blockIdx.x * rows_per_cta;
    const int64_t r1 = min(D, r0 + rows_per_cta);
    double gd[P][P];
    T gf[P][P];
#pragma unroll
    for (int q = 0; q < P; ++q)
#pragma unroll
        for (int b = 0; b < P; ++b) {
            gd[q][b] = 0.0;
            gf[q][b] = T(0);
        }
    int cnt = 0;
    for (int64_t base = r0 + ro; base < r1; base += RU * R) {
        Vec<T, P> w[RU];
#pragma unroll
        for (int u = 0; u < RU; ++u) {
            const int64_t r = base + (int64_t)u * R;
            if (r < r1) {
                w[u] = ldv<T, P>(W + r * ncols + s * P);
            } else {
#pragma unroll
                for (int q = 0; q < P; ++q) w[u].v[q] = T(0);
            }
        }
#pragma unroll
        for (int u = 0; u < RU; ++u) {
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                if (k < nR) {
                    Vec<T, P> o;
#pragma unroll
                    for (int q = P - 1; q >= 0; --q) {
                        T acc = T(0);
#pragma unroll
                        for (int b = 0; b <= q; ++b) acc += w[u].v[b] * rm[k][b][q];
                        o.v[q] = acc;
                    }
                    w[u] = o;
                }
            }
            const int64_t r = base + (int64_t)u * R;
            if (Vout && r < r1) stv<T, P>(Vout + r * ncols + s * P, w[u]);
            if (do_gram) {
#pragma unroll
                for (int q = 0; q < P; ++q)
#pragma unroll
                    for (int b = 0; b < P; ++b) gf[q][b] += w[u].v[q] * w[u].v[b];
            }
        }
        if (do_gram && ++cnt == 8) {  // FP64 flush every 32 rows
            cnt = 0;
#pragma unroll
            for (int q = 0; q < P; ++q)
#pragma unroll
                for (int b = 0; b < P; ++b) {
                    gd[q][b] += (double)gf[q][b];
                    gf[q][b] = T(0);
                }
        }
    }
    if (do_gram) {
#pragma unroll
        for (int q = 0; q < P; ++q)
#pragma unroll
            for (int b = 0; b < P; ++b) sG[(size_t)(q * P + b) * blockDim.x + threadIdx.x] = gd[q][b] + (double)gf[q][b];
        __syncthreads();
        for (int e = threadIdx.x; e < P * P * S; e += blockDim.x) {
            const int val = e / S, ss = e % S;
            const int q = val / P, b = val % P;
            double sum = 0.0;
            for (int u = 0; u < R; ++u) sum += sG[(size_t)val * blockDim.x + u * S + ss];
            gpart[((size_t)blockIdx.x * P + q) * ncols + ss * P + b] = sum;
        }
    }
}

// Packed FP32 pairs for the rotation's FMAs: one fma.rn.f32x2 performs two
// fused multiply-adds (each rounded to nearest, as the scalar form), halving
// the FMA instructions of an issue-bound loop.
__device__ __forceinline__ unsigned long long pack2(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void unpack2(unsigned long long v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ void fma2(unsigned long long& acc, unsigned long long x, unsigned long long y) {
    asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc) : "l"(x), "l"(y));
}

// Ritz rotation: for the processed solves ls < Sproc (input solve in_idx[ls],
// output slot out_idx[ls]):  out[:, i] = sum_{c < kc} V[:, c] Y_ls[c][i].
// Input column c of solve s is V_{c/p}[r][s p + c%p] (row stride ld_in).
// Output: blocks of p columns  Vout[i/p][r][o p + i%p]  (block stride
// ostride, row stride ld_out), or with single != 0 one row-major array
// Vout[r][o nout + i].
// A CTA takes Sg solves (their Y in shared memory, rows zero-padded to npad,
// a multiple of NO, and solves ystride apart so that the Sg rows read together
// fall in different banks) and a chunk of rows; thread = (solve ls = tid % Sg,
// RB rows rstep apart).  The Sg solves of one row are adjacent in memory (one
// sector for Sg p = 32 B / T), so a warp's loads cover whole sectors.  Each Y
// value read from shared memory feeds RB rows' FMAs (shared memory, not the
// FMA pipe, bounds a rotation with RB = 1).  NO outputs per row stay in
// registers; more outputs take further passes over the inputs.  PV = p for
// p in {1, 2, 4} (one vector load per basis block), else 0 (scalar loads).
template <class T, int NO, int PV, int RB>
__global__ void __launch_bounds__(128)
k_rotate(int64_t D, int Sproc, int ld_in, int p, int kc, int nout, int64_t bstride,
         const T* __restrict__ V, const T* __restrict__ Yg, const int* __restrict__ in_idx,
         const int* __restrict__ out_idx, T* __restrict__ Vout, int64_t ostride, int ld_out,
         int single, int Sg, int npad, int ystride, int64_t rows_per_chunk) {
    constexpr int V4 = 16 / sizeof(T);
    extern __shared__ __align__(16) unsigned char s_raw[];
    T* sY = reinterpret_cast<T*>(s_raw);
    const int sg0 = blockIdx.x * Sg;
    const int nsg = min(Sg, Sproc - sg0);
    for (int i = threadIdx.x; i < nsg * kc * npad; i += blockDim.x) {
        const int ls = i / (kc * npad), e = i - ls * (kc * npad);
        const int c = e / npad, o = e - c * npad;
        sY[(size_t)ls * ystride + e] = o < nout ? Yg[((size_t)(sg0 + ls) * kc + c) * nout + o] : T(0);
    }
    __syncthreads();
    const int ls = threadIdx.x % Sg;
    if (ls >= nsg) return;
    const int rstep = blockDim.x / Sg;
    const int sin = in_idx[sg0 + ls], sout = out_idx[sg0 + ls];
    const int nblk = kc / p;
    const int64_t r0 = (int64_t)blockIdx.y * rows_per_chunk;
    const int64_t r1 = min(D, r0 + rows_per_chunk);
    const T* ys = sY + (size_t)ls * ystride;
    for (int64_t base = r0 + threadIdx.x / Sg; base < r1; base += (int64_t)RB * rstep) {
        const T* vr[RB];
        bool ok[RB];
#pragma unroll
        for (int k = 0; k < RB; ++k) {
            const int64_t r = base + (int64_t)k * rstep;
            ok[k] = r < r1;
            vr[k] = V + (ok[k] ? r : base) * ld_in + (int64_t)sin * p;  // invalid rows read row base
        }
        for (int o0 = 0; o0 < nout; o0 += NO) {
            T acc[RB][NO];
#pragma unroll
            for (int k = 0; k < RB; ++k)
#pragma unroll
                for (int u = 0; u < NO; ++u) acc[k][u] = T(0);
            if constexpr (PV >= 1 && std::is_same<T, float>::value && NO % 4 == 0) {
                // FP32: accumulators as packed pairs, two outputs per FMA instruction
                unsigned long long acc2[RB][NO / 2];
#pragma unroll
                for (int k = 0; k < RB; ++k)
#pragma unroll
                    for (int u = 0; u < NO / 2; ++u) acc2[k][u] = 0ull;
                constexpr int UJ = PV == 1 ? 4 : 2;
                // PF: the next UJ blocks' values are requested before this
                // group's products (one group of loads always in flight), where
                // the extra registers keep three CTAs per SM
                constexpr bool PF = PV * UJ * RB <= 8;
                Vec<T, PV> xn[PF ? UJ : 1][RB];
                if constexpr (PF) {
#pragma unroll
                    for (int u = 0; u < UJ; ++u)
#pragma unroll
                        for (int k = 0; k < RB; ++k)
                            if (u < nblk) xn[u][k] = ldv<T, PV>(vr[k] + (int64_t)u * bstride);
                }
                for (int j = 0; j < nblk; j += UJ) {
                    Vec<T, PV> x[UJ][RB];
                    if constexpr (PF) {
#pragma unroll
                        for (int u = 0; u < UJ; ++u)
#pragma unroll
                            for (int k = 0; k < RB; ++k) x[u][k] = xn[u][k];
#pragma unroll
                        for (int u = 0; u < UJ; ++u)
#pragma unroll
                            for (int k = 0; k < RB; ++k)
                                if (j + UJ + u < nblk)
                                    xn[u][k] = ldv<T, PV>(vr[k] + (int64_t)(j + UJ + u) * bstride);
                    } else {
#pragma unroll
                        for (int u = 0; u < UJ; ++u)
#pragma unroll
                            for (int k = 0; k < RB; ++k)
                                if (j + u < nblk) x[u][k] = ldv<T, PV>(vr[k] + (int64_t)(j + u) * bstride);
                    }
#pragma unroll
                    for (int u = 0; u < UJ; ++u) {
                        if (j + u < nblk) {
#pragma unroll
                            for (int q = 0; q < PV; ++q) {
                                const T* yc = ys + (size_t)((j + u) * PV + q) * npad + o0;
                                unsigned long long xx[RB];
#pragma unroll
                                for (int k = 0; k < RB; ++k) xx[k] = pack2(x[u][k].v[q], x[u][k].v[q]);
#pragma unroll
                                for (int o = 0; o < NO; o += 4) {
                                    const Vec<T, 4> y = ldv<T, 4>(yc + o);
                                    const unsigned long long y01 = pack2(y.v[0], y.v[1]);
                                    const unsigned long long y23 = pack2(y.v[2], y.v[3]);
#pragma unroll
                                    for (int k = 0; k < RB; ++k) {
                                        fma2(acc2[k][o / 2], xx[k], y01);
                                        fma2(acc2[k][o / 2 + 1], xx[k], y23);
                                    }
                                }
                            }
                        }
                    }
                }
#pragma unroll
                for (int k = 0; k < RB; ++k)
#pragma unroll
                    for (int u = 0; u < NO / 2; ++u) {
                        float lo, hi;
                        unpack2(acc2[k][u], lo, hi);
                        acc[k][2 * u] = lo;
                        acc[k][2 * u + 1] = hi;
                    }
            } else if constexpr (PV >= 1) {
                constexpr int UJ = PV == 1 ? 4 : 2;
                for (int j = 0; j < nblk; j += UJ) {
                    Vec<T, PV> x[UJ][RB];
#pragma unroll
                    for (int u = 0; u < UJ; ++u)
#pragma unroll
                        for (int k = 0; k < RB; ++k)
                            if (j + u < nblk) x[u][k] = ldv<T, PV>(vr[k] + (int64_t)(j + u) * bstride);
#pragma unroll
                    for (int u = 0; u < UJ; ++u) {
                        if (j + u < nblk) {
#pragma unroll
                            for (int q = 0; q < PV; ++q) {
                                const T* yc = ys + (size_t)((j + u) * PV + q) * npad + o0;
#pragma unroll
                                for (int o = 0; o < NO; o += V4) {
                                    const Vec<T, V4> y = ldv<T, V4>(yc + o);
#pragma unroll
                                    for (int k = 0; k < RB; ++k)
#pragma unroll
                                        for (int w = 0; w < V4; ++w) acc[k][o + w] += x[u][k].v[q] * y.v[w];
                                }
                            }
                        }
                    }
                }
            } else {
                for (int c = 0; c < kc; ++c) {
                    T x[RB];
#pragma unroll
                    for (int k = 0; k < RB; ++k) x[k] = vr[k][(int64_t)(c / p) * bstride + c % p];
                    const T* yc = ys + (size_t)c * npad + o0;
#pragma unroll
                    for (int o = 0; o < NO; o += V4) {
                        const Vec<T, V4> y = ldv<T, V4>(yc + o);
#pragma unroll
                        for (int k = 0; k < RB; ++k)
#pragma unroll
                            for (int w = 0; w < V4; ++w) acc[k][o + w] += x[k] * y.v[w];
                    }
                }
            }
            const int no = min(NO, nout - o0);
#pragma unroll
            for (int k = 0; k < RB; ++k) {
                if (!ok[k]) continue;
                const int64_t r = base + (int64_t)k * rstep;
                if (single) {
                    T* dst = Vout + r * ld_out + (int64_t)sout * nout + o0;
#pragma unroll
                    for (int u = 0; u < NO; ++u)
                        if (u < no) dst[u] = acc[k][u];
                } else {
#pragma unroll
                    for (int u = 0; u < NO; ++u) {
                        if (u < no) {
                            const int i = o0 + u;
                            Vout[(int64_t)(i / p) * ostride + r * ld_out + (int64_t)sout * p + i % p] = acc[k][u];
                        }
                    }
                }
            }
        }
    }
}

// Vout[r][a p + q] = Vin[r][in_idx[a] p + q]  (compaction of one block)
template <class T>
__global__ void k_gather_block(int64_t D, int Snew, int p, int ld_in, int ld_out,
                               const int* __restrict__ in_idx, const T* __restrict__ Vin,
                               T* __restrict__ Vout) {
    const int64_t total = D * ld_out;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / ld_out;
        const int t = (int)(idx - r * ld_out);
        const int a = t / p, q = t % p;
        Vout[idx] = Vin[r * ld_in + in_idx[a] * p + q];
    }
}

// Spectra's SimpleRandom stream (Park-Miller, x <- 16807 x mod 2^31-1, seed 0
// mapped to 1), value x / (2^31 - 1) - 0.5.  Column q of the start block takes
// stream positions [q D, (q+1) D); row r takes position perm[r] (the index of
// row r in the caller's order).
__device__ __forceinline__ uint64_t mulmod31(uint64_t a, uint64_t b) { return (a * b) % 2147483647ull; }

template <class T>
__global__ void k_start_block(int64_t D, int ncols, int p, uint64_t seed,
                              const int32_t* __restrict__ perm, T* __restrict__ W) {
    const uint64_t M = 2147483647ull;
    const uint64_t s0 = seed ? (seed & M) : 1ull;
    const int64_t total = D * ncols;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / ncols;
        const int t = (int)(idx - r * ncols);
        const int q = t % p;
        const uint64_t pos = (uint64_t)q * (uint64_t)D + (uint64_t)(perm ? perm[r] : r);
        uint64_t e = pos + 1, base = 16807ull, acc = 1ull;
        while (e) {
            if (e & 1ull) acc = mulmod31(acc, base);
            base = mulmod31(base, base);
            e >>= 1;
        }
        const uint64_t x = mulmod31(s0 % M, acc);
        W[idx] = (T)((double)x / (double)M - 0.5);
    }
}

template <class A, class B>
__global__ void k_convert(int64_t n, const A* __restrict__ in, B* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (B)in[i];
}

// Combination of Ritz-type columns (FP64), column t = s K + i of a group:
//   v = sum_a (Y1 - theta_t X1)[r][s K + a] Z1_s[a][i] + sum_a (Y2 - theta_t X2)[r][s K + a] Z2_s[a][i]
// (X1, X2 may be null: no theta term; Y2 null: no second sum), written to
// out[r][t] (if not null) and/or summed as |v|^2 over a chunk of rows into
// part[chunk][t] (if not null).  Z_s[a][i] at Z + (s K + a) K + i.
__global__ void __launch_bounds__(512)
k_ritz_mix(int64_t D, int ncols, int ld, int K, const double* __restrict__ Y1, const double* __restrict__ X1,
           const double* __restrict__ Z1, const double* __restrict__ Y2, const double* __restrict__ X2,
           const double* __restrict__ Z2, const double* __restrict__ theta, double* __restrict__ out,
           int64_t rows_per_chunk, double* __restrict__ part) {
    extern __shared__ double s_red2[];
    const int t = threadIdx.x % ncols, ro = threadIdx.x / ncols, R = blockDim.x / ncols;
    const int s = t / K, i = t % K;
    const double th = theta ? theta[t] : 0.0;
    const double* z1 = Z1 + (size_t)s * K * K;
    const double* z2 = Z2 ? Z2 + (size_t)s * K * K : nullptr;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t r1 = min(D, r0 + rows_per_chunk);
    double acc = 0.0;
    for (int64_t r = r0 + ro; r < r1; r += R) {
        const size_t base = (size_t)r * ld + (size_t)s * K;
        double v = 0.0;
        for (int a = 0; a < K; ++a) {
            const double y = Y1[base + a];
            v += (X1 ? y - th * X1[base + a] : y) * __ldg(z1 + a * K + i);
        }
        if (Y2)
            for (int a = 0; a < K; ++a) {
                const double y = Y2[base + a];
                v += (X2 ? y - th * X2[base + a] : y) * __ldg(z2 + a * K + i);
            }
        if (out) out[(size_t)r * ld + t] = v;
        acc += v * v;
    }
    if (!part) return;
    s_red2[threadIdx.x] = acc;
    __syncthreads();
    if (ro == 0) {
        double sum = 0.0;
        for (int u = 0; u < R; ++u) sum += s_red2[u * ncols + t];
        part[(size_t)blockIdx.x * ncols + t] = sum;
    }
}

__global__ void k_sum_cols(int nchunks, int ncols, const double* __restrict__ part,
                           double* __restrict__ out) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ncols; t += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int ch = 0; ch < nchunks; ++ch) s += part[(size_t)ch * ncols + t];
        out[t] = s;
    }
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------

// Device attributes, looked up once per device ordinal.  The sectors of a
// multi-sector call query them from several host threads at once, so each
// cached value is an atomic (0 = not looked up yet; a racing lookup stores the
// same value).
static int device_attr_cached(std::atomic<int>* cache, cudaDeviceAttr attr, int fallback) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return fallback;
    if (dev < 0 || dev >= kMaxDevices) return fallback;
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v > 0) return v;
    if (cudaDeviceGetAttribute(&v, attr, dev) != cudaSuccess || v <= 0) return fallback;
    cache[dev].store(v, std::memory_order_relaxed);
    return v;
}

static std::atomic<int> g_sm_count[kMaxDevices];
static std::atomic<int> g_smem_optin[kMaxDevices];

int sm_count() { return device_attr_cached(g_sm_count, cudaDevAttrMultiProcessorCount, 132); }

static int max_smem_optin() {
    return device_attr_cached(g_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, 48 * 1024);
}

// BH_VERBOSE=1 in the environment prints one line per restart to stderr.
static bool verbose() {
    static int v = -1;
    if (v < 0) {
        const char* e = std::getenv("BH_VERBOSE");
        v = (e && *e && *e != '0') ? 1 : 0;
    }
    return v == 1;
}

// BH_DEBUG_ORTHO=1 additionally measures the orthogonality of the Krylov basis
// of the first active solve at every restart (diagnostic; costs one Gram pass).
// BH_NO_GRAPHS=1: launch every kernel of a restart cycle directly instead of
// replaying the captured cycle (for comparing the two)
static bool use_graphs() {
    static int v = -1;
    if (v < 0) {
        const char* e = std::getenv("BH_NO_GRAPHS");
        v = (e && *e && *e != '0') ? 0 : 1;
    }
    return v == 1;
}

// BH_SEPARATE_LOCAL_DOT=1: compute the local coefficient with its own
// reduction kernel instead of inside the SpMM (for comparing the two paths)
static bool separate_local_dot() {
    static int v = -1;
    if (v < 0) {
        const char* e = std::getenv("BH_SEPARATE_LOCAL_DOT");
        v = (e && *e && *e != '0') ? 1 : 0;
    }
    return v == 1;
}

// BH_RITZ_MARGIN=k: Ritz vectors refined in FP64 beyond the wanted ones
// (rounded up to whole blocks; default 0); BH_RITZ_STAGE2=0/1: the
// residual-augmented second Rayleigh-Ritz of the mixed-precision refinement
// (default 0); BH_KEEP_FRACTION=f: a thick restart keeps nev + f (ncv - nev)
// Ritz vectors (default 0.4: on the m=10 multi-sector grid 0.4 took 30
// restarts where 0.5 took 45, 6.6% more eigensolves/s; 0.3 and 0.6 were worse
// in speed or accuracy)
static int ritz_margin() {
    static int v = -1;
    if (v < 0) {
        const char* e = std::getenv("BH_RITZ_MARGIN");
        v = (e && *e) ? std::max(0, std::atoi(e)) : 0;
    }
    return v;
}

static bool ritz_stage2() {
    static int v = -1;
    if (v < 0) {
        const char* e = std::getenv("BH_RITZ_STAGE2");
        v = (e && *e && *e != '0') ? 1 : 0;
    }
    return v == 1;
}

static double keep_fraction() {
    static double v = -1.0;
    if (v < 0.0) {
        const char* e = std::getenv("BH_KEEP_FRACTION");
        const double f = (e && *e) ? std::atof(e) : 0.4;
        v = (f > 0.0 && f < 1.0) ? f : 0.4;
    }
    return v;
}

// BH_TC_ROTATE=1: the restart rotation of the FP32 basis on the tensor cores
// (bh_rotate_tc.cu) instead of the SIMT kernel.  Off by default: measured on
// the m=10, n=10 sector (64 solves, block 2) it took 108.5 ms over 47
// rotations against 23.0 ms for the SIMT kernel -- the exact three-piece TF32
// split of every basis value costs as many instructions per value as the SIMT
// kernel's FMAs, and one 132 KB CTA per SM leaves 4 warps to hide the loads
// (ncu: tensor pipe 2.3% active, warps active 6.3%).
static bool tc_rotation_on() {
    static int v = -1;
    if (v < 0) {
        const char* e = std::getenv("BH_TC_ROTATE");
        v = (e && *e == '1') ? 1 : 0;
    }
    return v == 1;
}

// The restart rotation of a batch whose solves all continue runs on the
// tensor cores, streamed by TMA (bh_rotate_tma.cu), with the split basis
// operand in tensor memory, for blocks of 1 and 2; BH_TMA_ROTATE=2 (or 1,
// the operand in shared memory) selects it for every block size,
// BH_TMA_ROTATE=0 keeps the SIMT kernel.  Measured on the m=10 multi-sector
// grid (64 J x 5 sectors, block 2): 261.7 eigensolves/s against 259.3 (1) and
// 253.3 (SIMT), the same eigenvalues within 4.95e-9 of FP64 (4.60e-9 SIMT),
// its rotations at 2.4-3.0 TB/s against 1.2-1.6 TB/s, and the same restart
// counts.  On the 4x4 torus (block 4, four-fold levels) its rounding
// (2^-22 per term, FP32 2^-24) took 65 restarts where SIMT took 60, so block 4
// keeps the SIMT rotation by default.
static int tma_rotation_mode() {
    static int v = -2;
    if (v == -2) {
        const char* e = std::getenv("BH_TMA_ROTATE");
        v = (e && (*e == '0' || *e == '1' || *e == '2')) ? *e - '0' : -1;  // -1: the default
    }
    return v;
}
static bool tma_rotation_on(int p) {
    const int m = tma_rotation_mode();
    return m > 0 || (m < 0 && p <= 2);
}

static bool debug_ortho() {
    static int v = -1;
    if (v < 0) {
        const char* e = std::getenv("BH_DEBUG_ORTHO");
        v = (e && *e && *e != '0') ? 1 : 0;
    }
    return v == 1;
}

static int ilog2(int p) {
    int l = 0;
    while ((1 << l) < p) ++l;
    return l;
}

template <class F>
static void parallel_for(int n, F&& f) {
    int hw = (int)std::thread::hardware_concurrency();
    int nt = std::min(n, std::max(1, std::min(hw, 16)));
    if (nt <= 1 || n < 4) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    std::vector<std::thread> th;
    for (int k = 0; k < nt; ++k)
        th.emplace_back([&, k] {
            for (int i = k; i < n; i += nt) f(i);
        });
    for (auto& t : th) t.join();
}

// geometry of the row-chunked reductions (k_dot, k_ritz_mix): at most 2 chunks per SM
struct Geo {
    int ncols = 0, R = 1, NT = 0;
    int64_t rows_per_chunk = 0;
    int nchunks = 0;
};

static Geo make_geo(int64_t D, int ncols) {
    Geo g;
    g.ncols = ncols;
    g.R = std::max(1, 256 / ncols);
    g.NT = ncols * g.R;
    const int64_t target = 2LL * sm_count();
    int64_t rpc = (D + target - 1) / target;
    rpc = std::max<int64_t>(rpc, (int64_t)g.R * 16);
    g.rows_per_chunk = rpc;
    g.nchunks = (int)((D + rpc - 1) / rpc);
    if (g.nchunks < 1) g.nchunks = 1;
    return g;
}

// geometry of k_update / k_normgram / k_qr_finalize: about 4 CTAs per SM
static Geo make_ugeo(int64_t D, int ncols) {
    Geo g;
    g.ncols = ncols;
    g.R = std::max(1, 256 / ncols);
    g.NT = ncols * g.R;
    const int64_t target = 4LL * sm_count();
    int64_t rpc = (D + target - 1) / target;
    rpc = std::max<int64_t>(rpc, (int64_t)g.R * 16);
    rpc = (rpc + 2 * g.R - 1) / (2 * g.R) * (2 * g.R);
    g.rows_per_chunk = rpc;
    g.nchunks = (int)((D + rpc - 1) / rpc);
    if (g.nchunks < 1) g.nchunks = 1;
    return g;
}

static unsigned elem_grid(int64_t n, int threads = 256) {
    int64_t g = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count() * 8;
    return (unsigned)std::max<int64_t>(1, std::min(g, cap));
}

template <class T>
struct Launcher {
    const OpView<T>& op;
    cudaStream_t st;
    int64_t* launches;
    int* tc_status = nullptr;  // error flag of the tensor-core rotation (device)

    void profile_begin_() const { profile_begin(st); }
    void done(const char* name, double bytes) const {
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) throw Error(BH_ERR_CUDA, std::string("launch of ") + name + ": " + cudaGetErrorString(e));
        ++*launches;
        profile_end(st, name, bytes);
    }

    void spmm(int ncols, int group, const double* prm, const T* X, T* Y, double* dpart = nullptr,
              int* dparts = nullptr) const {
        // launch shape of this operator and width class, timed at first use
        // (nothing happens when the table has it, the product fuses, or the
        // stream is being captured)
        *launches += tune_spmm<T>(op, ncols, group, prm, X, Y, st, dpart != nullptr);
        profile_begin(st);
        const double bytes = launch_spmm<T>(op, ncols, group, prm, X, Y, st, dpart, dparts);
        done(op.occ ? "k_spmm_mf" : "k_spmm", bytes);
    }

    template <int PMAX>
    void dot_t(const Geo& g, int ld, int p, int nblk, int64_t bstride, const T* V, const T* W, int kcap,
               double* part) const {
        constexpr int JT = PMAX >= 16 ? 1 : 16 / PMAX;
        dim3 grid(g.nchunks, (nblk + JT - 1) / JT);
        const size_t smem = (size_t)g.NT * JT * PMAX * sizeof(double);
        auto kern = k_dot<T, PMAX, JT>;
        allow_large_smem(kern, smem);
        profile_begin(st);
        kern<<<grid, g.NT, smem, st>>>(op.D, g.ncols, ld, p, nblk, bstride, V, W, g.rows_per_chunk, kcap, part);
        done(nblk == 1 ? "k_dot(1 block)" : "k_dot", (double)(nblk + 1) * op.D * g.ncols * sizeof(T));
    }
    // per-solve vector path: P = p in {1, 2, 4}, packed rows, aligned P-vectors
    bool vec_ok(int ld, int ncols, int p, int64_t bstride, const void* A, const void* B) const {
        if (!(p == 1 || p == 2 || p == 4) || ld != ncols || ncols / p > 256) return false;
        const uintptr_t al = (uintptr_t)p * sizeof(T);
        return bstride % p == 0 && ((uintptr_t)A % al) == 0 && ((uintptr_t)B % al) == 0;  // null passes
    }
    template <int P, int JT, int RU>
    void dotv_t(const Geo& g, int nblk, int64_t bstride, const T* V, const T* W, int kcap,
                double* part) const {
        const int S = g.ncols / P;
        const int NT = S * std::max(1, 128 / S);  // small CTAs: several resident per SM
        BH_REQUIRE(g.nchunks <= 65535, "too many row chunks for the reduction grid");
        dim3 grid((nblk + JT - 1) / JT, g.nchunks);
        const size_t smem = (size_t)NT * JT * P * P * sizeof(double);
        auto kern = k_dotv<T, P, JT, RU>;
        allow_large_smem(kern, smem);
        profile_begin(st);
        kern<<<grid, NT, smem, st>>>(op.D, S, nblk, bstride, V, W, g.rows_per_chunk, kcap, part);
        done(nblk == 1 ? "k_dot(1 block)" : "k_dot", (double)(nblk + 1) * op.D * g.ncols * sizeof(T));
    }
    void dot(const Geo& g, int ld, int p, int nblk, int64_t bstride, const T* V, const T* W,
             int kcap, double* part) const {
        if (vec_ok(ld, g.ncols, p, bstride, V, W)) {
            // (JT blocks, RU rows) per step: 1 block and 4 rows for the local
            // step, else 4 blocks (2 for P = 4) and 2 rows
            if (p == 1) {
                if (nblk == 1) dotv_t<1, 1, 4>(g, nblk, bstride, V, W, kcap, part);
                else dotv_t<1, 8, 2>(g, nblk, bstride, V, W, kcap, part);
            } else if (p == 2) {
                if (nblk == 1) dotv_t<2, 1, 4>(g, nblk, bstride, V, W, kcap, part);
                else dotv_t<2, 2, 4>(g, nblk, bstride, V, W, kcap, part);
            } else {
                if (nblk == 1) dotv_t<4, 1, 2>(g, nblk, bstride, V, W, kcap, part);
                else dotv_t<4, 2, 2>(g, nblk, bstride, V, W, kcap, part);
            }
            return;
        }
        if (p <= 1) dot_t<1>(g, ld, p, nblk, bstride, V, W, kcap, part);
        else if (p <= 2) dot_t<2>(g, ld, p, nblk, bstride, V, W, kcap, part);
        else if (p <= 4) dot_t<4>(g, ld, p, nblk, bstride, V, W, kcap, part);
        else if (p <= 8) dot_t<8>(g, ld, p, nblk, bstride, V, W, kcap, part);
        else if (p <= 16) dot_t<16>(g, ld, p, nblk, bstride, V, W, kcap, part);
        else dot_t<32>(g, ld, p, nblk, bstride, V, W, kcap, part);
    }
    void dot_finalize(const Geo& g, int kc, int ldC, int p, int kcap, const double* part, double* C,
                      T* Cf, double* Tm, int Tdim, int jcol) const {
        profile_begin(st);
        k_dot_finalize<T><<<elem_grid((int64_t)kc * g.ncols * 32), 256, 0, st>>>(
            g.nchunks, kc, g.ncols, ldC, p, kcap, part, C, Cf, Tm, Tdim, jcol);
        done("k_dot_finalize", (double)g.nchunks * kc * g.ncols * 8.0);
    }
    void local_coef(const Geo& g, int j, int c_lo, int p, int kcap, const double* part, double* Tm,
                    int Tdim, T* Cf) const {
        const int64_t total = (int64_t)((j + 1) * p - c_lo) * g.ncols;
        profile_begin(st);
        k_local_coef<T><<<elem_grid(total * 32), 256, 0, st>>>(g.nchunks, j, c_lo, g.ncols, p, kcap, part,
                                                          Tm, Tdim, Cf);
        done("k_local_coef", (double)g.nchunks * p * g.ncols * 8.0);
    }
    template <int PMAX>
    void update_t(const Geo& g, int p, int kc, int64_t bstride, const T* V, const T* Cf, T* W,
                  int do_gram, double* gpart, const char* name) const {
        const size_t smem = (((size_t)kc * g.ncols * sizeof(T) + 15) & ~(size_t)15) +
                            (size_t)g.NT * PMAX * sizeof(double);
        if ((int)smem > max_smem_optin()) throw Error(BH_ERR_ARG, "Krylov basis too wide for shared memory (reduce ncv or batch)");
        auto kern = k_update<T, PMAX>;
        allow_large_smem(kern, smem);
        profile_begin(st);
        kern<<<g.nchunks, g.NT, smem, st>>>(op.D, g.ncols, p, ilog2(p), kc, bstride, V, Cf, W,
                                            g.rows_per_chunk, do_gram, gpart);
        done(name ? name : (kc > 0 ? "k_update" : "k_update(gram)"),
             (double)(kc > 0 ? kc / p + 2 : 1) * op.D * g.ncols * sizeof(T));
    }
    template <int P>
    void updatev_t(const Geo& g, int kc, int64_t bstride, const T* V, const T* Cf, T* W, int do_gram,
                   double* gpart, const char* name) const {
        const int S = g.ncols / P;
        const int NT = S * std::max(1, 256 / S);
        const size_t smem = (((size_t)kc * g.ncols * sizeof(T) + 15) & ~(size_t)15) +
                            (size_t)NT * P * P * sizeof(double);
        if ((int)smem > max_smem_optin()) throw Error(BH_ERR_ARG, "Krylov basis too wide for shared memory (reduce ncv or batch)");
        auto kern = k_updatev<T, P>;
        allow_large_smem(kern, smem);
        profile_begin(st);
        kern<<<g.nchunks, NT, smem, st>>>(op.D, S, kc / P, bstride, V, Cf, W, g.rows_per_chunk, do_gram, gpart);
        done(name ? name : (kc > 0 ? "k_update" : "k_update(gram)"),
             (double)(kc > 0 ? kc / P + 2 : 1) * op.D * g.ncols * sizeof(T));
    }
    void update(const Geo& g, int p, int kc, int64_t bstride, const T* V, const T* Cf, T* W,
                int do_gram, double* gpart, const char* name = nullptr) const {
        if (kc % std::max(p, 1) == 0 && vec_ok(g.ncols, g.ncols, p, kc > 0 ? bstride : 0, kc > 0 ? V : W, W)) {
            if (p == 1) updatev_t<1>(g, kc, bstride, V, Cf, W, do_gram, gpart, name);
            else if (p == 2) updatev_t<2>(g, kc, bstride, V, Cf, W, do_gram, gpart, name);
            else updatev_t<4>(g, kc, bstride, V, Cf, W, do_gram, gpart, name);
            return;
        }
        if (p <= 1) update_t<1>(g, p, kc, bstride, V, Cf, W, do_gram, gpart, name);
        else if (p <= 2) update_t<2>(g, p, kc, bstride, V, Cf, W, do_gram, gpart, name);
        else if (p <= 4) update_t<4>(g, p, kc, bstride, V, Cf, W, do_gram, gpart, name);
        else if (p <= 8) update_t<8>(g, p, kc, bstride, V, Cf, W, do_gram, gpart, name);
        else update_t<16>(g, p, kc, bstride, V, Cf, W, do_gram, gpart, name);
    }
    void qr(const Geo& gu, int S, int p, const double* gpart, int mode, double shift_rel,
            double* Racc, double* Rinv, double* Tm, int Tdim, int jrow, double kill_abs,
            unsigned char* dead, int* need3 = nullptr) const {
        profile_begin(st);
        auto go = [&](auto kern) {
            kern<<<S, QR_THREADS, 0, st>>>(p, gu.nchunks, gu.ncols, gpart, mode, shift_rel, Racc, Rinv, Tm, Tdim,
                                          jrow, kill_abs, dead, need3);
        };
        if (p <= 1) go(k_qr_finalize<1>);
        else if (p <= 2) go(k_qr_finalize<2>);
        else if (p <= 4) go(k_qr_finalize<4>);
        else if (p <= 8) go(k_qr_finalize<8>);
        else go(k_qr_finalize<16>);
        done("k_qr_finalize", (double)gu.nchunks * p * gu.ncols * 8.0);
    }
    template <int P>
    void normgram_t(const Geo& g, int nR, const double* Rinv, int64_t rstride, const T* W, T* Vout,
                    int do_gram, double* gpart, const int* skip_if_zero, int* reset) const {
        const int S = g.ncols / P;
        const int NT = S * std::max(1, 256 / S);
        const size_t smem = do_gram ? (size_t)NT * P * P * sizeof(double) : 0;
        auto kern = k_normgram<T, P>;
        allow_large_smem(kern, smem);
        profile_begin(st);
        kern<<<g.nchunks, NT, smem, st>>>(op.D, S, nR, Rinv, rstride, W, Vout, g.rows_per_chunk, do_gram, gpart,
                                          skip_if_zero, reset);
        done(Vout ? "k_normalize" : "k_gram", (double)op.D * g.ncols * sizeof(T) * (Vout ? 2.0 : 1.0));
    }
    // nR factors applied to W; result to Vout (optional) and/or its Gram partials
    // skip_if_zero: the pass does nothing when *skip_if_zero == 0; reset: set to 0 by the pass
    void normgram(const Geo& g, int p, int nR, const double* Rinv, int64_t rstride, const T* W, T* Vout,
                  int do_gram, double* gpart, const int* skip_if_zero = nullptr, int* reset = nullptr) const {
        if (p == 1) normgram_t<1>(g, nR, Rinv, rstride, W, Vout, do_gram, gpart, skip_if_zero, reset);
        else if (p == 2) normgram_t<2>(g, nR, Rinv, rstride, W, Vout, do_gram, gpart, skip_if_zero, reset);
        else normgram_t<4>(g, nR, Rinv, rstride, W, Vout, do_gram, gpart, skip_if_zero, reset);
    }
    void normalize(int ncols, int p, const double* Rinv, const T* W, T* Vout) const {
        profile_begin(st);
        k_normalize<T><<<elem_grid(op.D * ncols), 256, 0, st>>>(op.D, ncols, p, Rinv, W, Vout);
        done("k_normalize", 2.0 * op.D * ncols * sizeof(T));
    }
    // rotation of Sproc solves (see k_rotate); Yg is Sproc x kc x nout
    // contiguous: the processed solves are 0 .. Sproc - 1 in and out (no solve
    // retired at this restart)
    void rotate(int Sproc, int ld_in, int p, int kc, int nout, int64_t bstride, const T* V,
                const T* Yg, const int* in_idx, const int* out_idx, T* Vout, int64_t ostride,
                int ld_out, int single, bool contiguous = false) const {
        if (Sproc <= 0) return;
        if constexpr (std::is_same<T, float>::value) {
            if (contiguous && !single && tma_rotation_on(p)) {
                profile_begin(st);
                if (rotate_tma(op.D, Sproc, ld_in, p, kc, nout, bstride, V, Yg, Vout, ostride, ld_out, tc_status,
                               st, tma_rotation_mode() != 1)) {
                    done("k_rotate_tma", (double)op.D * Sproc * p * ((double)kc / p + (double)nout / p) * sizeof(T));
                    return;
                }
            }
            // FP32 basis: the tensor-core rotation (bh_rotate_tc.cu) where its
            // shapes allow, else the SIMT kernel below
            if (tc_rotation_on()) {
                profile_begin(st);
                if (rotate_tc(op.D, Sproc, ld_in, p, kc, nout, bstride, V, Yg, in_idx, out_idx, Vout, ostride,
                              ld_out, single, tc_status, st)) {
                    done("k_rotate_tc", (double)op.D * Sproc * p * ((double)kc / p + (double)nout / p) * sizeof(T));
                    return;
                }
            }
        }
        constexpr int V4 = 16 / sizeof(T), E = 128 / sizeof(T);
        // outputs per pass (a template value below); Y rows padded to a whole
        // number of passes so that every pass reads inside its row
        const int NO = sizeof(T) == 4 ? (nout <= 16 ? 16 : (nout <= 24 ? 24 : (nout <= 40 ? 40 : 48)))
                                      : (nout <= 8 ? 8 : 16);
        const int npad = (nout + NO - 1) / NO * NO;
        const int ystride = ((kc * npad + E - 1) / E) * E + V4;
        const size_t per = (size_t)ystride * sizeof(T);
        const int smax = std::min(max_smem_optin(), 200 * 1024);
        if ((int)per > smax) throw Error(BH_ERR_ARG, "restart rotation too large for shared memory (reduce ncv)");
        // Sg solves per CTA: one 32-byte sector per row when p and shared memory allow
        int Sg = std::max(1, std::min(8, (int)(32 / ((size_t)p * sizeof(T)))));
        Sg = std::min(Sg, std::max(1, (int)((size_t)smax / per)));
        Sg = std::min(Sg, Sproc);
        while (Sg > 1 && 128 % Sg != 0) --Sg;
        const size_t smem = (size_t)Sg * per;
        const int ngroups = (Sproc + Sg - 1) / Sg;
        const int rstep = 128 / Sg;
        int64_t chunks = std::max<int64_t>(1, (6LL * sm_count() + ngroups - 1) / ngroups);
        int64_t rpc = (op.D + chunks - 1) / chunks;
        rpc = std::max<int64_t>(rpc, 4LL * rstep);
        chunks = (op.D + rpc - 1) / rpc;
        BH_REQUIRE(chunks <= 65535, "too many row chunks for the rotation grid");
        const bool vec = (p == 1 || p == 2 || p == 4) && ld_in % p == 0 && bstride % p == 0 &&
                         ((uintptr_t)V % ((uintptr_t)p * sizeof(T))) == 0;
        auto launch = [&](auto kern) {
            allow_large_smem(kern, smem);
            kern<<<dim3((unsigned)ngroups, (unsigned)chunks), 128, smem, st>>>(
                op.D, Sproc, ld_in, p, kc, nout, bstride, V, Yg, in_idx, out_idx, Vout, ostride,
                ld_out, single, Sg, npad, ystride, rpc);
        };
        auto pick = [&](auto pv) {
            constexpr int PV = decltype(pv)::value;
            // RB rows per thread: 4 on the FP32 vector path (2 with 40 or 48
            // outputs per pass, which keeps a restart's outputs in one pass), else 1
            constexpr int RB = (sizeof(T) == 4 && PV >= 1) ? 4 : 1;
            if constexpr (sizeof(T) == 4) {
                constexpr int RB48 = PV >= 1 ? 2 : 1;
                if (NO == 16) launch(k_rotate<T, 16, PV, RB>);
                else if (NO == 24) launch(k_rotate<T, 24, PV, RB>);
                else if (NO == 40) launch(k_rotate<T, 40, PV, RB48>);
                else launch(k_rotate<T, 48, PV, RB48>);
            } else {
                if (NO == 8) launch(k_rotate<T, 8, PV, RB>);
                else launch(k_rotate<T, 16, PV, RB>);
            }
        };
        profile_begin(st);
        if (vec && p == 1) pick(std::integral_constant<int, 1>());
        else if (vec && p == 2) pick(std::integral_constant<int, 2>());
        else if (vec && p == 4) pick(std::integral_constant<int, 4>());
        else pick(std::integral_constant<int, 0>());  // scalar loads
        done("k_rotate", (double)op.D * Sproc * p * ((double)kc / p + (double)nout / p) * sizeof(T));
    }
    void gather_block(int Snew, int p, int ld_in, int ld_out, const int* in_idx, const T* Vin,
                      T* Vout) const {
        profile_begin(st);
        k_gather_block<T><<<elem_grid(op.D * ld_out), 256, 0, st>>>(op.D, Snew, p, ld_in, ld_out,
                                                                     in_idx, Vin, Vout);
        done("k_gather_block", 2.0 * op.D * ld_out * sizeof(T));
    }
};

// host small dense linear algebra helpers (column-major)
static bool cholesky_lower(int n, std::vector<double>& a) {  // a = L L^T, L in lower part
    for (int j = 0; j < n; ++j) {
        double d = a[(size_t)j * n + j];
        for (int k = 0; k < j; ++k) d -= a[(size_t)k * n + j] * a[(size_t)k * n + j];
        if (!(d > 0.0)) return false;
        d = std::sqrt(d);
        a[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; ++i) {
            double v = a[(size_t)j * n + i];
            for (int k = 0; k < j; ++k) v -= a[(size_t)k * n + i] * a[(size_t)k * n + j];
            a[(size_t)j * n + i] = v / d;
        }
        for (int i = 0; i < j; ++i) a[(size_t)j * n + i] = 0.0;
    }
    return true;
}

// Generalised symmetric eigenproblem A z = theta G z of order n (column-major,
// both symmetrised here), G positive definite: Cholesky G = L L^T, then the
// standard problem L^{-1} A L^{-T}.  w receives the `want` lowest eigenvalues
// (ascending), zz their vectors (column i at zz[i n ..]).  False if G is not
// numerically positive definite or the eigensolve fails.
static bool rayleigh_ritz(int n, std::vector<double> G, std::vector<double> A, int want,
                          std::vector<double>& w, std::vector<double>& zz) {
    for (int a = 0; a < n; ++a)
        for (int b = a + 1; b < n; ++b) {
            const double g = 0.5 * (G[(size_t)b * n + a] + G[(size_t)a * n + b]);
            const double h = 0.5 * (A[(size_t)b * n + a] + A[(size_t)a * n + b]);
            G[(size_t)b * n + a] = G[(size_t)a * n + b] = g;
            A[(size_t)b * n + a] = A[(size_t)a * n + b] = h;
        }
    if (!cholesky_lower(n, G)) return false;
    auto Lv = [&](int i, int j) { return G[(size_t)j * n + i]; };
    std::vector<double> B(A);  // L B = A, column by column
    for (int c = 0; c < n; ++c)
        for (int i = 0; i < n; ++i) {
            double v = B[(size_t)c * n + i];
            for (int k = 0; k < i; ++k) v -= Lv(i, k) * B[(size_t)c * n + k];
            B[(size_t)c * n + i] = v / Lv(i, i);
        }
    std::vector<double> M((size_t)n * n);  // M L^T = B, row by row
    for (int r = 0; r < n; ++r)
        for (int j = 0; j < n; ++j) {
            double v = B[(size_t)j * n + r];
            for (int k = 0; k < j; ++k) v -= M[(size_t)k * n + r] * Lv(j, k);
            M[(size_t)j * n + r] = v / Lv(j, j);
        }
    for (int a = 0; a < n; ++a)
        for (int b = a + 1; b < n; ++b) {
            const double v = 0.5 * (M[(size_t)b * n + a] + M[(size_t)a * n + b]);
            M[(size_t)b * n + a] = M[(size_t)a * n + b] = v;
        }
    std::vector<double> ev(n);
    if (!symeig(n, M.data(), ev.data())) return false;
    w.assign(ev.begin(), ev.begin() + want);
    zz.assign((size_t)want * n, 0.0);
    for (int i = 0; i < want; ++i)  // z = L^{-T} u
        for (int a = n - 1; a >= 0; --a) {
            double v = M[(size_t)i * n + a];
            for (int k = a + 1; k < n; ++k) v -= Lv(k, a) * zz[(size_t)i * n + k];
            zz[(size_t)i * n + a] = v / Lv(a, a);
        }
    return true;
}

// ---------------------------------------------------------------------------
// the Lanczos phase (precision T for vectors)
// ---------------------------------------------------------------------------

template <class T>
static void lanczos_phase(const OpView<T>& op, const SolveRequest& rq,
                          const std::vector<double>& prm_all, cudaStream_t st, SolveResult& res,
                          int K, DevBuf<T>& Xout, std::vector<double>& theta_out) {
    const int64_t D = op.D;
    const int S0 = rq.S, p = rq.p;
    const int kmax = rq.kmax, nb = kmax / p, Tdim = kmax + p;
    const int64_t bmax = D * (int64_t)S0 * p;
    Launcher<T> L{op, st, &res.launches};
    DevBuf<int> tc_status(1);
    BH_CUDA(cudaMemsetAsync(tc_status.p, 0, sizeof(int), st));
    L.tc_status = tc_status.p;
    const int kcap = Tdim;
    int nch_max = 0, nchu_max = 0;
    for (int S = 1; S <= S0; ++S) {
        nch_max = std::max(nch_max, make_geo(D, S * p).nchunks);
        nchu_max = std::max(nchu_max, make_ugeo(D, S * p).nchunks);
    }

    // Va: basis (nb blocks + residual block).  Vb: restart target, and scratch
    // for the CholQR2 intermediate while a segment runs.
    DevBuf<T> Va((size_t)(nb + 1) * bmax), Vb((size_t)(nb + 1) * bmax), W((size_t)bmax);
    // part: chunk partials of the projections, and of the local coefficient
    // fused into the SpMM (at most 4 SM chunks of p rows)
    const size_t part_rows = std::max((size_t)nch_max * kcap, (size_t)4 * sm_count() * p);
    DevBuf<double> part(part_rows * S0 * p), gpart((size_t)nchu_max * p * S0 * p);
    DevBuf<T> Cf((size_t)kcap * S0 * p);
    DevBuf<double> Rinv((size_t)3 * S0 * p * p), Racc((size_t)S0 * p * p), Tm((size_t)S0 * Tdim * Tdim),
        d_prm((size_t)3 * S0);
    DevBuf<unsigned char> dead((size_t)S0 * Tdim);
    DevBuf<int> need3(1);
    BH_CUDA(cudaMemsetAsync(need3.p, 0, sizeof(int), st));
    DevBuf<int> d_in(S0), d_out(S0);
    DevBuf<T> Yd((size_t)S0 * kmax * kmax);
    Xout.alloc((size_t)D * S0 * K);
    theta_out.assign((size_t)S0 * K, 0.0);
    res.nconv.assign(S0, 0);
    res.conv_at.assign(S0, -1);
    res.scale.assign(S0, 1.0);
    res.status.assign(S0, BH_OK);
    res.live.assign(S0, kmax);

    std::vector<int> act(S0);  // original index of each active solve
    std::iota(act.begin(), act.end(), 0);
    int S = S0;
    auto upload_prm = [&]() {
        std::vector<double> pr((size_t)3 * S);
        for (int a = 0; a < S; ++a)
            for (int k = 0; k < 3; ++k) pr[3 * a + k] = prm_all[3 * act[a] + k];
        BH_CUDA(cudaMemcpyAsync(d_prm.p, pr.data(), pr.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaStreamSynchronize(st));  // host vector goes out of scope
    };
    upload_prm();
    BH_CUDA(cudaMemsetAsync(Tm.p, 0, Tm.bytes(), st));
    BH_CUDA(cudaMemsetAsync(dead.p, 0, dead.bytes(), st));
    const bool fp32 = std::is_same<T, float>::value;
    // shifted first pass: cond(W R0^{-1})^2 <= 1 / shift_rel, small enough for
    // two plain Cholesky QR passes in this precision
    const double shift_rel = fp32 ? 1e3 * 1.1920929e-7 : 1e3 * 2.220446049250313e-16;
    // a direction is dropped only at rounding-noise level
    const double kill_abs = fp32 ? 3.0 * 1.1920929e-7 : 1e2 * 2.220446049250313e-16;

    // orthonormalise the block W into Vout (scratch: Vb); T coupling written for jrow > 0
    auto orthonormalize = [&](const Geo& gu, int ncols, T* Wb, T* Vout, int jrow, bool gram_done) {
        T* scratch = Vb.p;
        double* Tj = jrow > 0 ? Tm.p : nullptr;
        if (L.vec_ok(ncols, ncols, p, 0, Wb, Vout)) {
            // factors in three slots; each pass re-reads W and applies them in registers
            const int64_t rs = (int64_t)S * p * p;
            if (!gram_done) L.normgram(gu, p, 0, Rinv.p, rs, Wb, nullptr, 1, gpart.p);
            if (p == 1) {
                L.qr(gu, S, p, gpart.p, 2, 0.0, Racc.p, Rinv.p, Tj, Tdim, jrow, kill_abs, dead.p);
                L.normgram(gu, p, 1, Rinv.p, rs, Wb, Vout, 0, gpart.p);
                return;
            }
            // need3 counts the solves whose first pass needed the shift; when
            // none did, the third pass is skipped on the device (CholQR2)
            L.qr(gu, S, p, gpart.p, 0, shift_rel, Racc.p, Rinv.p, nullptr, Tdim, jrow, kill_abs, nullptr, need3.p);
            L.normgram(gu, p, 1, Rinv.p, rs, Wb, nullptr, 1, gpart.p);
            L.qr(gu, S, p, gpart.p, 1, 0.0, Racc.p, Rinv.p + rs, nullptr, Tdim, jrow, kill_abs, nullptr);
            L.normgram(gu, p, 2, Rinv.p, rs, Wb, nullptr, 1, gpart.p, need3.p);
            L.qr(gu, S, p, gpart.p, 2, 0.0, Racc.p, Rinv.p + 2 * rs, Tj, Tdim, jrow, kill_abs, dead.p, need3.p);
            L.normgram(gu, p, 3, Rinv.p, rs, Wb, Vout, 0, gpart.p, nullptr, need3.p);
            return;
        }
        if (!gram_done) L.update(gu, p, 0, 0, Va.p, Cf.p, Wb, 1, gpart.p);
        if (p == 1) {
            L.qr(gu, S, p, gpart.p, 2, 0.0, Racc.p, Rinv.p, Tj, Tdim, jrow, kill_abs, dead.p);
            L.normalize(ncols, p, Rinv.p, Wb, Vout);
            return;
        }
        // shifted CholQR3: Wb -> scratch -> Wb -> Vout (no device-side pass skipping here)
        L.qr(gu, S, p, gpart.p, 0, shift_rel, Racc.p, Rinv.p, nullptr, Tdim, jrow, kill_abs, nullptr);
        L.normalize(ncols, p, Rinv.p, Wb, scratch);
        L.update(gu, p, 0, 0, Va.p, Cf.p, scratch, 1, gpart.p);
        L.qr(gu, S, p, gpart.p, 1, 0.0, Racc.p, Rinv.p, nullptr, Tdim, jrow, kill_abs, nullptr);
        L.normalize(ncols, p, Rinv.p, scratch, Wb);
        L.update(gu, p, 0, 0, Va.p, Cf.p, Wb, 1, gpart.p);
        L.qr(gu, S, p, gpart.p, 2, 0.0, Racc.p, Rinv.p, Tj, Tdim, jrow, kill_abs, dead.p);
        L.normalize(ncols, p, Rinv.p, Wb, Vout);
    };

    // start block: W = seeded stream; V_1 = H W (Spectra forces v into range(A)); V_0 = QR(V_1)
    {
        const int ncols = S * p;
        const int64_t bstride = D * ncols;
        k_start_block<T><<<elem_grid(bstride), 256, 0, st>>>(D, ncols, p, rq.seed, rq.d_perm, W.p);
        BH_CUDA(cudaGetLastError());
        ++res.launches;
        T* V1 = Va.p + bstride;
        L.spmm(ncols, p, d_prm.p, W.p, V1);
        res.matvecs += p;
        const Geo gu0 = make_ugeo(D, ncols);
        orthonormalize(gu0, ncols, V1, Va.p, 0, false);
        // H W can lose rank (H singular on the seeded block, e.g. the
        // one-state sector with H = 0): then start from the seeded block itself
        std::vector<double> hr((size_t)S * p * p);
        BH_CUDA(cudaMemcpyAsync(hr.data(), Racc.p, hr.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaStreamSynchronize(st));
        bool degenerate = false;
        for (int a = 0; a < S; ++a)
            for (int q = 0; q < p; ++q) degenerate |= !(hr[(size_t)a * p * p + q * p + q] != 0.0);
        if (degenerate) orthonormalize(gu0, ncols, W.p, Va.p, 0, false);
    }

    std::vector<double> hT, theta((size_t)S0 * kmax), Yh((size_t)S0 * kmax * kmax), resid((size_t)S0 * kmax);
    std::vector<unsigned char> hdead;
    std::vector<int> kuse(S0, kmax);
    std::vector<T> Yt;
    int jstart = 0;
    bool after_restart = false;
    int restarts = 0;
    const double eps23 = std::pow(2.220446049250313e-16, 2.0 / 3.0);
    // The block steps jstart..nb-1 of a restart cycle launch the same kernels
    // with the same arguments whenever the batch (S, jstart, after_restart) is
    // unchanged, and need no host synchronisation: they are captured once as a
    // CUDA graph and replayed (the slow last solves of a batch run many
    // cycles at S = 1, where launch latency dominates).
    // Va and Vb swap at every restart, so two graphs (one per buffer) are kept.
    struct CycleGraph {
        cudaGraphExec_t exec = nullptr;
        int S = -1, jstart = -1;
        bool after = false;
        const T* va = nullptr;
        int64_t launches = 0, matvecs = 0;
        ~CycleGraph() {
            if (exec) cudaGraphExecDestroy(exec);
        }
    } cgs[2];
    bool graphs_failed = false;
    auto run_steps = [&](int ncols, int64_t bstride, const Geo& g, const Geo& gu) {
        for (int j = jstart; j < nb; ++j) {
            T* Vj = Va.p + (int64_t)j * bstride;
            // W = H V_j, with the partials of A = V_j^T W fused in where possible
            int dparts = 0;
            L.spmm(ncols, p, d_prm.p, Vj, W.p, separate_local_dot() ? nullptr : part.p, &dparts);
            res.matvecs += p;
            // local step: A = V_j^T W, then W -= V_j A + earlier couplings
            const int c_lo = (j == jstart && after_restart) ? 0 : std::max(0, (j - 1) * p);
            if (dparts > 0) {
                Geo gs = g;
                gs.nchunks = dparts;
                L.local_coef(gs, j, c_lo, p, p, part.p, Tm.p, Tdim, Cf.p);
            } else {
                L.dot(g, ncols, p, 1, bstride, Vj, W.p, kcap, part.p);
                L.local_coef(g, j, c_lo, p, kcap, part.p, Tm.p, Tdim, Cf.p);
            }
            L.update(gu, p, (j + 1) * p - c_lo, bstride, Va.p + (int64_t)(c_lo / p) * bstride, Cf.p,
                     W.p, 0, gpart.p, "k_update(local)");
            // one full re-orthogonalisation pass, Gram matrix of the result
            const int kc = (j + 1) * p;
            L.dot(g, ncols, p, j + 1, bstride, Va.p, W.p, kcap, part.p);
            L.dot_finalize(g, kc, ncols, p, kcap, part.p, nullptr, Cf.p, Tm.p, Tdim, j);
            L.update(gu, p, kc, bstride, Va.p, Cf.p, W.p, 1, gpart.p);
            orthonormalize(gu, ncols, W.p, Va.p + (int64_t)(j + 1) * bstride, j + 1, true);
        }
    };
    for (;;) {
        const int ncols = S * p;
        const int64_t bstride = D * ncols;
        const Geo g = make_geo(D, ncols), gu = make_ugeo(D, ncols);
        const bool graphs = after_restart && !graphs_failed && use_graphs() && !profile_on() && !debug_ortho();
        CycleGraph& cg = cgs[restarts & 1];
        if (graphs && cg.exec && cg.S == S && cg.jstart == jstart && cg.after == after_restart &&
            cg.va == Va.p) {
            BH_CUDA(cudaGraphLaunch(cg.exec, st));
            res.launches += cg.launches;
            res.matvecs += cg.matvecs;
        } else if (graphs) {
            if (cg.exec) {
                BH_CUDA(cudaGraphExecDestroy(cg.exec));
                cg.exec = nullptr;
            }
            // the products of the captured steps take the tuned shape of this
            // width: time it now if the table lacks it (W is overwritten by
            // the cycle's first product before anything reads it)
            res.launches += tune_spmm<T>(op, ncols, p, d_prm.p, Va.p + (int64_t)jstart * bstride, W.p, st,
                                         !separate_local_dot());
            const int64_t l0 = res.launches, m0 = res.matvecs;
            cudaGraph_t graph = nullptr;
            BH_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            try {
                run_steps(ncols, bstride, g, gu);
            } catch (...) {
                cudaStreamEndCapture(st, &graph);
                if (graph) cudaGraphDestroy(graph);
                throw;
            }
            BH_CUDA(cudaStreamEndCapture(st, &graph));
            cudaGraphExec_t exec = nullptr;
            const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                // nothing of the captured cycle has run: launch it directly
                // and keep direct launches for the rest of this solve
                (void)cudaGetLastError();
                if (verbose())
                    std::fprintf(stderr, "[bh] cycle graph not instantiated (%s): direct launches\n",
                                 cudaGetErrorString(e));
                graphs_failed = true;
                res.launches = l0;
                res.matvecs = m0;
                run_steps(ncols, bstride, g, gu);
                goto cycle_done;
            }
            cg.exec = exec;
            cg.S = S;
            cg.jstart = jstart;
            cg.after = after_restart;
            cg.va = Va.p;
            cg.launches = res.launches - l0;
            cg.matvecs = res.matvecs - m0;
            BH_CUDA(cudaGraphLaunch(cg.exec, st));
        } else {
            run_steps(ncols, bstride, g, gu);
        }
    cycle_done:
        if (debug_ortho()) {
            // Gram matrix of all nb + 1 blocks against each block, solve 0
            double worst = 0.0;
            std::vector<double> hc((size_t)(kmax + p) * ncols);
            DevBuf<double> dC((size_t)(kmax + p) * ncols);
            for (int jb = 0; jb <= nb; ++jb) {
                L.dot(g, ncols, p, nb + 1, bstride, Va.p, Va.p + (int64_t)jb * bstride, kcap, part.p);
                L.dot_finalize(g, kmax + p, ncols, p, kcap, part.p, dC.p, nullptr, nullptr, 0, 0);
                BH_CUDA(cudaMemcpyAsync(hc.data(), dC.p, hc.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
                BH_CUDA(cudaStreamSynchronize(st));
                for (int c = 0; c < kmax + p; ++c)
                    for (int q = 0; q < p; ++q) {
                        const double want = (c == jb * p + q) ? 1.0 : 0.0;
                        worst = std::max(worst, std::fabs(hc[(size_t)c * ncols + q] - want));
                    }
            }
            std::fprintf(stderr, "[bh] restart %d: solve %d basis max|V^T V - I| = %.3e\n", restarts, act[0], worst);
        }
        hT.resize((size_t)S * Tdim * Tdim);
        hdead.resize((size_t)S * Tdim);
        BH_CUDA(cudaMemcpyAsync(hT.data(), Tm.p, hT.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaMemcpyAsync(hdead.data(), dead.p, hdead.size(), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaStreamSynchronize(st));

        // Rayleigh-Ritz per active solve (host, FP64) on the live columns of T
        std::vector<int> nconv(S, 0);
        std::vector<double> hscale(S, 1.0);
        bool symeig_failed = false;
        parallel_for(S, [&](int a) {
            const double* Ts = hT.data() + (size_t)a * Tdim * Tdim;
            const unsigned char* dd = hdead.data() + (size_t)a * Tdim;
            std::vector<int> live;
            for (int c = 0; c < kmax; ++c)
                if (!dd[c]) live.push_back(c);
            const int k = (int)live.size();
            kuse[a] = k;
            std::vector<double> m((size_t)k * k), w(k);
            for (int jj = 0; jj < k; ++jj)
                for (int ii = 0; ii < k; ++ii) {
                    const int lo = std::min(live[ii], live[jj]), hi = std::max(live[ii], live[jj]);
                    m[(size_t)jj * k + ii] = Ts[(size_t)hi * Tdim + lo];  // upper triangle
                }
            if (!symeig(k, m.data(), w.data())) symeig_failed = true;
            double sc = 0.0;
            for (int i = 0; i < k; ++i) sc = std::max(sc, std::fabs(w[i]));
            hscale[a] = std::max(sc, 1e-300);
            for (int i = 0; i < kmax; ++i)
                for (int c = 0; c < kmax; ++c) Yh[((size_t)a * kmax + c) * kmax + i] = 0.0;
            for (int i = 0; i < k; ++i) {
                theta[(size_t)a * kmax + i] = w[i];
                for (int ii = 0; ii < k; ++ii) Yh[((size_t)a * kmax + live[ii]) * kmax + i] = m[(size_t)i * k + ii];
                double r2 = 0.0;
                for (int a2 = 0; a2 < p; ++a2) {
                    double v = 0.0;
                    for (int b2 = 0; b2 < p; ++b2)
                        v += Ts[(size_t)(kmax - p + b2) * Tdim + kmax + a2] *
                             Yh[((size_t)a * kmax + kmax - p + b2) * kmax + i];
                    r2 += v * v;
                }
                resid[(size_t)a * kmax + i] = std::sqrt(r2);
            }
            // Convergence: resid <= tol * max(|theta|, floor).  Spectra uses
            // floor = eps^(2/3); a residual estimate built from the computed
            // projection cannot fall below ~eps * ||H||, so the floor here is
            // a fraction of the spectral radius estimate (largest |Ritz value|).
            int nc = 0;
            const double floor_abs = rq.precision == BH_PREC_MIXED ? hscale[a] : std::max(eps23, 1e-3 * hscale[a]);
            for (int i = 0; i < std::min(rq.nev, k); ++i) {
                const double th = std::fabs(w[i]);
                if (resid[(size_t)a * kmax + i] <= rq.tol * std::max(th, floor_abs)) ++nc;
            }
            nconv[a] = nc;
        });
        if (symeig_failed) throw Error(BH_ERR_NOCONV, "projected eigenproblem did not converge");
        const bool last = restarts >= rq.max_restarts;
        std::vector<int> fin, cont;  // active positions
        int minconv = rq.nev, ndead = 0;
        for (int a = 0; a < S; ++a) {
            const int o = act[a];
            res.nconv[o] = nconv[a];
            res.scale[o] = hscale[a];
            res.live[o] = kuse[a];
            ndead += kmax - kuse[a];
            if (kuse[a] < rq.nev) {
                // Krylov space exhausted before nev directions (an invariant
                // start block, or a sector smaller than the request): retire
                // the solve with the Ritz pairs it holds
                res.status[o] = BH_ERR_BREAKDOWN;
                fin.push_back(a);
                minconv = std::min(minconv, nconv[a]);
                continue;
            }
            const bool conv_a = nconv[a] >= rq.nev;
            if (conv_a && res.conv_at[o] < 0) res.conv_at[o] = restarts;
            if (conv_a || last) fin.push_back(a);
            else cont.push_back(a);
            minconv = std::min(minconv, nconv[a]);
        }
        if (verbose()) {
            double worst = 0.0;
            for (int a = 0; a < S; ++a)
                for (int i = 0; i < rq.nev && i < kuse[a]; ++i) {
                    const double floor_abs = rq.precision == BH_PREC_MIXED ? hscale[a] : std::max(eps23, 1e-3 * hscale[a]);
                    worst = std::max(worst, resid[(size_t)a * kmax + i] / std::max(std::fabs(theta[(size_t)a * kmax + i]), floor_abs));
                }
            std::fprintf(stderr, "[bh] restart %d: active %d, retiring %d, min nconv %d, dropped dirs %d, worst rel resid %.3e\n",
                         restarts, S, (int)fin.size(), minconv, ndead, worst);
            for (int a : fin) {
                std::fprintf(stderr, "[bh]   retire solve %d: live %d theta0 %.10f resid:", act[a], kuse[a],
                             theta[(size_t)a * kmax]);
                for (int i = 0; i < rq.nev && i < kuse[a]; ++i) std::fprintf(stderr, " %.1e", resid[(size_t)a * kmax + i]);
                std::fprintf(stderr, "\n");
            }
        }

        // retire finished solves: their K lowest Ritz vectors go to Xout[:, orig K + i]
        if (!fin.empty()) {
            const int nf = (int)fin.size();
            Yt.assign((size_t)nf * kmax * K, T(0));
            std::vector<int> in(nf), out(nf);
            for (int f = 0; f < nf; ++f) {
                const int a = fin[f], o = act[a];
                in[f] = a;
                out[f] = o;
                for (int i = 0; i < K; ++i) {
                    theta_out[(size_t)o * K + i] = i < kuse[a] ? theta[(size_t)a * kmax + i] : 0.0;
                    for (int c = 0; c < kmax; ++c)
                        Yt[((size_t)f * kmax + c) * K + i] = i < kuse[a] ? (T)Yh[((size_t)a * kmax + c) * kmax + i] : T(0);
                }
            }
            BH_CUDA(cudaMemcpyAsync(Yd.p, Yt.data(), Yt.size() * sizeof(T), cudaMemcpyHostToDevice, st));
            BH_CUDA(cudaMemcpyAsync(d_in.p, in.data(), nf * sizeof(int), cudaMemcpyHostToDevice, st));
            BH_CUDA(cudaMemcpyAsync(d_out.p, out.data(), nf * sizeof(int), cudaMemcpyHostToDevice, st));
            L.rotate(nf, ncols, p, kmax, K, bstride, Va.p, Yd.p, d_in.p, d_out.p, Xout.p, 0, S0 * K, 1);
            BH_CUDA(cudaStreamSynchronize(st));
        }
        if (cont.empty()) break;

        // thick restart of the continuing solves, compacted to the front
        int nkeep = rq.nev + std::max(p, (int)(keep_fraction() * (kmax - rq.nev)));
        nkeep = (nkeep + p - 1) / p * p;
        nkeep = std::min(nkeep, kmax - 2 * p);
        if (nkeep < p) nkeep = p;
        for (int a : cont) nkeep = std::min(nkeep, kuse[a] / p * p);
        const int nc = (int)cont.size();
        const int ncols2 = nc * p;
        const int64_t bstride2 = D * ncols2;
        Yt.assign((size_t)nc * kmax * nkeep, T(0));
        std::vector<int> in(nc), out(nc);
        for (int f = 0; f < nc; ++f) {
            const int a = cont[f];
            in[f] = a;
            out[f] = f;
            for (int c = 0; c < kmax; ++c)
                for (int i = 0; i < nkeep; ++i)
                    Yt[((size_t)f * kmax + c) * nkeep + i] = (T)Yh[((size_t)a * kmax + c) * kmax + i];
        }
        BH_CUDA(cudaMemcpyAsync(Yd.p, Yt.data(), Yt.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaMemcpyAsync(d_in.p, in.data(), nc * sizeof(int), cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaMemcpyAsync(d_out.p, out.data(), nc * sizeof(int), cudaMemcpyHostToDevice, st));
        L.rotate(nc, ncols, p, kmax, nkeep, bstride, Va.p, Yd.p, d_in.p, d_out.p, Vb.p, bstride2, ncols2, 0,
                 nc == S);
        L.gather_block(nc, p, ncols, ncols2, d_in.p, Va.p + (int64_t)nb * bstride,
                       Vb.p + (int64_t)(nkeep / p) * bstride2);
        std::swap(Va.p, Vb.p);  // equal sizes: ownership stays balanced
        if (debug_ortho()) {
            // orthonormality of the rotated basis (nkeep/p + 1 blocks), solve 0
            const Geo g2 = make_geo(D, ncols2);
            const int nbk = nkeep / p + 1;
            double worst = 0.0;
            std::vector<double> hc((size_t)nbk * p * ncols2);
            DevBuf<double> dC((size_t)nbk * p * ncols2);
            for (int jb = 0; jb < nbk; ++jb) {
                L.dot(g2, ncols2, p, nbk, bstride2, Va.p, Va.p + (int64_t)jb * bstride2, kcap, part.p);
                L.dot_finalize(g2, nbk * p, ncols2, p, kcap, part.p, dC.p, nullptr, nullptr, 0, 0);
                BH_CUDA(cudaMemcpyAsync(hc.data(), dC.p, hc.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
                BH_CUDA(cudaStreamSynchronize(st));
                for (int c = 0; c < nbk * p; ++c)
                    for (int q = 0; q < p; ++q) {
                        const double want = (c == jb * p + q) ? 1.0 : 0.0;
                        worst = std::max(worst, std::fabs(hc[(size_t)c * ncols2 + q] - want));
                    }
            }
            std::fprintf(stderr, "[bh] restart %d: rotated basis max|V^T V - I| = %.3e (nkeep %d)\n", restarts, worst, nkeep);
        }
        // projected matrix of the continuing solves: diag(theta_keep) plus the
        // coupling rows  T[nkeep + a][i] = sum_b R_last[a][b] Y[kmax - p + b][i]
        // (the upper arrowhead is filled by the next local step); the dropped
        // flags of the residual block move with it
        std::vector<double> hTn((size_t)nc * Tdim * Tdim, 0.0);
        std::vector<unsigned char> hdn((size_t)nc * Tdim, 0);
        for (int f = 0; f < nc; ++f) {
            const int a = cont[f];
            const double* To = hT.data() + (size_t)a * Tdim * Tdim;
            double* Ts = hTn.data() + (size_t)f * Tdim * Tdim;
            for (int i = 0; i < nkeep; ++i) Ts[(size_t)i * Tdim + i] = theta[(size_t)a * kmax + i];
            for (int a2 = 0; a2 < p; ++a2) {
                hdn[(size_t)f * Tdim + nkeep + a2] = hdead[(size_t)a * Tdim + kmax + a2];
                for (int i = 0; i < nkeep; ++i) {
                    double v = 0.0;
                    for (int b = 0; b < p; ++b)
                        v += To[(size_t)(kmax - p + b) * Tdim + kmax + a2] *
                             Yh[((size_t)a * kmax + kmax - p + b) * kmax + i];
                    Ts[(size_t)i * Tdim + nkeep + a2] = v;
                }
            }
        }
        std::vector<int> act2(nc);
        for (int f = 0; f < nc; ++f) act2[f] = act[cont[f]];
        act.swap(act2);
        S = nc;
        BH_CUDA(cudaMemcpyAsync(Tm.p, hTn.data(), hTn.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaMemcpyAsync(dead.p, hdn.data(), hdn.size(), cudaMemcpyHostToDevice, st));
        upload_prm();
        jstart = nkeep / p;
        after_restart = true;
        ++restarts;
    }
    res.restarts = restarts;
    int tc_err = 0;
    BH_CUDA(cudaMemcpyAsync(&tc_err, tc_status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    BH_CUDA(cudaStreamSynchronize(st));
    if (tc_err) throw Error(BH_ERR_TIMEOUT, "tensor-core rotation: a bounded mbarrier wait ran out");
}

void apply_operator(const OpView<double>& op, int ncols, int group, const double* d_prm,
                    const double* d_X, double* d_Y, cudaStream_t st) {
    int64_t launches = 0;
    Launcher<double> L{op, st, &launches};
    L.spmm(ncols, group, d_prm, d_X, d_Y);
}

// Same product, launched with no profiling events and no host allocation.
void apply_operator_raw(const OpView<double>& op, int ncols, int group, const double* d_prm,
                        const double* d_X, double* d_Y, cudaStream_t st) {
    (void)launch_spmm<double>(op, ncols, group, d_prm, d_X, d_Y, st, nullptr, nullptr, false);
    BH_CUDA(cudaGetLastError());
}

SolveResult block_lanczos(const OpView<double>& op64, const OpView<float>& op32,
                          const SolveRequest& rq, cudaStream_t st) {
    SolveResult res;
    const int S = rq.S, p = rq.p;
    const int64_t D = op64.D;
    BH_REQUIRE(S >= 1 && p >= 1 && p <= 16 && (p & (p - 1)) == 0, "block size must be 1, 2, 4, 8 or 16");
    BH_REQUIRE(rq.nev >= 1 && rq.nev <= 32, "nev must be in [1, 32]");
    BH_REQUIRE((int64_t)S * p <= 512, "batch too wide: S * block must be <= 512");
    BH_REQUIRE(rq.kmax % p == 0 && (rq.kmax >= rq.nev + p || (rq.kmax == D && rq.kmax >= rq.nev)),
               "ncv must be a multiple of the block size and >= nev + block (or the whole space)");
    BH_REQUIRE((int64_t)rq.kmax <= D, "ncv exceeds the dimension");
    const int K0 = (rq.nev + p - 1) / p * p;  // Ritz vectors needed
    BH_REQUIRE(K0 <= 32 && K0 <= rq.kmax, "too many wanted eigenvalues for this block size");
    // Ritz vectors refined in FP64: the wanted ones plus a margin (whole
    // blocks), so that the Rayleigh-Ritz error of the highest wanted values is
    // set by their gap to the first level outside the refined space
    const int K = std::max(K0, std::min({32, rq.kmax, (rq.nev + ritz_margin() + p - 1) / p * p}));

    // per-solve parameters (J, U, shift) and start scale
    std::vector<double> prm((size_t)3 * S);
    for (int s = 0; s < S; ++s) {
        prm[3 * s] = rq.J[s];
        prm[3 * s + 1] = rq.U[s];
        prm[3 * s + 2] = rq.shift[s];
    }
    DevBuf<double> d_prm(prm.size());
    BH_CUDA(cudaMemcpyAsync(d_prm.p, prm.data(), prm.size() * sizeof(double), cudaMemcpyHostToDevice, st));

    // ---- Lanczos phase ----
    DevBuf<double> X64;
    std::vector<double> theta0;
    if (rq.precision == BH_PREC_MIXED) {
        BH_REQUIRE(op32.tv != nullptr || op32.occ != nullptr, "mixed precision needs FP32 operator values");
        DevBuf<float> X32;
        lanczos_phase<float>(op32, rq, prm, st, res, K, X32, theta0);
        X64.alloc((size_t)D * S * K);
        k_convert<float, double><<<elem_grid(D * S * K), 256, 0, st>>>(D * S * K, X32.p, X64.p);
        BH_CUDA(cudaGetLastError());
        ++res.launches;
        BH_CUDA(cudaStreamSynchronize(st));
    } else {
        lanczos_phase<double>(op64, rq, prm, st, res, K, X64, theta0);
    }

    // ---- FP64 refinement of the K Ritz vectors per solve ----
    // Stage 1: Rayleigh-Ritz on X (FP64 product, FP64 Gram matrices).
    // Stage 2 (mixed precision, BH_RITZ_STAGE2=1): Rayleigh-Ritz on [X, R]
    // with the stage-1 residual vectors R = H X z_i - theta_i X z_i (one
    // step of a block Davidson iteration without preconditioner).
    const int nc2 = S * K;
    Launcher<double> L{op64, st, &res.launches};
    DevBuf<double> Y64((size_t)D * nc2);
    L.spmm(nc2, K, d_prm.p, X64.p, Y64.p);
    res.matvecs += K;
    // Gram matrices per solve, in groups of at most 512 columns
    const int sgrp = std::max(1, std::min(S, 512 / K));
    const Geo gmax = make_geo(D, sgrp * K);
    DevBuf<double> part((size_t)gmax.nchunks * K * sgrp * K), rpart((size_t)gmax.nchunks * sgrp * K);
    // C[a * nc2 + s K + b] = sum_r A[r][s K + a] B[r][s K + b] for every solve
    auto gram = [&](const double* A, const double* B, DevBuf<double>& C) {
        if (C.n < (size_t)K * nc2) C.alloc((size_t)K * nc2);
        for (int s0 = 0; s0 < S; s0 += sgrp) {
            const int ns = std::min(sgrp, S - s0);
            const Geo gg = make_geo(D, ns * K);
            const int64_t off = (int64_t)s0 * K;
            L.dot(gg, nc2, K, 1, 0, A + off, B + off, K, part.p);
            L.dot_finalize(gg, K, nc2, K, K, part.p, C.p + off, nullptr, nullptr, 0, 0);
        }
    };
    auto to_host = [&](const DevBuf<double>& C) {
        std::vector<double> h((size_t)K * nc2);
        BH_CUDA(cudaMemcpyAsync(h.data(), C.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        return h;
    };
    // out (optional) and/or squared-norm partials of the columns
    //   sum_a (Y1 - theta X1)[:, a] Z1[a][i] + sum_a (Y2 - theta X2)[:, a] Z2[a][i]
    auto mix = [&](const double* Y1, const double* X1, const double* Z1, const double* Y2,
                   const double* X2, const double* Z2, const double* theta, double* out,
                   double* norms) {
        for (int s0 = 0; s0 < S; s0 += sgrp) {
            const int ns = std::min(sgrp, S - s0);
            const Geo gg = make_geo(D, ns * K);
            const int64_t off = (int64_t)s0 * K;
            const int64_t zoff = off * K;
            // operands read once (Y1, X1 and the second pair when present), result written once
            const int nin = (Y1 ? 1 : 0) + (X1 ? 1 : 0) + (Y2 ? 1 : 0) + (X2 ? 1 : 0);
            L.profile_begin_();
            k_ritz_mix<<<gg.nchunks, gg.NT, norms ? gg.NT * sizeof(double) : 0, st>>>(
                D, ns * K, nc2, K, Y1 + off, X1 ? X1 + off : nullptr, Z1 + zoff, Y2 ? Y2 + off : nullptr,
                X2 ? X2 + off : nullptr, Z2 ? Z2 + zoff : nullptr, theta ? theta + off : nullptr,
                out ? out + off : nullptr, gg.rows_per_chunk, norms ? rpart.p : nullptr);
            L.done("k_ritz_mix", (double)(nin + (out ? 1 : 0)) * D * ns * K * sizeof(double));
            if (norms) {
                L.profile_begin_();
                k_sum_cols<<<(ns * K + 255) / 256, 256, 0, st>>>(gg.nchunks, ns * K, rpart.p, norms + off);
                L.done("k_sum_cols", (double)gg.nchunks * ns * K * sizeof(double));
            }
        }
    };
    DevBuf<double> Gd, Ad;
    gram(X64.p, X64.p, Gd);
    gram(X64.p, Y64.p, Ad);
    const std::vector<double> hG = to_host(Gd), hA = to_host(Ad);
    BH_CUDA(cudaStreamSynchronize(st));
    const double nan = std::numeric_limits<double>::quiet_NaN();
    std::vector<double> th((size_t)nc2, nan), Z((size_t)S * K * K, 0.0);
    std::vector<int> kref(S, K);  // Ritz vectors refined per solve
    parallel_for(S, [&](int s) {
        // a solve whose Krylov space broke down holds only res.live[s] Ritz
        // vectors (the rest are zero): the refinement uses those
        const int k = std::min(K, std::max(0, res.live[s]));
        kref[s] = k;
        if (k == 0) return;
        std::vector<double> Gm((size_t)k * k), Am((size_t)k * k), w, zz;
        for (int a = 0; a < k; ++a)
            for (int b = 0; b < k; ++b) {
                Gm[(size_t)b * k + a] = hG[(size_t)a * nc2 + s * K + b];
                Am[(size_t)b * k + a] = hA[(size_t)a * nc2 + s * K + b];
            }
        if (!rayleigh_ritz(k, Gm, Am, k, w, zz)) {
            kref[s] = 0;
            if (res.status[s] == BH_OK) res.status[s] = BH_ERR_NOCONV;
            return;
        }
        // Z_s is K x K (entry [a][i] at (s K + a) K + i); rows and columns beyond k stay zero
        for (int i = 0; i < k; ++i) {
            th[(size_t)s * K + i] = w[i];
            for (int a = 0; a < k; ++a) Z[((size_t)s * K + a) * K + i] = zz[(size_t)i * k + a];
        }
    });
    DevBuf<double> d_th(nc2), d_Z(Z.size()), rn(nc2);
    BH_CUDA(cudaMemcpyAsync(d_th.p, th.data(), nc2 * sizeof(double), cudaMemcpyHostToDevice, st));
    BH_CUDA(cudaMemcpyAsync(d_Z.p, Z.data(), Z.size() * sizeof(double), cudaMemcpyHostToDevice, st));

    std::vector<double> Zr((size_t)S * K * K, 0.0);  // stage-2 coefficients on R (zero: not used)
    DevBuf<double> Rb, HRb;
    const bool stage2 = rq.precision == BH_PREC_MIXED && ritz_stage2();
    if (stage2) {
        Rb.alloc((size_t)D * nc2);
        HRb.alloc((size_t)D * nc2);
        mix(Y64.p, X64.p, d_Z.p, nullptr, nullptr, nullptr, d_th.p, Rb.p, nullptr);
        L.spmm(nc2, K, d_prm.p, Rb.p, HRb.p);
        res.matvecs += K;
        DevBuf<double> Gxr, Grr, Axh, Arh;
        gram(X64.p, Rb.p, Gxr);
        gram(Rb.p, Rb.p, Grr);
        gram(X64.p, HRb.p, Axh);
        gram(Rb.p, HRb.p, Arh);
        const std::vector<double> hGxr = to_host(Gxr), hGrr = to_host(Grr), hAxh = to_host(Axh),
                                  hArh = to_host(Arh);
        BH_CUDA(cudaStreamSynchronize(st));
        parallel_for(S, [&](int s) {
            if (res.status[s] != BH_OK || kref[s] < K) return;
            // residual directions above FP64 noise of the spectrum's scale,
            // each scaled to unit norm
            const double noise = 1e-13 * std::max(1.0, res.scale[s]);
            std::vector<int> keep;
            std::vector<double> sig;
            for (int b = 0; b < K; ++b) {
                const double g = hGrr[(size_t)b * nc2 + s * K + b];
                if (g > noise * noise) {
                    keep.push_back(b);
                    sig.push_back(1.0 / std::sqrt(g));
                }
            }
            const int kr = (int)keep.size();
            if (kr == 0) return;
            const int n2 = K + kr;
            auto G = [&](const std::vector<double>& h, int a, int b) { return h[(size_t)a * nc2 + s * K + b]; };
            std::vector<double> G2((size_t)n2 * n2), A2((size_t)n2 * n2), w, zz;
            for (int a = 0; a < n2; ++a)
                for (int b = 0; b < n2; ++b) {
                    double g, h;
                    if (a < K && b < K) {
                        g = G(hG, a, b);
                        h = G(hA, a, b);
                    } else if (a < K) {  // X_a^T r_b
                        const int rb = keep[b - K];
                        g = G(hGxr, a, rb) * sig[b - K];
                        h = G(hAxh, a, rb) * sig[b - K];
                    } else if (b < K) {  // r_a^T X_b
                        const int ra = keep[a - K];
                        g = G(hGxr, b, ra) * sig[a - K];
                        h = G(hAxh, b, ra) * sig[a - K];
                    } else {
                        const int ra = keep[a - K], rb = keep[b - K];
                        g = G(hGrr, ra, rb) * sig[a - K] * sig[b - K];
                        h = G(hArh, ra, rb) * sig[a - K] * sig[b - K];
                    }
                    G2[(size_t)b * n2 + a] = g;
                    A2[(size_t)b * n2 + a] = h;
                }
            if (!rayleigh_ritz(n2, G2, A2, K, w, zz)) return;  // keep the stage-1 pairs
            for (int i = 0; i < K; ++i) {
                th[(size_t)s * K + i] = w[i];
                for (int a = 0; a < K; ++a) Z[((size_t)s * K + a) * K + i] = zz[(size_t)i * n2 + a];
                for (int q = 0; q < kr; ++q)
                    Zr[((size_t)s * K + keep[q]) * K + i] = zz[(size_t)i * n2 + K + q] * sig[q];
            }
        });
        BH_CUDA(cudaMemcpyAsync(d_th.p, th.data(), nc2 * sizeof(double), cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaMemcpyAsync(d_Z.p, Z.data(), Z.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    DevBuf<double> d_Zr;
    if (stage2) {
        d_Zr.alloc(Zr.size());
        BH_CUDA(cudaMemcpyAsync(d_Zr.p, Zr.data(), Zr.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    // true residual norms ||H x_i - theta_i x_i||^2 of the returned pairs
    mix(Y64.p, X64.p, d_Z.p, stage2 ? HRb.p : nullptr, stage2 ? Rb.p : nullptr, stage2 ? d_Zr.p : nullptr,
        d_th.p, nullptr, rn.p);
    std::vector<double> hrn(nc2);
    BH_CUDA(cudaMemcpyAsync(hrn.data(), rn.p, nc2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    DevBuf<double> Xf;
    if (rq.want_vectors) {
        Xf.alloc((size_t)D * nc2);
        mix(X64.p, nullptr, d_Z.p, stage2 ? Rb.p : nullptr, nullptr, stage2 ? d_Zr.p : nullptr, nullptr,
            Xf.p, nullptr);
    }
    BH_CUDA(cudaStreamSynchronize(st));

    const int nev = rq.nev;
    const double eps23 = std::pow(2.220446049250313e-16, 2.0 / 3.0);
    res.evals.assign((size_t)S * nev, 0.0);
    res.resid.assign((size_t)S * nev, 0.0);
    for (int s = 0; s < S; ++s) {
        for (int i = 0; i < nev; ++i) {
            const double e = th[(size_t)s * K + i];
            res.evals[(size_t)s * nev + i] = e;
            const double fl = std::max(eps23, 1e-3 * res.scale[s]);
            res.resid[(size_t)s * nev + i] =
                i < kref[s] ? std::sqrt(std::max(0.0, hrn[(size_t)s * K + i])) / std::max(std::fabs(e), fl) : nan;
        }
        res.nconv[s] = std::min(res.nconv[s], kref[s]);
    }
    profile_flush();
    if (rq.want_vectors) {
        std::vector<double> hx((size_t)D * nc2);
        BH_CUDA(cudaMemcpyAsync(hx.data(), Xf.p, hx.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaStreamSynchronize(st));
        res.vecs.assign((size_t)S * nev * D, 0.0);
        for (int64_t r = 0; r < D; ++r)
            for (int s = 0; s < S; ++s)
                for (int i = 0; i < nev; ++i)
                    res.vecs[((size_t)s * nev + i) * D + r] = hx[(size_t)r * nc2 + s * K + i];
    }
    return res;
}

}  // namespace bh

namespace bh {

// Op::FOLM_diag (operator.cpp:39-71) as its comments describe it: nb_iter
// Lanczos steps from v0 in FP64 with full re-orthogonalisation.  Step i forms
// w = O v_i, removes its components along every vector so far (v_i included)
// with two classical Gram-Schmidt passes, and sets T_ii = alpha_i (the v_i
// coefficients of both passes) and T_{i,i+1} = T_{i+1,i} = beta_i = |w|,
// v_{i+1} = w / beta_i; it stops after nb_iter vectors or once beta_i < 1e-6
// (the reference's threshold).  T is k x k (zeros beyond the steps taken), V
// column-major D x k.  Returns the number of vectors.  (The reference's loop
// leaves v_i out of the orthogonalisation and stores beta_i one row late;
// callers of the API get the tridiagonal matrix the method defines.)
int folm_diag(const OpView<double>& op, int k, const double* v0, double* T, double* V, cudaStream_t st) {
    const int64_t D = op.D;
    int64_t launches = 0;
    Launcher<double> L{op, st, &launches};
    const Geo g = make_geo(D, 1), gu = make_ugeo(D, 1);
    const int kcap = k + 1;
    DevBuf<double> Vd((size_t)k * D), W((size_t)D), prm(3), part((size_t)g.nchunks * kcap), C((size_t)kcap),
        Cf((size_t)kcap), rinv(1);
    const double hp[3] = {1.0, 0.0, 0.0};  // J, U, shift: the product is O itself
    BH_CUDA(cudaMemcpyAsync(prm.p, hp, sizeof hp, cudaMemcpyHostToDevice, st));
    BH_CUDA(cudaMemcpyAsync(Vd.p, v0, (size_t)D * sizeof(double), cudaMemcpyHostToDevice, st));
    std::fill(T, T + (size_t)k * k, 0.0);
    auto read = [&](const double* dsrc) {
        double h = 0.0;
        BH_CUDA(cudaMemcpyAsync(&h, dsrc, sizeof(double), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaStreamSynchronize(st));
        return h;
    };
    int steps = 0;
    for (int i = 0; i < k; ++i) {
        L.spmm(1, 1, prm.p, Vd.p + (int64_t)i * D, W.p);
        double alpha = 0.0;
        for (int pass = 0; pass < 2; ++pass) {
            L.dot(g, 1, 1, i + 1, D, Vd.p, W.p, kcap, part.p);
            L.dot_finalize(g, i + 1, 1, 1, kcap, part.p, C.p, Cf.p, nullptr, 0, 0);
            L.update(gu, 1, i + 1, D, Vd.p, Cf.p, W.p, 0, nullptr);
            alpha += read(C.p + i);
        }
        L.dot(g, 1, 1, 1, D, W.p, W.p, kcap, part.p);
        L.dot_finalize(g, 1, 1, 1, kcap, part.p, C.p, nullptr, nullptr, 0, 0);
        const double beta = std::sqrt(std::max(read(C.p), 0.0));
        T[(size_t)i * k + i] = alpha;
        steps = i + 1;
        if (i + 1 == k || !(beta >= 1e-6)) break;
        T[(size_t)i * k + i + 1] = beta;
        T[(size_t)(i + 1) * k + i] = beta;
        const double r = 1.0 / beta;
        BH_CUDA(cudaMemcpyAsync(rinv.p, &r, sizeof r, cudaMemcpyHostToDevice, st));
        L.normalize(1, 1, rinv.p, W.p, Vd.p + (int64_t)(i + 1) * D);
    }
    BH_CUDA(cudaMemcpyAsync(V, Vd.p, (size_t)steps * D * sizeof(double), cudaMemcpyDeviceToHost, st));
    BH_CUDA(cudaStreamSynchronize(st));
    std::fill(V + (size_t)steps * D, V + (size_t)k * D, 0.0);
    return steps;
}

}  // namespace bh
