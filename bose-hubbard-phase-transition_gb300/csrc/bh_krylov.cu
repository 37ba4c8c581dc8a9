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
// of X is a contiguous S p-vector.  Per step (block Lanczos with full
// re-orthogonalisation by classical Gram-Schmidt applied twice):
//     W = H V_j                                   k_spmm
//     C = [V_0..V_j]^T W,  W -= [V_0..V_j] C      k_dot + k_dot_finalize + k_update  (x2)
//     W = V_{j+1} R  (Cholesky QR of W^T W)       k_update(gram) + k_qr_finalize + k_normalize
// The projected matrix T (FP64) is filled on the device from C and R; the
// host reads it only at a restart, solves the small eigenproblems in FP64,
// and sends back the Ritz rotation applied by k_rotate (thick restart).
// Vectors are FP64 (plain method) or FP32 (mixed); the coefficients C, R and
// all reductions are FP64 (FP32 partial sums over at most 32 rows are folded
// into FP64 accumulators).  A final FP64 Rayleigh-Ritz on the Ritz vectors
// (FP64 SpMM, FP64 Gram matrices, FP64 generalised eigensolve) gives the
// returned eigenvalues and their true FP64 residuals.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <type_traits>

#include "bh_krylov.cuh"

namespace bh {

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// Y = H X for ncols columns; column t belongs to solve t / group with
// prm[3 s + 0..2] = (J, U, shift).  L lanes per row, lanes over columns.
template <class T, int L>
__global__ void __launch_bounds__(256)
k_spmm(OpView<T> A, int ncols, int group, const double* __restrict__ prm,
       const T* __restrict__ X, T* __restrict__ Y) {
    const int gl = threadIdx.x % L;
    const int rows_per_block = blockDim.x / L;
    const int cpl = ncols / L;
    for (int64_t r = (int64_t)blockIdx.x * rows_per_block + threadIdx.x / L; r < A.D;
         r += (int64_t)gridDim.x * rows_per_block) {
        const int64_t e0 = A.rp[r], e1 = A.rp[r + 1];
        const T d = A.vd ? A.vd[r] : T(0);
        for (int c0 = 0; c0 < cpl; c0 += 8) {
            T acc[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) acc[u] = T(0);
            const int nc = min(8, cpl - c0);
            for (int64_t e = e0; e < e1; ++e) {
                const int64_t col = A.ci[e];
                const T v = A.tv[e];
                const T* xr = X + col * ncols + gl + c0 * L;
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (u < nc) acc[u] += v * xr[u * L];
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (u < nc) {
                    const int t = gl + (c0 + u) * L;
                    const int s = t / group;
                    const T Jc = (T)prm[3 * s], Uc = (T)prm[3 * s + 1], sh = (T)prm[3 * s + 2];
                    const T xv = X[r * ncols + t];
                    Y[r * ncols + t] = Jc * acc[u] + (Uc * d + sh) * xv;
                }
            }
        }
    }
}

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

// C = sum over chunks; Cf = (T)C; optionally T_s[c][jcol p + q'] += C
template <class T>
__global__ void k_dot_finalize(int nchunks, int kc, int ncols, int ldC, int p, int kcap,
                               const double* __restrict__ part, double* __restrict__ C,
                               T* __restrict__ Cf, double* __restrict__ Tm, int Tdim, int jcol) {
    const int total = kc * ncols;
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
        const int c = idx / ncols, t = idx % ncols;
        double sum = 0.0;
        for (int ch = 0; ch < nchunks; ++ch) sum += part[((size_t)ch * kcap + c) * ncols + t];
        if (C) C[(size_t)c * ldC + t] = sum;
        if (Cf) Cf[(size_t)c * ldC + t] = (T)sum;
        if (Tm) {
            const int s = t / p, q = t % p;
            Tm[(size_t)s * Tdim * Tdim + (size_t)(jcol * p + q) * Tdim + c] += sum;
        }
    }
}

// W[r][s p + q'] -= sum_{c < kc} V_{c/p}[r][s p + c%p] Cf[c][s p + q'], then
// (optionally) Gram partials G_s[q][q'] = sum_r W[r][s p + q] W[r][s p + q'].
template <class T, int PMAX>
__global__ void __launch_bounds__(512)
k_update(int64_t D, int ncols, int p, int lp, int kc, int64_t bstride, const T* __restrict__ V,
         const T* __restrict__ Cf, T* __restrict__ W, int64_t rows_per_chunk, int do_gram,
         double* __restrict__ gpart) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    T* sC = reinterpret_cast<T*>(s_raw);
    double* sG = reinterpret_cast<double*>(s_raw + (((size_t)kc * ncols * sizeof(T) + 15) & ~(size_t)15));
    for (int i = threadIdx.x; i < kc * ncols; i += blockDim.x) sC[i] = Cf[i];
    __syncthreads();
    const int t = threadIdx.x % ncols, ro = threadIdx.x / ncols, R = blockDim.x / ncols;
    const int s = t / p, q = t % p;
    const int lane = threadIdx.x & 31;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t r1 = min(D, r0 + rows_per_chunk);
    double gd[PMAX];
    T gf[PMAX];
#pragma unroll
    for (int b = 0; b < PMAX; ++b) {
        gd[b] = 0.0;
        gf[b] = T(0);
    }
    int cnt = 0;
    for (int64_t base = r0; base < r1; base += R) {
        const int64_t r = base + ro;
        const bool valid = r < r1;
        T w = valid ? W[r * ncols + t] : T(0);
        if (valid && kc > 0) {
            const T* vr = V + r * ncols + s * p;
            T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
            int c = 0;
            for (; c + 3 < kc; c += 4) {
                a0 += vr[(int64_t)(c >> lp) * bstride + (c & (p - 1))] * sC[c * ncols + t];
                a1 += vr[(int64_t)((c + 1) >> lp) * bstride + ((c + 1) & (p - 1))] * sC[(c + 1) * ncols + t];
                a2 += vr[(int64_t)((c + 2) >> lp) * bstride + ((c + 2) & (p - 1))] * sC[(c + 2) * ncols + t];
                a3 += vr[(int64_t)((c + 3) >> lp) * bstride + ((c + 3) & (p - 1))] * sC[(c + 3) * ncols + t];
            }
            for (; c < kc; ++c) a0 += vr[(int64_t)(c >> lp) * bstride + (c & (p - 1))] * sC[c * ncols + t];
            w -= (a0 + a1) + (a2 + a3);
            W[r * ncols + t] = w;
        }
        if (do_gram) {
#pragma unroll
            for (int b = 0; b < PMAX; ++b) {
                if (b < p) {
                    const T wb = __shfl_sync(0xffffffffu, w, lane - q + b);
                    gf[b] += wb * w;
                }
            }
            if (++cnt == 32) {
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

// One thread per solve: G = sum of Gram partials, Cholesky G = R^T R (R upper
// triangular), Rinv = R^{-1}; T_s[(jrow p + a)][(jrow - 1) p + b] = R[a][b].
// A pivot below tiny^2 (relative to the solve's scale) is a breakdown: the
// direction is dropped (zero column of Rinv) and brk[s] records jrow.
__global__ void k_qr_finalize(int S, int p, int nchunks, int ncols, const double* __restrict__ gpart,
                              double* __restrict__ Rinv, double* __restrict__ Tm, int Tdim,
                              int jrow, const double* __restrict__ scale, double rel_tiny,
                              int* __restrict__ brk) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    double G[16][16], R[16][16], Ri[16][16];
    for (int a = 0; a < p; ++a)
        for (int b = 0; b < p; ++b) {
            double sum = 0.0;
            for (int ch = 0; ch < nchunks; ++ch) sum += gpart[((size_t)ch * p + a) * ncols + s * p + b];
            G[a][b] = sum;
            R[a][b] = 0.0;
            Ri[a][b] = 0.0;
        }
    const double sc = scale ? scale[s] : 1.0;
    const double tiny = rel_tiny * (sc > 0.0 ? sc : 1.0);
    bool broke = false;
    for (int i = 0; i < p; ++i) {
        double d = 0.5 * (G[i][i] + G[i][i]);
        for (int k = 0; k < i; ++k) d -= R[k][i] * R[k][i];
        if (!(d > tiny * tiny)) {
            broke = true;
            R[i][i] = 0.0;
            for (int j = i + 1; j < p; ++j) R[i][j] = 0.0;
            continue;
        }
        const double rii = sqrt(d);
        R[i][i] = rii;
        for (int j = i + 1; j < p; ++j) {
            double v = 0.5 * (G[i][j] + G[j][i]);
            for (int k = 0; k < i; ++k) v -= R[k][i] * R[k][j];
            R[i][j] = v / rii;
        }
    }
    // inverse of the upper-triangular R (dropped directions stay zero)
    for (int j = 0; j < p; ++j) {
        if (R[j][j] == 0.0) continue;
        Ri[j][j] = 1.0 / R[j][j];
        for (int i = j - 1; i >= 0; --i) {
            if (R[i][i] == 0.0) continue;
            double v = 0.0;
            for (int k = i + 1; k <= j; ++k) v += R[i][k] * Ri[k][j];
            Ri[i][j] = -v / R[i][i];
        }
    }
    for (int a = 0; a < p; ++a)
        for (int b = 0; b < p; ++b) Rinv[(size_t)s * p * p + a * p + b] = Ri[a][b];
    if (Tm && jrow > 0) {
        double* Ts = Tm + (size_t)s * Tdim * Tdim;
        for (int a = 0; a < p; ++a)
            for (int b = 0; b < p; ++b) Ts[(size_t)((jrow - 1) * p + b) * Tdim + jrow * p + a] = R[a][b];
    }
    if (broke && brk && brk[s] < 0) brk[s] = jrow;
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

// Thick-restart rotation: out_s[:, i] = sum_{c < kc} V_s[:, c] Y_s[c][i], i < nout.
// Input column c of solve s is V_{c/p}[r][s p + c%p].  Output layout: blocks of
// p columns (Vout[i/p][r][s p + i%p], stride ostride) or, when out_cols > 0, one
// row-major block Vout[r][s nout + i] with out_cols = S nout columns.
template <class T>
__global__ void __launch_bounds__(256)
k_rotate(int64_t D, int S, int ncols, int p, int kc, int nout, int64_t bstride,
         const T* __restrict__ V, const T* __restrict__ Yg, T* __restrict__ Vout, int64_t ostride,
         int out_cols, int Sg, int64_t rows_per_chunk) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    T* sY = reinterpret_cast<T*>(s_raw);
    const int sg0 = blockIdx.y * Sg;
    const int nsg = min(Sg, S - sg0);
    for (int i = threadIdx.x; i < nsg * kc * nout; i += blockDim.x) sY[i] = Yg[(size_t)sg0 * kc * nout + i];
    __syncthreads();
    const int width = Sg * p;
    const int tl = threadIdx.x % width, ro = threadIdx.x / width, R = blockDim.x / width;
    const int ls = tl / p, qo = tl % p;
    if (ls >= nsg) return;
    const int s = sg0 + ls;
    const int nob = nout / p;
    const int64_t r0 = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t r1 = min(D, r0 + rows_per_chunk);
    const T* ys = sY + (size_t)ls * kc * nout;
    for (int64_t r = r0 + ro; r < r1; r += R) {
        for (int jo0 = 0; jo0 < nob; jo0 += 8) {
            T acc[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) acc[u] = T(0);
            for (int j = 0; j < kc / p; ++j) {
                const T* vr = V + (int64_t)j * bstride + r * ncols + s * p;
                for (int q = 0; q < p; ++q) {
                    const T v = vr[q];
                    const T* yrow = ys + (size_t)(j * p + q) * nout + qo;
#pragma unroll
                    for (int u = 0; u < 8; ++u)
                        if (jo0 + u < nob) acc[u] += v * yrow[(jo0 + u) * p];
                }
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (jo0 + u < nob) {
                    const int i = (jo0 + u) * p + qo;
                    if (out_cols > 0)
                        Vout[r * out_cols + (int64_t)s * nout + i] = acc[u];
                    else
                        Vout[(int64_t)(jo0 + u) * ostride + r * ncols + s * p + qo] = acc[u];
                }
            }
        }
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

// ||(Y - theta_i X) z_i||^2 partials for column t = s K + i (FP64)
__global__ void __launch_bounds__(512)
k_resid(int64_t D, int ncols, int ld, int K, const double* __restrict__ X, const double* __restrict__ Y,
        const double* __restrict__ theta, const double* __restrict__ Z, int64_t rows_per_chunk,
        double* __restrict__ part) {
    extern __shared__ double s_red2[];
    const int t = threadIdx.x % ncols, ro = threadIdx.x / ncols, R = blockDim.x / ncols;
    const int s = t / K, i = t % K;
    const double th = theta[t];
    const double* z = Z + (size_t)s * K * K;  // z[a * K + i]
    const int64_t r0 = (int64_t)blockIdx.x * rows_per_chunk;
    const int64_t r1 = min(D, r0 + rows_per_chunk);
    double acc = 0.0;
    for (int64_t r = r0 + ro; r < r1; r += R) {
        const double* xr = X + r * ld + s * K;
        const double* yr = Y + r * ld + s * K;
        double v = 0.0;
        for (int a = 0; a < K; ++a) v += (yr[a] - th * xr[a]) * __ldg(z + a * K + i);
        acc += v * v;
    }
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

int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return 132;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 132;
    }
    return n;
}

static int max_smem_optin() {
    static int v = 0;
    if (v == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0)
            v = 48 * 1024;
    }
    return v;
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

// geometry of the row-chunked reductions
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

    void spmm(int ncols, int group, const double* prm, const T* X, T* Y) const {
        const int64_t D = op.D;
        int L = 1;
        while (L < 32 && L * 2 <= ncols && ncols % (L * 2) == 0) L *= 2;
        const int rpb = 256 / L;
        int64_t g = (D + rpb - 1) / rpb;
        g = std::min<int64_t>(g, (int64_t)sm_count() * 16);
        g = std::max<int64_t>(g, 1);
        switch (L) {
            case 1: k_spmm<T, 1><<<(unsigned)g, 256, 0, st>>>(op, ncols, group, prm, X, Y); break;
            case 2: k_spmm<T, 2><<<(unsigned)g, 256, 0, st>>>(op, ncols, group, prm, X, Y); break;
            case 4: k_spmm<T, 4><<<(unsigned)g, 256, 0, st>>>(op, ncols, group, prm, X, Y); break;
            case 8: k_spmm<T, 8><<<(unsigned)g, 256, 0, st>>>(op, ncols, group, prm, X, Y); break;
            case 16: k_spmm<T, 16><<<(unsigned)g, 256, 0, st>>>(op, ncols, group, prm, X, Y); break;
            default: k_spmm<T, 32><<<(unsigned)g, 256, 0, st>>>(op, ncols, group, prm, X, Y); break;
        }
        BH_CUDA(cudaGetLastError());
        ++*launches;
    }

    template <int PMAX>
    void dot_t(const Geo& g, int ld, int p, int nblk, int64_t bstride, const T* V, const T* W, int kcap,
               double* part) const {
        constexpr int JT = PMAX >= 16 ? 1 : 16 / PMAX;
        dim3 grid(g.nchunks, (nblk + JT - 1) / JT);
        const size_t smem = (size_t)g.NT * JT * PMAX * sizeof(double);
        auto kern = k_dot<T, PMAX, JT>;
        if (smem > 48 * 1024) BH_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<grid, g.NT, smem, st>>>(op.D, g.ncols, ld, p, nblk, bstride, V, W, g.rows_per_chunk, kcap, part);
        BH_CUDA(cudaGetLastError());
        ++*launches;
    }
    void dot(const Geo& g, int ld, int p, int nblk, int64_t bstride, const T* V, const T* W,
             int kcap, double* part) const {
        if (p <= 1) dot_t<1>(g, ld, p, nblk, bstride, V, W, kcap, part);
        else if (p <= 2) dot_t<2>(g, ld, p, nblk, bstride, V, W, kcap, part);
        else if (p <= 4) dot_t<4>(g, ld, p, nblk, bstride, V, W, kcap, part);
        else if (p <= 8) dot_t<8>(g, ld, p, nblk, bstride, V, W, kcap, part);
        else if (p <= 16) dot_t<16>(g, ld, p, nblk, bstride, V, W, kcap, part);
        else dot_t<32>(g, ld, p, nblk, bstride, V, W, kcap, part);
    }
    void dot_finalize(const Geo& g, int kc, int ldC, int p, int kcap, const double* part, double* C,
                      T* Cf, double* Tm, int Tdim, int jcol) const {
        k_dot_finalize<T><<<elem_grid((int64_t)kc * g.ncols), 256, 0, st>>>(
            g.nchunks, kc, g.ncols, ldC, p, kcap, part, C, Cf, Tm, Tdim, jcol);
        BH_CUDA(cudaGetLastError());
        ++*launches;
    }
    template <int PMAX>
    void update_t(const Geo& g, int p, int kc, int64_t bstride, const T* V, const T* Cf, T* W,
                  int do_gram, double* gpart) const {
        const size_t smem = (((size_t)kc * g.ncols * sizeof(T) + 15) & ~(size_t)15) +
                            (size_t)g.NT * PMAX * sizeof(double);
        if ((int)smem > max_smem_optin()) throw Error(BH_ERR_ARG, "Krylov basis too wide for shared memory (reduce ncv or batch)");
        auto kern = k_update<T, PMAX>;
        if (smem > 48 * 1024) BH_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<g.nchunks, g.NT, smem, st>>>(op.D, g.ncols, p, ilog2(p), kc, bstride, V, Cf, W,
                                            g.rows_per_chunk, do_gram, gpart);
        BH_CUDA(cudaGetLastError());
        ++*launches;
    }
    void update(const Geo& g, int p, int kc, int64_t bstride, const T* V, const T* Cf, T* W,
                int do_gram, double* gpart) const {
        if (p <= 1) update_t<1>(g, p, kc, bstride, V, Cf, W, do_gram, gpart);
        else if (p <= 2) update_t<2>(g, p, kc, bstride, V, Cf, W, do_gram, gpart);
        else if (p <= 4) update_t<4>(g, p, kc, bstride, V, Cf, W, do_gram, gpart);
        else if (p <= 8) update_t<8>(g, p, kc, bstride, V, Cf, W, do_gram, gpart);
        else update_t<16>(g, p, kc, bstride, V, Cf, W, do_gram, gpart);
    }
    void qr(const Geo& g, int S, int p, const double* gpart, double* Rinv, double* Tm, int Tdim,
            int jrow, const double* scale, double rel_tiny, int* brk) const {
        k_qr_finalize<<<(S + 63) / 64, 64, 0, st>>>(S, p, g.nchunks, g.ncols, gpart, Rinv, Tm, Tdim,
                                                   jrow, scale, rel_tiny, brk);
        BH_CUDA(cudaGetLastError());
        ++*launches;
    }
    void normalize(int ncols, int p, const double* Rinv, const T* W, T* Vout) const {
        k_normalize<T><<<elem_grid(op.D * ncols), 256, 0, st>>>(op.D, ncols, p, Rinv, W, Vout);
        BH_CUDA(cudaGetLastError());
        ++*launches;
    }
    void rotate(int S, int ncols, int p, int kc, int nout, int64_t bstride, const T* V,
                const T* Yg, T* Vout, int64_t ostride, int out_cols) const {
        const int smax = max_smem_optin();
        const size_t per = (size_t)kc * nout * sizeof(T);
        if ((int)per > smax) throw Error(BH_ERR_ARG, "restart rotation too large for shared memory (reduce ncv)");
        int Sg = (int)std::min<size_t>((size_t)S, std::max<size_t>(1, (size_t)(48 * 1024) / per));
        Sg = std::min(Sg, std::max(1, 256 / p));
        while (Sg > 1 && 256 % (Sg * p) != 0) --Sg;
        const size_t smem = (size_t)Sg * per;
        const int width = Sg * p;
        const int NT = 256 / width * width;
        const int64_t target = 2LL * sm_count();
        const int ngroups = (S + Sg - 1) / Sg;
        int64_t chunks = std::max<int64_t>(1, target / ngroups);
        int64_t rpc = (op.D + chunks - 1) / chunks;
        rpc = std::max<int64_t>(rpc, 1);
        chunks = (op.D + rpc - 1) / rpc;
        auto kern = k_rotate<T>;
        if (smem > 48 * 1024) BH_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<dim3((unsigned)std::max<int64_t>(chunks, 1), ngroups), NT, smem, st>>>(
            op.D, S, ncols, p, kc, nout, bstride, V, Yg, Vout, ostride, out_cols, Sg, rpc);
        BH_CUDA(cudaGetLastError());
        ++*launches;
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

// ---------------------------------------------------------------------------
// the solver
// ---------------------------------------------------------------------------

template <class T>
static void lanczos_phase(const OpView<T>& op, const SolveRequest& rq, const double* d_prm,
                          const double* d_scale_init, cudaStream_t st, SolveResult& res,
                          int K, DevBuf<T>& Xout, std::vector<double>& theta_out) {
    const int64_t D = op.D;
    const int S = rq.S, p = rq.p, ncols = S * p;
    const int kmax = rq.kmax, nb = kmax / p, Tdim = kmax + p;
    const int64_t bstride = D * (int64_t)ncols;
    Launcher<T> L{op, st, &res.launches};
    const Geo g = make_geo(D, ncols);
    const int kcap = std::max(Tdim, K);

    DevBuf<T> Va((size_t)(nb + 1) * bstride), Vb((size_t)(nb + 1) * bstride), W((size_t)bstride);
    DevBuf<double> part((size_t)g.nchunks * kcap * ncols), gpart((size_t)g.nchunks * p * ncols);
    DevBuf<T> Cf((size_t)kcap * ncols);
    DevBuf<double> Rinv((size_t)S * p * p), Tm((size_t)S * Tdim * Tdim), scale(S);
    DevBuf<int> brk(S);
    DevBuf<T> Yd((size_t)S * kmax * kmax);
    BH_CUDA(cudaMemcpyAsync(scale.p, d_scale_init, S * sizeof(double), cudaMemcpyDeviceToDevice, st));
    BH_CUDA(cudaMemsetAsync(Tm.p, 0, Tm.bytes(), st));
    std::vector<int> hbrk(S, -1);
    BH_CUDA(cudaMemcpyAsync(brk.p, hbrk.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
    const double eps_t = std::is_same<T, float>::value ? 1.1920929e-7 : 2.220446049250313e-16;
    const double rel_tiny = 1e3 * eps_t;

    // start block: W = seeded stream; V_1 = H W (Spectra forces v into range(A)); V_0 = QR(V_1)
    k_start_block<T><<<elem_grid(bstride), 256, 0, st>>>(D, ncols, p, rq.seed, rq.d_perm, W.p);
    BH_CUDA(cudaGetLastError());
    ++res.launches;
    T* V1 = Va.p + bstride;
    L.spmm(ncols, p, d_prm, W.p, V1);
    res.matvecs += p;
    L.update(g, p, 0, bstride, Va.p, Cf.p, V1, 1, gpart.p);
    L.qr(g, S, p, gpart.p, Rinv.p, nullptr, Tdim, 0, nullptr, 0.0, nullptr);
    L.normalize(ncols, p, Rinv.p, V1, Va.p);

    std::vector<double> hT((size_t)S * Tdim * Tdim);
    std::vector<double> theta((size_t)S * kmax), Yh((size_t)S * kmax * kmax), resid((size_t)S * kmax);
    std::vector<int> kuse(S, kmax);
    std::vector<T> Yt;
    res.conv_at.assign(S, -1);
    res.scale.assign(S, 1.0);
    int jstart = 0;
    int restarts = 0;
    const double eps23 = std::pow(2.220446049250313e-16, 2.0 / 3.0);
    for (;;) {
        for (int j = jstart; j < nb; ++j) {
            T* Vj = Va.p + (int64_t)j * bstride;
            L.spmm(ncols, p, d_prm, Vj, W.p);
            res.matvecs += p;
            const int kc = (j + 1) * p;
            for (int pass = 0; pass < 2; ++pass) {
                L.dot(g, ncols, p, j + 1, bstride, Va.p, W.p, kcap, part.p);
                L.dot_finalize(g, kc, ncols, p, kcap, part.p, nullptr, Cf.p, Tm.p, Tdim, j);
                L.update(g, p, kc, bstride, Va.p, Cf.p, W.p, pass == 1, gpart.p);
            }
            L.qr(g, S, p, gpart.p, Rinv.p, Tm.p, Tdim, j + 1, scale.p, rel_tiny, brk.p);
            L.normalize(ncols, p, Rinv.p, W.p, Va.p + (int64_t)(j + 1) * bstride);
        }
        BH_CUDA(cudaMemcpyAsync(hT.data(), Tm.p, hT.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaMemcpyAsync(hbrk.data(), brk.p, S * sizeof(int), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaStreamSynchronize(st));

        // Rayleigh-Ritz per solve (host, FP64)
        std::vector<int> nconv(S, 0);
        std::vector<double> hscale(S, 1.0);
        bool symeig_failed = false;
        parallel_for(S, [&](int s) {
            const double* Ts = hT.data() + (size_t)s * Tdim * Tdim;
            int k = kmax;
            if (hbrk[s] >= 0) k = std::min(k, hbrk[s] * p);
            kuse[s] = k;
            std::vector<double> a((size_t)k * k), w(k);
            for (int jj = 0; jj < k; ++jj)
                for (int ii = 0; ii < k; ++ii) {
                    const int lo = std::min(ii, jj), hi = std::max(ii, jj);
                    a[(size_t)jj * k + ii] = Ts[(size_t)hi * Tdim + lo];  // upper triangle
                }
            if (!symeig(k, a.data(), w.data())) symeig_failed = true;
            double sc = 0.0;
            for (int i = 0; i < k; ++i) sc = std::max(sc, std::fabs(w[i]));
            hscale[s] = std::max(sc, 1e-300);
            for (int i = 0; i < k; ++i) {
                theta[(size_t)s * kmax + i] = w[i];
                for (int c = 0; c < k; ++c) Yh[((size_t)s * kmax + c) * kmax + i] = a[(size_t)i * k + c];
                double r2 = 0.0;
                if (k == kmax && hbrk[s] < 0) {
                    for (int a2 = 0; a2 < p; ++a2) {
                        double v = 0.0;
                        for (int b2 = 0; b2 < p; ++b2)
                            v += Ts[(size_t)(kmax - p + b2) * Tdim + kmax + a2] * a[(size_t)i * k + kmax - p + b2];
                        r2 += v * v;
                    }
                }
                resid[(size_t)s * kmax + i] = std::sqrt(r2);
            }
            // Convergence: resid <= tol * max(|theta|, floor).  Spectra uses
            // floor = eps^(2/3); a residual estimate built from the computed
            // projection cannot fall below ~eps * ||H||, so the floor here is a
            // fraction of the spectral radius estimate (largest |Ritz value|).
            int nc = 0;
            const double floor_abs = rq.precision == BH_PREC_MIXED ? hscale[s] : std::max(eps23, 1e-3 * hscale[s]);
            for (int i = 0; i < std::min(rq.nev, k); ++i) {
                const double th = std::fabs(w[i]);
                if (resid[(size_t)s * kmax + i] <= rq.tol * std::max(th, floor_abs)) ++nc;
            }
            nconv[s] = nc;
        });
        if (symeig_failed) throw Error(BH_ERR_NOCONV, "projected eigenproblem did not converge");
        res.scale = hscale;
        bool done = true;
        int minconv = rq.nev, nact = 0;
        for (int s = 0; s < S; ++s) {
            if (kuse[s] < rq.nev) throw Error(BH_ERR_BREAKDOWN, "Krylov space exhausted before nev eigenvalues (dimension too small or invariant start block)");
            const bool conv_s = nconv[s] >= rq.nev || hbrk[s] >= 0;
            if (!conv_s) {
                done = false;
                ++nact;
            }
            if (conv_s && res.conv_at[s] < 0) res.conv_at[s] = restarts;
            minconv = std::min(minconv, nconv[s]);
        }
        res.nconv.assign(nconv.begin(), nconv.end());
        if (verbose()) {
            double worst = 0.0;
            for (int s = 0; s < S; ++s)
                for (int i = 0; i < rq.nev && i < kuse[s]; ++i) {
                    const double floor_abs = rq.precision == BH_PREC_MIXED ? hscale[s] : std::max(eps23, 1e-3 * hscale[s]);
                    worst = std::max(worst, resid[(size_t)s * kmax + i] / std::max(std::fabs(theta[(size_t)s * kmax + i]), floor_abs));
                }
            std::fprintf(stderr, "[bh] restart %d: unconverged solves %d/%d, min nconv %d, worst rel resid %.3e\n",
                         restarts, nact, S, minconv, worst);
        }
        if (done || restarts >= rq.max_restarts) break;

        // thick restart: keep the nkeep lowest Ritz vectors + the residual block
        int nkeep = rq.nev + std::max(p, (kmax - rq.nev) / 2);
        nkeep = (nkeep + p - 1) / p * p;
        nkeep = std::min(nkeep, kmax - 2 * p);
        if (nkeep < p) nkeep = p;
        Yt.assign((size_t)S * kmax * nkeep, T(0));
        for (int s = 0; s < S; ++s)
            for (int c = 0; c < kmax; ++c)
                for (int i = 0; i < nkeep; ++i)
                    Yt[((size_t)s * kmax + c) * nkeep + i] = (T)Yh[((size_t)s * kmax + c) * kmax + i];
        BH_CUDA(cudaMemcpyAsync(Yd.p, Yt.data(), Yt.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        L.rotate(S, ncols, p, kmax, nkeep, bstride, Va.p, Yd.p, Vb.p, bstride, 0);
        BH_CUDA(cudaMemcpyAsync(Vb.p + (int64_t)(nkeep / p) * bstride, Va.p + (int64_t)nb * bstride,
                                bstride * sizeof(T), cudaMemcpyDeviceToDevice, st));
        std::swap(Va.p, Vb.p);  // equal sizes: ownership stays balanced
        // new projected matrix: diag(theta_keep) plus the coupling rows
        //   T[nkeep + a][i] = sum_b R_last[a][b] Y[kmax - p + b][i]
        // (the upper arrowhead is recomputed by the next expansion step)
        std::vector<double> hTn(hT.size(), 0.0);
        for (int s = 0; s < S; ++s) {
            const double* To = hT.data() + (size_t)s * Tdim * Tdim;
            double* Ts = hTn.data() + (size_t)s * Tdim * Tdim;
            for (int i = 0; i < nkeep; ++i) Ts[(size_t)i * Tdim + i] = theta[(size_t)s * kmax + i];
            for (int a = 0; a < p; ++a)
                for (int i = 0; i < nkeep; ++i) {
                    double v = 0.0;
                    for (int b = 0; b < p; ++b)
                        v += To[(size_t)(kmax - p + b) * Tdim + kmax + a] *
                             Yh[((size_t)s * kmax + kmax - p + b) * kmax + i];
                    Ts[(size_t)i * Tdim + nkeep + a] = v;
                }
        }
        hT.swap(hTn);
        BH_CUDA(cudaMemcpyAsync(Tm.p, hT.data(), hT.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaMemcpyAsync(scale.p, hscale.data(), S * sizeof(double), cudaMemcpyHostToDevice, st));
        jstart = nkeep / p;
        ++restarts;
    }
    res.restarts = restarts;

    // Ritz vectors of the K lowest values: X[r][s K + i]
    Yt.assign((size_t)S * kmax * K, T(0));
    theta_out.assign((size_t)S * K, 0.0);
    for (int s = 0; s < S; ++s) {
        const int k = kuse[s];
        for (int i = 0; i < K; ++i) {
            theta_out[(size_t)s * K + i] = i < k ? theta[(size_t)s * kmax + i] : 0.0;
            for (int c = 0; c < k; ++c)
                Yt[((size_t)s * kmax + c) * K + i] = i < k ? (T)Yh[((size_t)s * kmax + c) * kmax + i] : T(0);
        }
    }
    BH_CUDA(cudaMemcpyAsync(Yd.p, Yt.data(), Yt.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    Xout.alloc((size_t)D * S * K);
    L.rotate(S, ncols, p, kmax, K, bstride, Va.p, Yd.p, Xout.p, 0, S * K);
    BH_CUDA(cudaStreamSynchronize(st));
    // Va/Vb swapped raw pointers above: keep ownership consistent
}

void apply_operator(const OpView<double>& op, int ncols, int group, const double* d_prm,
                    const double* d_X, double* d_Y, cudaStream_t st) {
    int64_t launches = 0;
    Launcher<double> L{op, st, &launches};
    L.spmm(ncols, group, d_prm, d_X, d_Y);
}

SolveResult block_lanczos(const OpView<double>& op64, const OpView<float>& op32,
                          const SolveRequest& rq, cudaStream_t st) {
    SolveResult res;
    const int S = rq.S, p = rq.p;
    const int64_t D = op64.D;
    BH_REQUIRE(S >= 1 && p >= 1 && p <= 16 && (p & (p - 1)) == 0, "block size must be 1, 2, 4, 8 or 16");
    BH_REQUIRE(rq.nev >= 1 && rq.nev <= 32, "nev must be in [1, 32]");
    BH_REQUIRE((int64_t)S * p <= 512, "batch too wide: S * block must be <= 512");
    BH_REQUIRE(rq.kmax % p == 0 && rq.kmax >= rq.nev + p, "ncv must be a multiple of the block size and >= nev + block");
    BH_REQUIRE((int64_t)rq.kmax <= D, "ncv exceeds the dimension");
    const int K = (rq.nev + p - 1) / p * p;  // Ritz vectors refined in FP64
    BH_REQUIRE(K <= 32 && K <= rq.kmax, "too many wanted eigenvalues for this block size");

    // per-solve parameters (J, U, shift) and start scale
    std::vector<double> prm((size_t)3 * S), sc(S, 1.0);
    for (int s = 0; s < S; ++s) {
        prm[3 * s] = rq.J[s];
        prm[3 * s + 1] = rq.U[s];
        prm[3 * s + 2] = rq.shift[s];
        sc[s] = std::fabs(rq.J[s]) + std::fabs(rq.U[s]) + std::fabs(rq.shift[s]) + 1e-300;
    }
    DevBuf<double> d_prm(prm.size()), d_sc(S);
    BH_CUDA(cudaMemcpyAsync(d_prm.p, prm.data(), prm.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    BH_CUDA(cudaMemcpyAsync(d_sc.p, sc.data(), S * sizeof(double), cudaMemcpyHostToDevice, st));

    // ---- Lanczos phase ----
    DevBuf<double> X64;
    std::vector<double> theta0;
    if (rq.precision == BH_PREC_MIXED) {
        BH_REQUIRE(op32.tv != nullptr, "mixed precision needs FP32 operator values");
        DevBuf<float> X32;
        lanczos_phase<float>(op32, rq, d_prm.p, d_sc.p, st, res, K, X32, theta0);
        X64.alloc((size_t)D * S * K);
        k_convert<float, double><<<elem_grid(D * S * K), 256, 0, st>>>(D * S * K, X32.p, X64.p);
        BH_CUDA(cudaGetLastError());
        ++res.launches;
        BH_CUDA(cudaStreamSynchronize(st));
    } else {
        lanczos_phase<double>(op64, rq, d_prm.p, d_sc.p, st, res, K, X64, theta0);
    }

    // ---- FP64 Rayleigh-Ritz refinement on the K Ritz vectors per solve ----
    const int nc2 = S * K;
    Launcher<double> L{op64, st, &res.launches};
    DevBuf<double> Y64((size_t)D * nc2);
    L.spmm(nc2, K, d_prm.p, X64.p, Y64.p);
    res.matvecs += K;
    // Gram matrices per solve, in groups of at most 512 columns
    const int sgrp = std::max(1, std::min(S, 512 / K));
    const Geo gmax = make_geo(D, sgrp * K);
    DevBuf<double> part((size_t)gmax.nchunks * K * sgrp * K), Gd((size_t)K * nc2), Ad((size_t)K * nc2);
    for (int s0 = 0; s0 < S; s0 += sgrp) {
        const int ns = std::min(sgrp, S - s0);
        const Geo gg = make_geo(D, ns * K);
        const int64_t off = (int64_t)s0 * K;
        L.dot(gg, nc2, K, 1, 0, X64.p + off, X64.p + off, K, part.p);
        L.dot_finalize(gg, K, nc2, K, K, part.p, Gd.p + off, nullptr, nullptr, 0, 0);
        L.dot(gg, nc2, K, 1, 0, X64.p + off, Y64.p + off, K, part.p);
        L.dot_finalize(gg, K, nc2, K, K, part.p, Ad.p + off, nullptr, nullptr, 0, 0);
    }
    std::vector<double> hG((size_t)K * nc2), hA((size_t)K * nc2);
    BH_CUDA(cudaMemcpyAsync(hG.data(), Gd.p, hG.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    BH_CUDA(cudaMemcpyAsync(hA.data(), Ad.p, hA.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    BH_CUDA(cudaStreamSynchronize(st));
    std::vector<double> th((size_t)nc2), Z((size_t)S * K * K);
    bool fail = false;
    parallel_for(S, [&](int s) {
        // G_s[a][b] is at hG[a * nc2 + s K + b]
        std::vector<double> Gm((size_t)K * K), Am((size_t)K * K);
        for (int a = 0; a < K; ++a)
            for (int b = 0; b < K; ++b) {
                Gm[(size_t)b * K + a] = 0.5 * (hG[(size_t)a * nc2 + s * K + b] + hG[(size_t)b * nc2 + s * K + a]);
                Am[(size_t)b * K + a] = 0.5 * (hA[(size_t)a * nc2 + s * K + b] + hA[(size_t)b * nc2 + s * K + a]);
            }
        if (!cholesky_lower(K, Gm)) {
            fail = true;
            return;
        }
        // M = L^{-1} A L^{-T}
        auto Lv = [&](int i, int j) { return Gm[(size_t)j * K + i]; };
        std::vector<double> B(Am);  // solve L B = A (column by column)
        for (int c = 0; c < K; ++c)
            for (int i = 0; i < K; ++i) {
                double v = B[(size_t)c * K + i];
                for (int k = 0; k < i; ++k) v -= Lv(i, k) * B[(size_t)c * K + k];
                B[(size_t)c * K + i] = v / Lv(i, i);
            }
        std::vector<double> M((size_t)K * K);  // M = B L^{-T}: solve M L^T = B  -> rows
        for (int r = 0; r < K; ++r)
            for (int j = 0; j < K; ++j) {
                double v = B[(size_t)j * K + r];
                for (int k = 0; k < j; ++k) v -= M[(size_t)k * K + r] * Lv(j, k);
                M[(size_t)j * K + r] = v / Lv(j, j);
            }
        for (int a = 0; a < K; ++a)
            for (int b = a + 1; b < K; ++b) {
                const double v = 0.5 * (M[(size_t)b * K + a] + M[(size_t)a * K + b]);
                M[(size_t)b * K + a] = M[(size_t)a * K + b] = v;
            }
        std::vector<double> w(K);
        if (!symeig(K, M.data(), w.data())) {
            fail = true;
            return;
        }
        // z = L^{-T} u
        for (int i = 0; i < K; ++i) {
            th[(size_t)s * K + i] = w[i];
            for (int a = K - 1; a >= 0; --a) {
                double v = M[(size_t)i * K + a];
                for (int k = a + 1; k < K; ++k) v -= Lv(k, a) * Z[((size_t)s * K + k) * K + i];
                Z[((size_t)s * K + a) * K + i] = v / Lv(a, a);
            }
        }
    });
    if (fail) throw Error(BH_ERR_NOCONV, "final Rayleigh-Ritz failed (Ritz vectors not independent)");
    DevBuf<double> d_th(nc2), d_Z(Z.size()), rpart((size_t)gmax.nchunks * sgrp * K), rn(nc2);
    BH_CUDA(cudaMemcpyAsync(d_th.p, th.data(), nc2 * sizeof(double), cudaMemcpyHostToDevice, st));
    BH_CUDA(cudaMemcpyAsync(d_Z.p, Z.data(), Z.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    for (int s0 = 0; s0 < S; s0 += sgrp) {
        const int ns = std::min(sgrp, S - s0);
        const Geo gg = make_geo(D, ns * K);
        const int64_t off = (int64_t)s0 * K;
        k_resid<<<gg.nchunks, gg.NT, gg.NT * sizeof(double), st>>>(
            D, ns * K, nc2, K, X64.p + off, Y64.p + off, d_th.p + off, d_Z.p + off * K,
            gg.rows_per_chunk, rpart.p);
        BH_CUDA(cudaGetLastError());
        k_sum_cols<<<(ns * K + 255) / 256, 256, 0, st>>>(gg.nchunks, ns * K, rpart.p, rn.p + off);
        BH_CUDA(cudaGetLastError());
        res.launches += 2;
    }
    std::vector<double> hrn(nc2);
    BH_CUDA(cudaMemcpyAsync(hrn.data(), rn.p, nc2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    DevBuf<double> Xf;
    if (rq.want_vectors) {
        Xf.alloc((size_t)D * nc2);
        L.rotate(S, nc2, K, K, K, 0, X64.p, d_Z.p, Xf.p, 0, nc2);
    }
    BH_CUDA(cudaStreamSynchronize(st));

    const int nev = rq.nev;
    const double eps23 = std::pow(2.220446049250313e-16, 2.0 / 3.0);
    res.evals.assign((size_t)S * nev, 0.0);
    res.resid.assign((size_t)S * nev, 0.0);
    for (int s = 0; s < S; ++s)
        for (int i = 0; i < nev; ++i) {
            const double e = th[(size_t)s * K + i];
            res.evals[(size_t)s * nev + i] = e;
            const double fl = std::max(eps23, 1e-3 * res.scale[s]);
            res.resid[(size_t)s * nev + i] = std::sqrt(std::max(0.0, hrn[(size_t)s * K + i])) / std::max(std::fabs(e), fl);
        }
    if (rq.want_vectors) {
        std::vector<double> hx((size_t)D * nc2);
        BH_CUDA(cudaMemcpy(hx.data(), Xf.p, hx.size() * sizeof(double), cudaMemcpyDeviceToHost));
        res.vecs.assign((size_t)S * nev * D, 0.0);
        for (int64_t r = 0; r < D; ++r)
            for (int s = 0; s < S; ++s)
                for (int i = 0; i < nev; ++i)
                    res.vecs[((size_t)s * nev + i) * D + r] = hx[(size_t)r * nc2 + s * K + i];
    }
    return res;
}

}  // namespace bh
