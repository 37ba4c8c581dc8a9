// bh_basis.cu -- fixed-n Fock basis on the device.
//
// Replaces BH::init_lexicographic / calculate_tags / sort_basis /
// fixed_set_basis (src/hamiltonian.cpp:60-149).  Instead of materialising the
// m x D double matrix and a floating-point tag search, a state is its
// lexicographic index r; occupations are regenerated from r by combinadic
// unranking, and the reference's column order (argsort of the states by the
// prime-product tag, then the inverse permutation of the cycle loop in
// sort_basis) comes from an exact 128-bit key P = prod p_i^{n_i} sorted by a
// stable LSD radix sort written here.  The tag logarithm is order-equivalent
// to P, so the order is bit-exact without floating point.
#include <cmath>

#include "bh_internal.h"
#include "bh_device.cuh"

namespace bh {

__constant__ unsigned kPrimes[kMaxSites] = {2,  3,  5,  7,  11, 13, 17, 19, 23, 29, 31, 37, 41,
                                            43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89, 97};

int64_t binomial64(int n, int k) {
    if (k < 0 || n < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    unsigned __int128 r = 1;
    for (int i = 1; i <= k; ++i) r = r * (unsigned __int128)(n - k + i) / (unsigned __int128)i;
    if (r > (unsigned __int128)INT64_MAX) return -1;
    return (int64_t)r;
}

RankTable make_rank_table(int m, int n) {
    RankTable t;
    t.m = m;
    t.n = n;
    int rows = m > 1 ? m - 1 : 1;
    t.host.assign((size_t)rows * (n + 1), 0u);
    for (int i = 0; i + 1 < m; ++i)
        for (int s = 0; s <= n; ++s) {
            int64_t c = binomial64(s + m - i - 2, m - i - 1);
            t.host[(size_t)i * (n + 1) + s] = (uint32_t)c;
        }
    return t;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// key P = prod p_i^{n_i} of lexicographic state r, value = r
__global__ void k_basis_keys(uint32_t D, int m, int n, const uint32_t* __restrict__ rt,
                             unsigned long long* __restrict__ klo,
                             unsigned long long* __restrict__ khi, uint32_t* __restrict__ val) {
    extern __shared__ uint32_t s_rt[];
    const int nrt = (m > 1 ? m - 1 : 1) * (n + 1);
    for (int i = threadIdx.x; i < nrt; i += blockDim.x) s_rt[i] = rt[i];
    __syncthreads();
    uint8_t occ[kMaxSites];
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < D; r += gridDim.x * blockDim.x) {
        unrank_state(r, m, n, s_rt, occ);
        unsigned long long lo = 1ull, hi = 0ull;
        for (int i = 0; i < m; ++i) {
            const unsigned long long p = kPrimes[i];
            for (int k = 0; k < occ[i]; ++k) {
                const unsigned long long c = __umul64hi(lo, p);
                lo *= p;
                hi = hi * p + c;
            }
        }
        klo[r] = lo;
        khi[r] = hi;
        val[r] = r;
    }
}

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_BINS = 16;

__device__ __forceinline__ int rs_digit(unsigned long long lo, unsigned long long hi, int shift) {
    return shift < 64 ? (int)((lo >> shift) & 15ull) : (int)((hi >> (shift - 64)) & 15ull);
}

__global__ void k_rs_hist(const unsigned long long* __restrict__ klo,
                          const unsigned long long* __restrict__ khi, uint32_t D, int shift,
                          uint32_t* __restrict__ counts, int ntiles) {
    __shared__ uint32_t h[RS_BINS];
    if (threadIdx.x < RS_BINS) h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * (uint32_t)RS_TILE;
    for (int i = threadIdx.x; i < RS_TILE; i += RS_THREADS) {
        const uint32_t idx = base + i;
        if (idx < D) atomicAdd(&h[rs_digit(klo[idx], khi[idx], shift)], 1u);
    }
    __syncthreads();
    if (threadIdx.x < RS_BINS) counts[(size_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// exclusive scan of `total` uint32 values, one block of 1024 threads
__global__ void k_rs_scan(uint32_t* __restrict__ a, int total) {
    __shared__ uint32_t part[1024];
    const int t = threadIdx.x;
    const int seg = (total + 1023) / 1024;
    const int b = t * seg, e = min(total, b + seg);
    uint32_t s = 0;
    for (int i = b; i < e; ++i) s += a[i];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        uint32_t v = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = part[t] - s;
    for (int i = b; i < e; ++i) {
        uint32_t v = a[i];
        a[i] = run;
        run += v;
    }
}

__global__ void __launch_bounds__(RS_THREADS)
k_rs_scatter(const unsigned long long* __restrict__ klo, const unsigned long long* __restrict__ khi,
             const uint32_t* __restrict__ vin, unsigned long long* __restrict__ klo_o,
             unsigned long long* __restrict__ khi_o, uint32_t* __restrict__ vout, uint32_t D,
             int shift, const uint32_t* __restrict__ offs, int ntiles) {
    __shared__ uint32_t cnt[RS_BINS][RS_THREADS + 1];
    const int t = threadIdx.x;
    for (int d = 0; d < RS_BINS; ++d) cnt[d][t] = 0;
    const uint32_t base = blockIdx.x * (uint32_t)RS_TILE + (uint32_t)t * RS_ITEMS;
    uint8_t dg[RS_ITEMS], rk[RS_ITEMS];
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {
        const uint32_t idx = base + i;
        dg[i] = 0;
        rk[i] = 0;
        if (idx < D) {
            const int d = rs_digit(klo[idx], khi[idx], shift);
            dg[i] = (uint8_t)d;
            rk[i] = (uint8_t)cnt[d][t];
            cnt[d][t] += 1;
        }
    }
    __syncthreads();
    if (t < RS_BINS) {
        uint32_t run = 0;
        for (int u = 0; u < RS_THREADS; ++u) {
            const uint32_t c = cnt[t][u];
            cnt[t][u] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < RS_ITEMS; ++i) {
        const uint32_t idx = base + i;
        if (idx < D) {
            const int d = dg[i];
            const uint32_t pos = offs[(size_t)d * ntiles + blockIdx.x] + cnt[d][t] + rk[i];
            klo_o[pos] = klo[idx];
            khi_o[pos] = khi[idx];
            vout[pos] = vin[idx];
        }
    }
}

__global__ void k_basis_perm(uint32_t D, const uint32_t* __restrict__ sorted,
                             int32_t* __restrict__ col_of_lex, int32_t* __restrict__ lex_of_col) {
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < D; r += gridDim.x * blockDim.x) {
        const uint32_t v = sorted[r];
        col_of_lex[r] = (int32_t)v;
        lex_of_col[v] = (int32_t)r;
    }
}

// tags (uncontracted sum of n_i * log p_i, hamiltonian.cpp:91-97) and the
// occupation columns of the reference's basis matrix, per reference column
__global__ void k_basis_tags(uint32_t D, int m, int n, const uint32_t* __restrict__ rt,
                             const int32_t* __restrict__ lex_of_col, const double* __restrict__ logp,
                             double* __restrict__ tags, double* __restrict__ occ_cols) {
    extern __shared__ uint32_t s_rt[];
    const int nrt = (m > 1 ? m - 1 : 1) * (n + 1);
    for (int i = threadIdx.x; i < nrt; i += blockDim.x) s_rt[i] = rt[i];
    __syncthreads();
    uint8_t occ[kMaxSites];
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < D; c += gridDim.x * blockDim.x) {
        unrank_state((uint32_t)lex_of_col[c], m, n, s_rt, occ);
        double t = 0.0;
        for (int i = 0; i < m; ++i) {
            t = __dadd_rn(t, __dmul_rn((double)occ[i], logp[i]));
            if (occ_cols) occ_cols[(size_t)c * m + i] = (double)occ[i];
        }
        if (tags) tags[c] = t;
    }
}

__global__ void k_basis_index(int64_t nq, int m, int n, const uint32_t* __restrict__ rt,
                              const uint8_t* __restrict__ q, const int32_t* __restrict__ col_of_lex,
                              int32_t* __restrict__ out) {
    extern __shared__ uint32_t s_rt[];
    const int nrt = (m > 1 ? m - 1 : 1) * (n + 1);
    for (int i = threadIdx.x; i < nrt; i += blockDim.x) s_rt[i] = rt[i];
    __syncthreads();
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nq;
         k += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t* o = q + k * m;
        int tot = 0;
        for (int i = 0; i < m; ++i) tot += o[i];
        out[k] = tot == n ? col_of_lex[rank_state(o, m, n, s_rt)] : -1;
    }
}

// ---- exclusive scan of int64 (row pointers) ----
constexpr int SC_THREADS = 1024;
constexpr int SC_ITEMS = 4;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;

__global__ void k_scan_tile(const int64_t* __restrict__ in, int64_t* __restrict__ out, int64_t n,
                            int64_t* __restrict__ tile_sums) {
    __shared__ int64_t warp_tot[SC_THREADS / 32];
    const int64_t base = blockIdx.x * (int64_t)SC_TILE + threadIdx.x * SC_ITEMS;
    int64_t v[SC_ITEMS];
    int64_t s = 0;
#pragma unroll
    for (int i = 0; i < SC_ITEMS; ++i) {
        v[i] = base + i < n ? in[base + i] : 0;
        s += v[i];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t incl = s;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += y;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        int64_t x = warp_tot[lane];
        int64_t xi = x;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int64_t y = __shfl_up_sync(0xffffffffu, xi, off);
            if (lane >= off) xi += y;
        }
        warp_tot[lane] = xi - x;
        if (lane == 31 && tile_sums) tile_sums[blockIdx.x] = xi;
    }
    __syncthreads();
    int64_t run = warp_tot[w] + incl - s;
#pragma unroll
    for (int i = 0; i < SC_ITEMS; ++i) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
}

__global__ void k_scan_add(int64_t* __restrict__ out, int64_t n, const int64_t* __restrict__ offs) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] += offs[i / SC_TILE];
}

void scan_exclusive_i64(const int64_t* d_in, int64_t* d_out, int64_t n, cudaStream_t st) {
    if (n <= 0) return;
    const int64_t tiles = (n + SC_TILE - 1) / SC_TILE;
    if (tiles == 1) {
        k_scan_tile<<<1, SC_THREADS, 0, st>>>(d_in, d_out, n, nullptr);
        BH_CUDA(cudaGetLastError());
        return;
    }
    DevBuf<int64_t> sums(tiles), offs(tiles);
    k_scan_tile<<<(unsigned)tiles, SC_THREADS, 0, st>>>(d_in, d_out, n, sums.p);
    BH_CUDA(cudaGetLastError());
    scan_exclusive_i64(sums.p, offs.p, tiles, st);
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d_out, n, offs.p);
    BH_CUDA(cudaGetLastError());
    BH_CUDA(cudaStreamSynchronize(st));  // sums/offs are released on return
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------

static unsigned grid_for(int64_t work, int threads) {
    int64_t g = (work + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count() * 16;
    if (g > cap) g = cap;
    return (unsigned)(g < 1 ? 1 : g);
}

void basis_build(bh_basis* b, cudaStream_t st) {
    const uint32_t D = (uint32_t)b->D;
    const int m = b->m, n = b->n;
    b->d_rt.alloc(b->rt.host.size());
    BH_CUDA(cudaMemcpyAsync(b->d_rt.p, b->rt.host.data(), b->rt.host.size() * sizeof(uint32_t),
                            cudaMemcpyHostToDevice, st));
    b->d_col_of_lex.alloc(D);
    b->d_lex_of_col.alloc(D);
    // number of 4-bit digits of the largest key p_{m-1}^n
    static const int primes[kMaxSites] = {2,  3,  5,  7,  11, 13, 17, 19, 23, 29, 31, 37, 41,
                                          43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89, 97};
    const double bits = n * std::log2((double)primes[m - 1]);
    if (bits >= 127.5) throw Error(BH_ERR_ARG, "prime-product key of this sector exceeds 128 bits");
    const int passes = (int)std::ceil((bits + 1.0) / 4.0);

    DevBuf<unsigned long long> klo0(D), khi0(D), klo1(D), khi1(D);
    DevBuf<uint32_t> v0(D), v1(D);
    const size_t smem = b->rt.host.size() * sizeof(uint32_t);
    k_basis_keys<<<grid_for(D, 256), 256, smem, st>>>(D, m, n, b->d_rt.p, klo0.p, khi0.p, v0.p);
    BH_CUDA(cudaGetLastError());
    const int ntiles = (int)((D + RS_TILE - 1) / RS_TILE);
    DevBuf<uint32_t> counts((size_t)RS_BINS * ntiles);
    unsigned long long *ka = klo0.p, *kb = khi0.p, *kc = klo1.p, *kd = khi1.p;
    uint32_t *va = v0.p, *vb = v1.p;
    for (int pass = 0; pass < passes; ++pass) {
        const int shift = 4 * pass;
        k_rs_hist<<<ntiles, RS_THREADS, 0, st>>>(ka, kb, D, shift, counts.p, ntiles);
        k_rs_scan<<<1, 1024, 0, st>>>(counts.p, RS_BINS * ntiles);
        k_rs_scatter<<<ntiles, RS_THREADS, 0, st>>>(ka, kb, va, kc, kd, vb, D, shift, counts.p,
                                                    ntiles);
        BH_CUDA(cudaGetLastError());
        std::swap(ka, kc);
        std::swap(kb, kd);
        std::swap(va, vb);
    }
    k_basis_perm<<<grid_for(D, 256), 256, 0, st>>>(D, va, b->d_col_of_lex.p, b->d_lex_of_col.p);
    BH_CUDA(cudaGetLastError());
    BH_CUDA(cudaStreamSynchronize(st));
}

void basis_tags(const bh_basis* b, double* d_tags, double* d_occ_cols, cudaStream_t st) {
    double logp[kMaxSites];
    static const int primes[kMaxSites] = {2,  3,  5,  7,  11, 13, 17, 19, 23, 29, 31, 37, 41,
                                          43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89, 97};
    for (int i = 0; i < kMaxSites; ++i) logp[i] = std::log((double)primes[i]);
    DevBuf<double> d_logp(kMaxSites);
    BH_CUDA(cudaMemcpyAsync(d_logp.p, logp, sizeof logp, cudaMemcpyHostToDevice, st));
    const size_t smem = b->rt.host.size() * sizeof(uint32_t);
    k_basis_tags<<<grid_for(b->D, 256), 256, smem, st>>>((uint32_t)b->D, b->m, b->n, b->d_rt.p,
                                                         b->d_lex_of_col.p, d_logp.p, d_tags,
                                                         d_occ_cols);
    BH_CUDA(cudaGetLastError());
    BH_CUDA(cudaStreamSynchronize(st));
}

void basis_index(const bh_basis* b, int64_t nq, const uint8_t* d_occ, int32_t* d_col,
                 cudaStream_t st) {
    if (nq <= 0) return;
    const size_t smem = b->rt.host.size() * sizeof(uint32_t);
    k_basis_index<<<grid_for(nq, 256), 256, smem, st>>>(nq, b->m, b->n, b->d_rt.p, d_occ,
                                                        b->d_col_of_lex.p, d_col);
    BH_CUDA(cudaGetLastError());
}

}  // namespace bh
