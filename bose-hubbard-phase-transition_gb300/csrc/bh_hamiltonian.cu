// bh_hamiltonian.cu -- device assembly of the Bose-Hubbard Hamiltonian terms.
//
// Replaces BH::fill_hopping / fill_interaction / fill_chemical /
// fixed_bosons_hamiltonian (src/hamiltonian.cpp:170-256).  One warp per row:
// the lanes take the directed bonds (i, j in nbr(i)) of the row state, each
// computes the target state's index by combinadic ranking (exact, no tag
// search), the warp sorts the entries by column, merges duplicate bonds (for
// instance the two bonds of a 2-site ring) and writes one CSR row.  Row counts
// come from the same kernel in count mode followed by a device exclusive scan.
//
// Matrix element: <s - e_i + e_j| b+_j b_i |s> ... written per row state s as
//   T[s][s - e_i + e_j] = -sqrt(n_i (n_j + 1)),  for each j in nbr(i), n_i >= 1,
// which is T = -sum_i sum_{j in nbr(i)} b+_i b_j for symmetric lists.
#include <algorithm>
#include <cmath>

#include "bh_device.cuh"
#include "bh_internal.h"

namespace bh {

constexpr int kMaxSlots = 4;  // up to 32 * 4 - 1 = 127 directed bonds per row

__device__ __forceinline__ float to_f32(double v) { return (float)v; }

template <bool FILL>
__global__ void __launch_bounds__(256)
k_csr_rows(uint32_t D, int m, int n, const uint32_t* __restrict__ rt,
           const int32_t* __restrict__ bi, const int32_t* __restrict__ bj, int nbonds,
           const int32_t* __restrict__ lex_of_row, const int32_t* __restrict__ col_of_lex,
           int with_diag, double J, double U, double shift, int64_t* __restrict__ counts,
           const int64_t* __restrict__ rp, int32_t* __restrict__ ci, double* __restrict__ val,
           float* __restrict__ val32) {
    extern __shared__ uint32_t s_rt[];
    const int nrt = (m > 1 ? m - 1 : 1) * (n + 1);
    for (int i = threadIdx.x; i < nrt; i += blockDim.x) s_rt[i] = rt[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint32_t warps_total = (gridDim.x * blockDim.x) >> 5;
    const int nslots = nbonds + (with_diag ? 1 : 0);
    uint8_t occ[kMaxSites], tgt[kMaxSites];
    for (uint32_t row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < D; row += warps_total) {
        const uint32_t lr = lex_of_row ? (uint32_t)lex_of_row[row] : row;
        unrank_state(lr, m, n, s_rt, occ);
        int col[kMaxSlots];
        double v[kMaxSlots];
        bool ok[kMaxSlots];
#pragma unroll
        for (int s = 0; s < kMaxSlots; ++s) {
            const int k = s * 32 + lane;
            ok[s] = false;
            col[s] = 0;
            v[s] = 0.0;
            if (k < nbonds) {
                const int i = bi[k], j = bj[k];
                if (occ[i] >= 1) {
                    for (int t = 0; t < m; ++t) tgt[t] = occ[t];
                    tgt[i] -= 1;
                    tgt[j] += 1;
                    const uint32_t tr = rank_state(tgt, m, n, s_rt);
                    col[s] = col_of_lex ? col_of_lex[tr] : (int)tr;
                    v[s] = -sqrt((double)occ[i] * (double)(occ[j] + 1));
                    ok[s] = true;
                }
            } else if (k == nbonds && with_diag) {
                double a = 0.0;
                for (int t = 0; t < m; ++t) {
                    const double x = occ[t];
                    a += 0.5 * x * (x - 1.0);
                }
                col[s] = (int)row;
                // (U V) + (-mu n) with one rounding each, no contraction
                v[s] = __dadd_rn(__dmul_rn(U, a), shift);
                ok[s] = true;
            }
        }
        // first-occurrence flags, merged values and sorted positions
        bool first[kMaxSlots];
        double sum[kMaxSlots];
        int pos[kMaxSlots];
#pragma unroll
        for (int s = 0; s < kMaxSlots; ++s) {
            first[s] = ok[s];
            sum[s] = 0.0;
        }
        for (int s2 = 0; s2 < kMaxSlots; ++s2) {
            if (s2 * 32 >= nslots) break;
            for (int src = 0; src < 32; ++src) {
                const int c2 = __shfl_sync(0xffffffffu, col[s2], src);
                const int ok2 = __shfl_sync(0xffffffffu, (int)ok[s2], src);
                const double v2 = __shfl_sync(0xffffffffu, v[s2], src);
                if (!ok2) continue;
                const int idx2 = s2 * 32 + src;
#pragma unroll
                for (int s = 0; s < kMaxSlots; ++s) {
                    if (!ok[s] || c2 != col[s]) continue;
                    if (idx2 < s * 32 + lane) first[s] = false;
                    sum[s] += v2;  // in index order: s2 outer, src inner
                }
            }
        }
#pragma unroll
        for (int s = 0; s < kMaxSlots; ++s) pos[s] = 0;
        int cnt = 0;
        for (int s2 = 0; s2 < kMaxSlots; ++s2) {
            if (s2 * 32 >= nslots) break;
            const unsigned fm = __ballot_sync(0xffffffffu, first[s2]);
            cnt += __popc(fm);
            for (int src = 0; src < 32; ++src) {
                if (!((fm >> src) & 1u)) continue;
                const int c2 = __shfl_sync(0xffffffffu, col[s2], src);
#pragma unroll
                for (int s = 0; s < kMaxSlots; ++s)
                    if (first[s] && c2 < col[s]) pos[s] += 1;
            }
        }
        if (!FILL) {
            if (lane == 0) counts[row] = cnt;
        } else {
            const int64_t base = rp[row];
#pragma unroll
            for (int s = 0; s < kMaxSlots; ++s) {
                if (!first[s]) continue;
                const bool is_diag = with_diag && (s * 32 + lane == nbonds);
                const double out = is_diag ? sum[s] : J * sum[s];
                ci[base + pos[s]] = col[s];
                if (val) val[base + pos[s]] = out;
                if (val32) val32[base + pos[s]] = to_f32(out);
            }
        }
    }
}

// V_r = 1/2 sum n_i (n_i - 1) in lexicographic order
__global__ void k_diag_V(uint32_t D, int m, int n, const uint32_t* __restrict__ rt,
                         double* __restrict__ v64, float* __restrict__ v32) {
    extern __shared__ uint32_t s_rt[];
    const int nrt = (m > 1 ? m - 1 : 1) * (n + 1);
    for (int i = threadIdx.x; i < nrt; i += blockDim.x) s_rt[i] = rt[i];
    __syncthreads();
    uint8_t occ[kMaxSites];
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < D; r += gridDim.x * blockDim.x) {
        unrank_state(r, m, n, s_rt, occ);
        double a = 0.0;
        for (int t = 0; t < m; ++t) {
            const double x = occ[t];
            a += 0.5 * x * (x - 1.0);
        }
        v64[r] = a;
        v32[r] = (float)a;
    }
}

// Single-particle density matrix <phi| b+_i b_j |phi> over lexicographic rows,
// one block-partial m x m per CTA (deterministic second stage below).  The
// target index of b+_i b_j applied to row state s differs from r only in the
// suffix sums between i and j, so it is updated incrementally.
__global__ void k_spdm_partial(uint32_t D, int m, int n, const uint32_t* __restrict__ rt,
                               const double* __restrict__ phi, double* __restrict__ part) {
    extern __shared__ double s_acc[];  // m*m doubles, then rank table
    uint32_t* s_rt = reinterpret_cast<uint32_t*>(s_acc + m * m);
    const int nrt = (m > 1 ? m - 1 : 1) * (n + 1);
    for (int i = threadIdx.x; i < nrt; i += blockDim.x) s_rt[i] = rt[i];
    for (int i = threadIdx.x; i < m * m; i += blockDim.x) s_acc[i] = 0.0;
    __syncthreads();
    uint8_t occ[kMaxSites];
    int suf[kMaxSites];
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < D; r += gridDim.x * blockDim.x) {
        const double pr = phi[r];
        if (pr == 0.0) continue;
        unrank_state(r, m, n, s_rt, occ);
        int acc = 0;
        for (int k = m - 1; k >= 0; --k) {
            suf[k] = acc;  // bosons on sites > k
            acc += occ[k];
        }
        for (int i = 0; i < m; ++i) {
            atomicAdd(&s_acc[i * m + i], pr * pr * (double)occ[i]);
            for (int j = 0; j < m; ++j) {
                if (j == i || occ[j] == 0) continue;
                // boson moves j -> i
                int64_t t = r;
                if (i < j) {
                    for (int k = i; k < j; ++k)
                        t += (int64_t)s_rt[k * (n + 1) + suf[k] - 1] - (int64_t)s_rt[k * (n + 1) + suf[k]];
                } else {
                    for (int k = j; k < i; ++k)
                        t += (int64_t)s_rt[k * (n + 1) + suf[k] + 1] - (int64_t)s_rt[k * (n + 1) + suf[k]];
                }
                atomicAdd(&s_acc[i * m + j],
                          phi[t] * pr * sqrt((double)(occ[i] + 1) * (double)occ[j]));
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m * m; i += blockDim.x) part[(size_t)blockIdx.x * m * m + i] = s_acc[i];
}

__global__ void k_sum_partials(int nparts, int len, const double* __restrict__ part,
                               double* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int p = 0; p < nparts; ++p) s += part[(size_t)p * len + i];
        out[i] = s;
    }
}

__global__ void k_gather_rows(int64_t D, int ncols, const int32_t* __restrict__ map,
                              const double* __restrict__ in, double* __restrict__ out) {
    const int64_t total = D * ncols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / ncols;
        const int c = (int)(i - r * ncols);
        out[i] = in[(int64_t)map[r] * ncols + c];
    }
}

// Phase map from sector ground energies E0(n, J) (computed at mu = 0): for
// each (J, mu) the occupied sector n* = argmin_n E0(n) - mu n gives the
// density n*/m; the compressibility is d density / d mu by central
// differences on the mu grid (one-sided at the ends).
__global__ void k_phase_density(int m, int n_lo, int nsec, int nJ, const double* __restrict__ e0,
                                int nmu, const double* __restrict__ mu, double* __restrict__ dens) {
    const int total = nJ * nmu;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int jj = i / nmu, k = i % nmu;
        int best = 0;
        double bv = e0[jj] - mu[k] * (double)n_lo;
        for (int sct = 1; sct < nsec; ++sct) {
            const double v = e0[(size_t)sct * nJ + jj] - mu[k] * (double)(n_lo + sct);
            if (v < bv) {
                bv = v;
                best = sct;
            }
        }
        dens[i] = (double)(n_lo + best) / (double)m;
    }
}

__global__ void k_phase_kappa(int nJ, int nmu, const double* __restrict__ mu,
                              const double* __restrict__ dens, double* __restrict__ kappa) {
    const int total = nJ * nmu;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int jj = i / nmu, k = i % nmu;
        const double* d = dens + (size_t)jj * nmu;
        double v = 0.0;
        if (nmu > 1) {
            const int a = k > 0 ? k - 1 : k, b = k + 1 < nmu ? k + 1 : k;
            v = (d[b] - d[a]) / (mu[b] - mu[a]);
        }
        kappa[i] = v;
    }
}

// ---------------------------------------------------------------------------

static void bond_arrays(const bh_hamiltonian* h, std::vector<int32_t>& bi, std::vector<int32_t>& bj) {
    for (int i = 0; i < h->m; ++i)
        for (int k = h->h_nbr_off[i]; k < h->h_nbr_off[i + 1]; ++k) {
            bi.push_back(i);
            bj.push_back(h->h_nbr[k]);
        }
}

static unsigned warp_grid(int64_t rows) {
    int64_t g = (rows + 7) / 8;  // 8 warps per 256-thread block
    const int64_t cap = (int64_t)sm_count() * 32;
    if (g > cap) g = cap;
    return (unsigned)(g < 1 ? 1 : g);
}

// Builds CSR rows; returns nnz.  counts/rp are allocated here.
static int64_t build_rows(const bh_hamiltonian* h, const int32_t* lex_of_row,
                          const int32_t* col_of_lex, int with_diag, double J, double U,
                          double shift, DevBuf<int64_t>& rp, DevBuf<int32_t>* ci,
                          DevBuf<double>* val, DevBuf<float>* val32, int64_t* d_rp_out,
                          int32_t* d_ci_out, double* d_val_out, cudaStream_t st) {
    const bh_basis* b = h->basis;
    const uint32_t D = (uint32_t)h->D;
    std::vector<int32_t> hbi, hbj;
    bond_arrays(h, hbi, hbj);
    const int nb = (int)hbi.size();
    BH_REQUIRE(nb + (with_diag ? 1 : 0) <= 32 * kMaxSlots, "too many directed bonds per site set");
    DevBuf<int32_t> dbi(nb), dbj(nb);
    if (nb) {
        BH_CUDA(cudaMemcpyAsync(dbi.p, hbi.data(), nb * sizeof(int32_t), cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaMemcpyAsync(dbj.p, hbj.data(), nb * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    }
    const size_t smem = b->rt.host.size() * sizeof(uint32_t);
    DevBuf<int64_t> counts(D + 1);
    BH_CUDA(cudaMemsetAsync(counts.p, 0, (D + 1) * sizeof(int64_t), st));
    k_csr_rows<false><<<warp_grid(D), 256, smem, st>>>(D, h->m, h->n, b->d_rt.p, dbi.p, dbj.p, nb,
                                                       lex_of_row, col_of_lex, with_diag, J, U,
                                                       shift, counts.p, nullptr, nullptr, nullptr,
                                                       nullptr);
    BH_CUDA(cudaGetLastError());
    int64_t* rpp = d_rp_out;
    if (!rpp) {
        rp.alloc(D + 1);
        rpp = rp.p;
    }
    scan_exclusive_i64(counts.p, rpp, (int64_t)D + 1, st);
    int64_t nnz = 0;
    BH_CUDA(cudaMemcpyAsync(&nnz, rpp + D, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    BH_CUDA(cudaStreamSynchronize(st));
    int32_t* cip = d_ci_out;
    double* vp = d_val_out;
    float* vp32 = nullptr;
    if (!cip) {
        ci->alloc(nnz);
        cip = ci->p;
    }
    if (!vp && val) {
        val->alloc(nnz);
        vp = val->p;
    }
    if (val32) {
        val32->alloc(nnz);
        vp32 = val32->p;
    }
    k_csr_rows<true><<<warp_grid(D), 256, smem, st>>>(D, h->m, h->n, b->d_rt.p, dbi.p, dbj.p, nb,
                                                      lex_of_row, col_of_lex, with_diag, J, U,
                                                      shift, nullptr, rpp, cip, vp, vp32);
    BH_CUDA(cudaGetLastError());
    BH_CUDA(cudaStreamSynchronize(st));
    return nnz;
}

void hamiltonian_build(bh_hamiltonian* h, cudaStream_t st) {
    h->nnz = build_rows(h, nullptr, nullptr, 0, 1.0, 0.0, 0.0, h->d_rp, &h->d_ci, &h->d_tv64,
                        &h->d_tv32, nullptr, nullptr, nullptr, st);
    h->d_vd64.alloc(h->D);
    h->d_vd32.alloc(h->D);
    const bh_basis* b = h->basis;
    const size_t smem = b->rt.host.size() * sizeof(uint32_t);
    int64_t g = (h->D + 255) / 256;
    if (g > sm_count() * 16) g = sm_count() * 16;
    k_diag_V<<<(unsigned)(g < 1 ? 1 : g), 256, smem, st>>>((uint32_t)h->D, h->m, h->n, b->d_rt.p,
                                                           h->d_vd64.p, h->d_vd32.p);
    BH_CUDA(cudaGetLastError());
    BH_CUDA(cudaStreamSynchronize(st));
}

int occupation_bits(int m, int n) {
    int b = 1;
    while ((1 << b) - 1 < n) ++b;
    return (int64_t)m * b <= 64 ? b : 0;
}

// Packed occupation string of each lexicographic state: site i in bits
// [bits i, bits (i + 1)).
__global__ void k_pack_occ(uint32_t D, int m, int n, int bits, const uint32_t* __restrict__ rt,
                           uint64_t* __restrict__ out) {
    extern __shared__ uint32_t s_rt[];
    const int nrt = (m > 1 ? m - 1 : 1) * (n + 1);
    for (int i = threadIdx.x; i < nrt; i += blockDim.x) s_rt[i] = rt[i];
    __syncthreads();
    uint8_t occ[kMaxSites];
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < D; r += gridDim.x * blockDim.x) {
        unrank_state(r, m, n, s_rt, occ);
        uint64_t w = 0;
        for (int i = 0; i < m; ++i) w |= (uint64_t)occ[i] << (bits * i);
        out[r] = w;
    }
}

void hamiltonian_build_matrix_free(bh_hamiltonian* h, cudaStream_t st) {
    const bh_basis* b = h->basis;
    const int bits = occupation_bits(h->m, h->n);
    BH_REQUIRE(bits > 0, "matrix-free operator: the occupations of m sites do not fit 64 bits");
    std::vector<int32_t> hbi, hbj;
    bond_arrays(h, hbi, hbj);
    const int nb = (int)hbi.size();
    BH_REQUIRE(nb <= 128, "matrix-free operator: at most 128 directed bonds");
    h->matrix_free = true;
    h->occ_bits = bits;
    h->nbonds = nb;
    std::vector<uint8_t> hb((size_t)2 * nb);
    for (int k = 0; k < nb; ++k) {
        hb[2 * k] = (uint8_t)hbi[k];
        hb[2 * k + 1] = (uint8_t)hbj[k];
    }
    h->d_bonds.alloc(hb.size());
    if (nb) BH_CUDA(cudaMemcpyAsync(h->d_bonds.p, hb.data(), hb.size(), cudaMemcpyHostToDevice, st));
    // hop amplitudes -sqrt(n_i (n_j + 1)) by table, a = n_i (n_j + 1) <= n (n + 1)
    const int na = h->n * (h->n + 1) + 1;
    std::vector<double> sq64(na);
    std::vector<float> sq32(na);
    for (int a = 0; a < na; ++a) {
        sq64[a] = -std::sqrt((double)a);
        sq32[a] = (float)sq64[a];
    }
    h->d_sq64.alloc(na);
    h->d_sq32.alloc(na);
    BH_CUDA(cudaMemcpyAsync(h->d_sq64.p, sq64.data(), na * sizeof(double), cudaMemcpyHostToDevice, st));
    BH_CUDA(cudaMemcpyAsync(h->d_sq32.p, sq32.data(), na * sizeof(float), cudaMemcpyHostToDevice, st));
    h->d_occ.alloc(h->D);
    const size_t smem = b->rt.host.size() * sizeof(uint32_t);
    int64_t g = (h->D + 255) / 256;
    if (g > sm_count() * 16) g = sm_count() * 16;
    k_pack_occ<<<(unsigned)(g < 1 ? 1 : g), 256, smem, st>>>((uint32_t)h->D, h->m, h->n, bits,
                                                             b->d_rt.p, h->d_occ.p);
    BH_CUDA(cudaGetLastError());
    // entries of the equivalent stored T (duplicate bonds merged), for reporting
    DevBuf<int64_t> counts(h->D + 1), rp(h->D + 1);
    DevBuf<int32_t> dbi(nb), dbj(nb);
    if (nb) {
        BH_CUDA(cudaMemcpyAsync(dbi.p, hbi.data(), nb * sizeof(int32_t), cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaMemcpyAsync(dbj.p, hbj.data(), nb * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    }
    BH_CUDA(cudaMemsetAsync(counts.p, 0, (h->D + 1) * sizeof(int64_t), st));
    k_csr_rows<false><<<warp_grid(h->D), 256, smem, st>>>((uint32_t)h->D, h->m, h->n, b->d_rt.p, dbi.p,
                                                          dbj.p, nb, nullptr, nullptr, 0, 1.0, 0.0, 0.0,
                                                          counts.p, nullptr, nullptr, nullptr, nullptr);
    BH_CUDA(cudaGetLastError());
    scan_exclusive_i64(counts.p, rp.p, h->D + 1, st);
    BH_CUDA(cudaMemcpyAsync(&h->nnz, rp.p + h->D, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    BH_CUDA(cudaStreamSynchronize(st));
}

void hamiltonian_csr(const bh_hamiltonian* h, int order, double J, double U, double mu,
                     int64_t* d_rp, int32_t* d_ci, double* d_val, cudaStream_t st) {
    const bh_basis* b = h->basis;
    const bool ref = order == BH_ORDER_REFERENCE;
    DevBuf<int64_t> unused;
    build_rows(h, ref ? b->d_lex_of_col.p : nullptr, ref ? b->d_col_of_lex.p : nullptr, 1, J, U,
               -mu * (double)h->n, unused, nullptr, nullptr, nullptr, d_rp, d_ci, d_val, st);
}

// Moves one sector's CSR (rows and columns 0..D-1, entries from 0) to its
// place in a block-diagonal matrix: row pointers + nnz_off, columns + row_off.
__global__ void k_shift_csr(int64_t nrow1, int64_t* __restrict__ rp, int64_t nnz, int32_t* __restrict__ ci,
                            int64_t row_off, int64_t nnz_off) {
    const int64_t n = nrow1 > nnz ? nrow1 : nnz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < nrow1) rp[i] += nnz_off;
        if (i < nnz) ci[i] += (int32_t)row_off;
    }
}

void hamiltonian_multi_csr(int nh, const bh_hamiltonian* const* hs, int order, double J, double U, double mu,
                           int64_t* d_rp, int32_t* d_ci, double* d_val, cudaStream_t st) {
    int64_t row_off = 0, nnz_off = 0;
    for (int k = 0; k < nh; ++k) {
        const bh_hamiltonian* h = hs[k];
        const int64_t nz = h->nnz + h->D;
        hamiltonian_csr(h, order, J, U, mu, d_rp + row_off, d_ci + nnz_off, d_val + nnz_off, st);
        const int64_t n = std::max<int64_t>(h->D + 1, nz);
        const int64_t g = std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8));
        k_shift_csr<<<(unsigned)g, 256, 0, st>>>(h->D + 1, d_rp + row_off, nz, d_ci + nnz_off, row_off, nnz_off);
        BH_CUDA(cudaGetLastError());
        row_off += h->D;
        nnz_off += nz;
    }
    BH_CUDA(cudaStreamSynchronize(st));
}

void spdm_device(const bh_hamiltonian* h, const double* d_phi_lex, double* d_rho, cudaStream_t st) {
    const bh_basis* b = h->basis;
    const int m = h->m;
    int64_t g = (h->D + 255) / 256;
    const int64_t cap = (int64_t)sm_count() * 4;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    DevBuf<double> part((size_t)g * m * m);
    const size_t smem = (size_t)m * m * sizeof(double) + b->rt.host.size() * sizeof(uint32_t);
    k_spdm_partial<<<(unsigned)g, 256, smem, st>>>((uint32_t)h->D, m, h->n, b->d_rt.p, d_phi_lex,
                                                   part.p);
    BH_CUDA(cudaGetLastError());
    k_sum_partials<<<(m * m + 255) / 256, 256, 0, st>>>((int)g, m * m, part.p, d_rho);
    BH_CUDA(cudaGetLastError());
    BH_CUDA(cudaStreamSynchronize(st));
}

void gather_rows(int64_t D, int ncols, const int32_t* d_map, const double* d_in, double* d_out,
                 cudaStream_t st) {
    int64_t g = (D * ncols + 255) / 256;
    if (g > sm_count() * 16) g = sm_count() * 16;
    k_gather_rows<<<(unsigned)(g < 1 ? 1 : g), 256, 0, st>>>(D, ncols, d_map, d_in, d_out);
    BH_CUDA(cudaGetLastError());
}

void phase_map_device(int m, int n_lo, int nsec, int nJ, const double* d_e0, int nmu,
                      const double* d_mu, double* d_density, double* d_kappa, cudaStream_t st) {
    const int total = nJ * nmu;
    const unsigned g = (unsigned)std::max(1, std::min((total + 255) / 256, sm_count() * 8));
    k_phase_density<<<g, 256, 0, st>>>(m, n_lo, nsec, nJ, d_e0, nmu, d_mu, d_density);
    BH_CUDA(cudaGetLastError());
    k_phase_kappa<<<g, 256, 0, st>>>(nJ, nmu, d_mu, d_density, d_kappa);
    BH_CUDA(cudaGetLastError());
}

}  // namespace bh
