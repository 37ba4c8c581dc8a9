// bh_internal.h -- internal declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/bh_gb300.h"

namespace bh {

// ---------------------------------------------------------------------------
// errors: internal code throws bh::Error; the C ABI converts it to a status
// code and stores the message for bh_last_error().
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void set_last_error(const std::string& msg);

#define BH_CUDA(call)                                                                    \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            throw ::bh::Error(BH_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

#define BH_REQUIRE(cond, msg)                                  \
    do {                                                       \
        if (!(cond)) throw ::bh::Error(BH_ERR_ARG, (msg));     \
    } while (0)

// Owning device buffer.
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    explicit DevBuf(size_t count) { alloc(count); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count) {
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            (void)cudaGetLastError();
            throw Error(BH_ERR_NOMEM, "cudaMalloc of " + std::to_string(count * sizeof(T)) +
                                          " bytes failed: " + cudaGetErrorString(e));
        }
        n = count;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
};

// Stream owned by one library call (calls are re-entrant across threads).
struct Stream {
    cudaStream_t s = nullptr;
    Stream() { BH_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
    ~Stream() { if (s) cudaStreamDestroy(s); }
    operator cudaStream_t() const { return s; }
};

constexpr int kMaxDevices = 64;  // device ordinals with cached attributes
int sm_count();                  // multiprocessors of the current device

// ---------------------------------------------------------------------------
// Fock basis.  States are identified by their lexicographic index r (the
// enumeration order of the reference's init_lexicographic).  rank table
// RT[i][s] = C(s + m - i - 2, m - i - 1), i in [0, m-2], s in [0, n]:
//   r = sum_i RT[i][s_i],  s_i = sum_{j > i} n_j.
// ---------------------------------------------------------------------------
constexpr int kMaxSites = 25;   // primes table of the reference (hamiltonian.cpp:144)
constexpr int kMaxBosons = 60;  // occupations stored as uint8, keys must fit 128 bits

struct RankTable {
    int m = 0, n = 0;
    std::vector<uint32_t> host;  // (m-1) x (n+1)
};
RankTable make_rank_table(int m, int n);
int64_t binomial64(int n, int k);

}  // namespace bh

struct bh_basis {
    int m = 0, n = 0;
    int64_t D = 0;
    int device = 0;
    bh::RankTable rt;
    bh::DevBuf<uint32_t> d_rt;          // rank table
    bh::DevBuf<int32_t> d_col_of_lex;   // lexicographic -> reference column
    bh::DevBuf<int32_t> d_lex_of_col;   // reference column -> lexicographic
};

struct bh_hamiltonian {
    const bh_basis* basis = nullptr;
    int m = 0, n = 0;
    int64_t D = 0;
    int64_t nnz = 0;  // off-diagonal entries of T
    int device = 0;
    std::vector<int32_t> h_nbr_off, h_nbr;
    bh::DevBuf<int32_t> d_nbr_off, d_nbr;
    // T in lexicographic order (rows and columns), values of T (J = 1)
    bh::DevBuf<int64_t> d_rp;
    bh::DevBuf<int32_t> d_ci;
    bh::DevBuf<double> d_tv64;
    bh::DevBuf<float> d_tv32;
    // diagonal V in lexicographic order
    bh::DevBuf<double> d_vd64;
    bh::DevBuf<float> d_vd32;
    // matrix-free variant: no stored T or V; packed occupation strings (lex
    // order), the directed bonds and the table of -sqrt(a) instead
    bool matrix_free = false;
    int occ_bits = 0;
    int nbonds = 0;
    bh::DevBuf<uint64_t> d_occ;
    bh::DevBuf<uint8_t> d_bonds;
    bh::DevBuf<double> d_sq64;
    bh::DevBuf<float> d_sq32;
};

namespace bh {

// ---- launchers (bh_basis.cu) ----
void basis_build(bh_basis* b, cudaStream_t st);
void basis_tags(const bh_basis* b, double* d_tags, double* d_occ_cols, cudaStream_t st);
void basis_index(const bh_basis* b, int64_t nq, const uint8_t* d_occ, int32_t* d_col,
                 cudaStream_t st);
void scan_exclusive_i64(const int64_t* d_in, int64_t* d_out, int64_t n, cudaStream_t st);

// ---- launchers (bh_hamiltonian.cu) ----
void hamiltonian_build(bh_hamiltonian* h, cudaStream_t st);
// matrix-free variant: packed occupations, bonds, -sqrt table and the entry count
void hamiltonian_build_matrix_free(bh_hamiltonian* h, cudaStream_t st);
// bits per site of the packed occupation strings (0 if m sites do not fit 64 bits)
int occupation_bits(int m, int n);
// CSR of H = J T + U V - mu N with diagonal entries, rows/cols in `order`.
void hamiltonian_csr(const bh_hamiltonian* h, int order, double J, double U, double mu,
                     int64_t* d_rp, int32_t* d_ci, double* d_val, cudaStream_t st);
// Block-diagonal H of several sectors (in the given order), sector k's rows
// and columns offset by the dimensions of the sectors before it.
void hamiltonian_multi_csr(int nh, const bh_hamiltonian* const* hs, int order, double J, double U, double mu,
                           int64_t* d_rp, int32_t* d_ci, double* d_val, cudaStream_t st);
void spdm_device(const bh_hamiltonian* h, const double* d_phi_lex, double* d_rho,
                 cudaStream_t st);
// out[r][0..ncols) = in[map[r]][0..ncols)  (double)
void gather_rows(int64_t D, int ncols, const int32_t* d_map, const double* d_in, double* d_out,
                 cudaStream_t st);
// density / compressibility maps from sector ground energies (device)
void phase_map_device(int m, int n_lo, int nsec, int nJ, const double* d_e0, int nmu,
                      const double* d_mu, double* d_density, double* d_kappa, cudaStream_t st);

// ---- mean field (bh_meanfield.cu) ----
// psi[k] of the self-consistent mean-field iteration at (mu[k], J[k]) from
// psi0[k]; iters[k] = outer iterations (-1: truncation limit, -2: max_outer)
void scmf_device(int npts, const double* d_mu, const double* d_J, int q, const double* d_psi0,
                 int precision, int max_outer, double* d_psi, int* d_iters, cudaStream_t st);

// ---- lattices (bh_lattice.cpp) ----
using Lists = std::vector<std::vector<int32_t>>;
Lists chain_lists(int m, bool closed);
Lists square_lists(int m, bool closed);
Lists cube_lists(int m, bool closed);
void flatten(const Lists& nb, int32_t* off, int32_t* out, int cap, int* count);

// ---- dense symmetric eigensolver on the device (bh_dense.cu) ----
// a: n x n column-major (host); w: eigenvalues ascending; z (optional): vectors
void dense_eigh(int64_t n, const double* h_a, double* h_w, double* h_z);

// ---- optional per-kernel timing (bh_profile.cpp) ----
bool profile_on();
void profile_begin(cudaStream_t st);
void profile_end(cudaStream_t st, const char* name, double bytes);
void profile_flush();

// ---- host dense symmetric eigensolver (bh_symeig.cpp) ----
// a: n x n column-major symmetric, overwritten with eigenvectors (columns);
// w: eigenvalues ascending.  Returns false if the iteration did not converge.
bool symeig(int n, double* a, double* w);

}  // namespace bh
