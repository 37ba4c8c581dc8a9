// bh_capi.cpp -- the C ABI (include/bh_gb300.h).  Every entry point converts
// internal exceptions to a status code and keeps the message per thread.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "bh_internal.h"
#include "bh_krylov.cuh"

namespace bh {

static thread_local std::string g_last_error;

void set_last_error(const std::string& msg) { g_last_error = msg; }

template <class F>
static int guard(F&& f) {
    try {
        f();
        g_last_error.clear();
        return BH_OK;
    } catch (const Error& e) {
        g_last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return BH_ERR_NOMEM;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return BH_ERR_ARG;
    }
}

static std::vector<int32_t> host_copy_i32(const int32_t* d, int64_t n) {
    std::vector<int32_t> h((size_t)n);
    if (n) BH_CUDA(cudaMemcpy(h.data(), d, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    return h;
}

static void check_solver_opts(const bh_solver_opts* o) {
    BH_REQUIRE(o != nullptr, "options pointer is null");
    BH_REQUIRE(o->precision == BH_PREC_FP64 || o->precision == BH_PREC_MIXED, "unknown precision mode");
    BH_REQUIRE(o->order == BH_ORDER_REFERENCE || o->order == BH_ORDER_LEX, "unknown vector order");
    BH_REQUIRE(o->nev >= 1, "nb_eigen must be >= 1");
    BH_REQUIRE(std::isfinite(o->tol) && o->tol >= 0.0, "tol must be finite and >= 0");
}

// Hamiltonian parameters (and any other real inputs) must be finite: a NaN or
// an infinity would run a whole solve on garbage, so it is rejected before
// any device work.
static void require_finite(const double* v, int64_t n, const char* what) {
    for (int64_t i = 0; i < n; ++i)
        if (!std::isfinite(v[i])) throw Error(BH_ERR_ARG, std::string(what) + " must be finite (entry " +
                                                              std::to_string(i) + " is not)");
}

static void require_finite_params(double J, double U, double mu) {
    BH_REQUIRE(std::isfinite(J), "J must be finite");
    BH_REQUIRE(std::isfinite(U), "U must be finite");
    BH_REQUIRE(std::isfinite(mu), "mu must be finite");
}

// fills the geometry of a request from the options and the dimension
static SolveRequest make_request(const bh_solver_opts* o, int64_t D, int S) {
    SolveRequest rq;
    rq.S = S;
    rq.nev = o->nev;
    rq.precision = o->precision;
    int p = o->block > 0 ? o->block : 2;
    if ((int64_t)p * 2 > D) p = 1;
    rq.p = p;
    BH_REQUIRE(o->nev <= D - 2 || (D <= 2 && o->nev <= D), "nb_eigen must be <= dimension - 2");
    // automatic basis size: 7 nev (measured best on the m=10 multi-sector grid
    // among 4..10 nev: fewer restarts, each rotation still one pass), at least
    // nev + 8 blocks
    int kmax = o->ncv > 0 ? o->ncv : std::max(7 * o->nev, o->nev + 8 * p);
    kmax = (kmax + p - 1) / p * p;
    if (kmax > D) kmax = (int)(D / p * p);
    if (kmax < o->nev + p) {
        // tiny dimension: the whole space
        p = 1;
        rq.p = 1;
        kmax = (int)D;
    }
    rq.kmax = kmax;
    rq.max_restarts = o->max_restarts > 0 ? o->max_restarts : 1000;
    rq.tol = o->tol > 0.0 ? o->tol : (o->precision == BH_PREC_MIXED ? 3e-7 : 1e-10);
    rq.seed = o->seed;
    rq.want_vectors = o->want_vectors != 0;
    return rq;
}

// single-point calls: the reference throws when the solve fails (operator.cpp:27-29)
static void throw_if_failed(const SolveResult& r, int nev) {
    if (r.status[0] == BH_ERR_BREAKDOWN)
        throw Error(BH_ERR_BREAKDOWN, "Krylov space exhausted before nb_eigen eigenvalues "
                                      "(invariant start block, or fewer states than requested)");
    if (r.nconv[0] < nev) throw Error(BH_ERR_NOCONV, "Eigenvalue computation failed.");
}

static void fill_info(bh_solve_info* info, const SolveResult& r, int nev, double secs) {
    if (!info) return;
    int mn = nev;
    for (int c : r.nconv) mn = std::min(mn, c);
    info->nconv = r.nconv.empty() ? 0 : mn;
    info->restarts = r.restarts;
    info->matvecs = r.matvecs;
    double mx = 0.0;
    for (double v : r.resid) mx = std::max(mx, v);
    info->max_resid = mx;
    info->seconds = secs;
    info->launches = r.launches;
}

}  // namespace bh

using namespace bh;

extern "C" {

const char* bh_last_error(void) { return g_last_error.c_str(); }

int bh_version(void) { return 10000; }

// ---- lattices ----
int bh_neighbours_chain(int m, int closed, int32_t* off, int32_t* nbr, int cap, int* count) {
    return guard([&] {
        BH_REQUIRE(off != nullptr, "offsets pointer is null");
        flatten(chain_lists(m, closed != 0), off, nbr, cap, count);
    });
}
int bh_neighbours_square(int m, int closed, int32_t* off, int32_t* nbr, int cap, int* count) {
    return guard([&] {
        BH_REQUIRE(off != nullptr, "offsets pointer is null");
        flatten(square_lists(m, closed != 0), off, nbr, cap, count);
    });
}
int bh_neighbours_cube(int m, int closed, int32_t* off, int32_t* nbr, int cap, int* count) {
    return guard([&] {
        BH_REQUIRE(off != nullptr, "offsets pointer is null");
        flatten(cube_lists(m, closed != 0), off, nbr, cap, count);
    });
}

// ---- basis ----
int bh_dimension(int m, int n, int64_t* dim) {
    return guard([&] {
        BH_REQUIRE(dim != nullptr, "dim pointer is null");
        BH_REQUIRE(m >= 1 && n >= 0, "m must be >= 1 and n >= 0");
        const int64_t d = binomial64(m + n - 1, n);
        BH_REQUIRE(d > 0, "dimension overflows 64 bits");
        *dim = d;
    });
}

int bh_basis_create(int m, int n, bh_basis** out) {
    return guard([&] {
        BH_REQUIRE(out != nullptr, "output pointer is null");
        *out = nullptr;
        BH_REQUIRE(m >= 1 && m <= kMaxSites, "m must be in [1, 25] (the reference's primes table)");
        BH_REQUIRE(n >= 0 && n <= kMaxBosons, "n must be in [0, 60]");
        const int64_t D = binomial64(m + n - 1, n);
        BH_REQUIRE(D > 0 && D <= 2147483647LL, "dimension exceeds 2^31 - 1");
        auto* b = new bh_basis();
        try {
            b->m = m;
            b->n = n;
            b->D = D;
            BH_CUDA(cudaGetDevice(&b->device));
            b->rt = make_rank_table(m, n);
            Stream st;
            basis_build(b, st);
        } catch (...) {
            delete b;
            throw;
        }
        *out = b;
    });
}

int bh_basis_destroy(bh_basis* b) {
    return guard([&] { delete b; });
}

int bh_basis_info(const bh_basis* b, int* m, int* n, int64_t* dim) {
    return guard([&] {
        BH_REQUIRE(b != nullptr, "basis is null");
        if (m) *m = b->m;
        if (n) *n = b->n;
        if (dim) *dim = b->D;
    });
}

int bh_basis_copy(const bh_basis* b, double* tags, double* basis, int32_t* col_of_lex,
                  int32_t* lex_of_col) {
    return guard([&] {
        BH_REQUIRE(b != nullptr, "basis is null");
        const int64_t D = b->D;
        Stream st;
        if (tags || basis) {
            DevBuf<double> dt(tags ? D : 1), db(basis ? D * b->m : 1);
            basis_tags(b, tags ? dt.p : nullptr, basis ? db.p : nullptr, st);
            if (tags) BH_CUDA(cudaMemcpy(tags, dt.p, D * sizeof(double), cudaMemcpyDeviceToHost));
            if (basis) BH_CUDA(cudaMemcpy(basis, db.p, D * b->m * sizeof(double), cudaMemcpyDeviceToHost));
        }
        if (col_of_lex)
            BH_CUDA(cudaMemcpy(col_of_lex, b->d_col_of_lex.p, D * sizeof(int32_t), cudaMemcpyDeviceToHost));
        if (lex_of_col)
            BH_CUDA(cudaMemcpy(lex_of_col, b->d_lex_of_col.p, D * sizeof(int32_t), cudaMemcpyDeviceToHost));
    });
}

int bh_basis_index(const bh_basis* b, int64_t nq, const uint8_t* occ, int32_t* col) {
    return guard([&] {
        BH_REQUIRE(b != nullptr && (nq == 0 || (occ && col)), "null argument");
        if (nq == 0) return;
        Stream st;
        DevBuf<uint8_t> dq((size_t)nq * b->m);
        DevBuf<int32_t> dc(nq);
        BH_CUDA(cudaMemcpyAsync(dq.p, occ, (size_t)nq * b->m, cudaMemcpyHostToDevice, st));
        basis_index(b, nq, dq.p, dc.p, st);
        BH_CUDA(cudaMemcpyAsync(col, dc.p, nq * sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaStreamSynchronize(st));
    });
}

// ---- Hamiltonian ----
static bh_hamiltonian* new_hamiltonian(const bh_basis* b, const int32_t* nbr_off, const int32_t* nbr) {
    BH_REQUIRE(b != nullptr && nbr_off != nullptr, "null argument");
    const int m = b->m;
    BH_REQUIRE(nbr_off[0] == 0, "neighbour offsets must start at 0");
    for (int i = 0; i < m; ++i) BH_REQUIRE(nbr_off[i + 1] >= nbr_off[i], "neighbour offsets must be non-decreasing");
    const int tot = nbr_off[m];
    BH_REQUIRE(tot == 0 || nbr != nullptr, "neighbour list is null");
    std::vector<int> cnt((size_t)m * m, 0);
    for (int i = 0; i < m; ++i)
        for (int k = nbr_off[i]; k < nbr_off[i + 1]; ++k) {
            const int j = nbr[k];
            BH_REQUIRE(j >= 0 && j < m, "neighbour index out of range");
            BH_REQUIRE(j != i, "self-bond in the neighbour list");
            cnt[(size_t)i * m + j] += 1;
        }
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j)
            BH_REQUIRE(cnt[(size_t)i * m + j] == cnt[(size_t)j * m + i], "neighbour lists must be symmetric");
    auto* h = new bh_hamiltonian();
    h->basis = b;
    h->m = m;
    h->n = b->n;
    h->D = b->D;
    h->device = b->device;
    h->h_nbr_off.assign(nbr_off, nbr_off + m + 1);
    h->h_nbr.assign(nbr, nbr + tot);
    return h;
}

int bh_hamiltonian_create(const bh_basis* b, const int32_t* nbr_off, const int32_t* nbr,
                          bh_hamiltonian** out) {
    return guard([&] {
        BH_REQUIRE(out != nullptr, "null argument");
        *out = nullptr;
        bh_hamiltonian* h = new_hamiltonian(b, nbr_off, nbr);
        try {
            Stream st;
            hamiltonian_build(h, st);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int bh_hamiltonian_create_matrix_free(const bh_basis* b, const int32_t* nbr_off, const int32_t* nbr,
                                      bh_hamiltonian** out) {
    return guard([&] {
        BH_REQUIRE(out != nullptr, "null argument");
        *out = nullptr;
        bh_hamiltonian* h = new_hamiltonian(b, nbr_off, nbr);
        try {
            Stream st;
            hamiltonian_build_matrix_free(h, st);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int bh_hamiltonian_is_matrix_free(const bh_hamiltonian* h, int* matrix_free) {
    return guard([&] {
        BH_REQUIRE(h != nullptr && matrix_free != nullptr, "null argument");
        *matrix_free = h->matrix_free ? 1 : 0;
    });
}

int bh_hamiltonian_destroy(bh_hamiltonian* h) {
    return guard([&] { delete h; });
}

int bh_hamiltonian_nnz(const bh_hamiltonian* h, int64_t* nnz) {
    return guard([&] {
        BH_REQUIRE(h != nullptr && nnz != nullptr, "null argument");
        *nnz = h->nnz;
    });
}

int bh_hamiltonian_csr(const bh_hamiltonian* h, int order, double J, double U, double mu,
                       int64_t* row_ptr, int32_t* col, double* val) {
    return guard([&] {
        BH_REQUIRE(h != nullptr && row_ptr && col && val, "null argument");
        BH_REQUIRE(order == BH_ORDER_REFERENCE || order == BH_ORDER_LEX, "unknown order");
        require_finite_params(J, U, mu);
        const int64_t D = h->D, nz = h->nnz + D;
        Stream st;
        DevBuf<int64_t> rp(D + 1);
        DevBuf<int32_t> ci(nz);
        DevBuf<double> v(nz);
        hamiltonian_csr(h, order, J, U, mu, rp.p, ci.p, v.p, st);
        BH_CUDA(cudaMemcpy(row_ptr, rp.p, (D + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost));
        BH_CUDA(cudaMemcpy(col, ci.p, nz * sizeof(int32_t), cudaMemcpyDeviceToHost));
        BH_CUDA(cudaMemcpy(val, v.p, nz * sizeof(double), cudaMemcpyDeviceToHost));
    });
}

int bh_hamiltonian_multi_csr(int nh, const bh_hamiltonian* const* hs, int order, double J, double U,
                             double mu, int64_t* row_ptr, int32_t* col, double* val) {
    return guard([&] {
        BH_REQUIRE(nh >= 1 && hs && row_ptr && col && val, "null argument or nh < 1");
        BH_REQUIRE(order == BH_ORDER_REFERENCE || order == BH_ORDER_LEX, "unknown order");
        require_finite_params(J, U, mu);
        int64_t D = 0, nz = 0;
        for (int k = 0; k < nh; ++k) {
            BH_REQUIRE(hs[k] != nullptr, "null Hamiltonian");
            BH_REQUIRE(k == 0 || hs[k]->device == hs[0]->device, "Hamiltonians on different devices");
            D += hs[k]->D;
            nz += hs[k]->nnz + hs[k]->D;
        }
        BH_REQUIRE(D <= 2147483647LL, "combined dimension exceeds 2^31 - 1");
        Stream st;
        DevBuf<int64_t> rp(D + 1);
        DevBuf<int32_t> ci(nz);
        DevBuf<double> v(nz);
        hamiltonian_multi_csr(nh, hs, order, J, U, mu, rp.p, ci.p, v.p, st);
        BH_CUDA(cudaMemcpy(row_ptr, rp.p, (D + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost));
        BH_CUDA(cudaMemcpy(col, ci.p, nz * sizeof(int32_t), cudaMemcpyDeviceToHost));
        BH_CUDA(cudaMemcpy(val, v.p, nz * sizeof(double), cudaMemcpyDeviceToHost));
    });
}

static OpView<double> op64_of(const bh_hamiltonian* h) { return op_view<double>(h); }
static OpView<float> op32_of(const bh_hamiltonian* h) { return op_view<float>(h); }

int bh_hamiltonian_apply(const bh_hamiltonian* h, int order, double J, double U, double mu,
                         int nvec, const double* x, double* y) {
    return guard([&] {
        BH_REQUIRE(h != nullptr && x && y && nvec >= 1, "null argument");
        require_finite_params(J, U, mu);
        const int64_t D = h->D;
        Stream st;
        DevBuf<double> dx(D * nvec), dy(D * nvec), tmp(D * nvec), prm(3);
        const double hp[3] = {J, U, -mu * (double)h->n};
        BH_CUDA(cudaMemcpyAsync(prm.p, hp, sizeof hp, cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaMemcpyAsync(dx.p, x, D * nvec * sizeof(double), cudaMemcpyHostToDevice, st));
        const bool ref = order == BH_ORDER_REFERENCE;
        if (ref) gather_rows(D, nvec, h->basis->d_col_of_lex.p, dx.p, tmp.p, st);
        apply_operator(op64_of(h), nvec, nvec, prm.p, ref ? tmp.p : dx.p, dy.p, st);
        if (ref) gather_rows(D, nvec, h->basis->d_lex_of_col.p, dy.p, tmp.p, st);
        BH_CUDA(cudaMemcpyAsync(y, ref ? tmp.p : dy.p, D * nvec * sizeof(double), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaStreamSynchronize(st));
    });
}

// ---- eigensolver ----
void bh_solver_opts_default(bh_solver_opts* o) {
    if (!o) return;
    o->nev = 10;
    o->ncv = 0;
    o->block = 0;
    o->precision = BH_PREC_FP64;
    o->max_restarts = 1000;
    o->tol = 0.0;
    o->seed = 0;
    o->want_vectors = 0;
    o->order = BH_ORDER_REFERENCE;
}

static void write_vectors(const bh_hamiltonian* h, const SolveResult& r, int S, int nev, int order,
                          double* evecs) {
    if (!evecs) return;
    const int64_t D = h->D;
    if (order == BH_ORDER_LEX) {
        std::memcpy(evecs, r.vecs.data(), (size_t)S * nev * D * sizeof(double));
        return;
    }
    const std::vector<int32_t> col = host_copy_i32(h->basis->d_col_of_lex.p, D);
    for (int k = 0; k < S * nev; ++k)
        for (int64_t rr = 0; rr < D; ++rr) evecs[(size_t)k * D + col[rr]] = r.vecs[(size_t)k * D + rr];
}

static void batch_solve(const bh_hamiltonian* h, int nsolve, const double* J, const double* U,
                        const double* mu, const bh_solver_opts* o, double* evals, double* resid,
                        int* nconv, int* status, double* evecs, bh_solve_info* info) {
    const auto t0 = std::chrono::steady_clock::now();
    BH_REQUIRE(h != nullptr && J && U && mu && evals, "null argument");
    BH_REQUIRE(nsolve >= 1, "nsolve must be >= 1");
    check_solver_opts(o);
    require_finite(J, nsolve, "J");
    require_finite(U, nsolve, "U");
    require_finite(mu, nsolve, "mu");
    SolveRequest rq = make_request(o, h->D, nsolve);
    rq.want_vectors = evecs != nullptr;
    rq.d_perm = h->basis->d_col_of_lex.p;
    rq.J.assign(J, J + nsolve);
    rq.U.assign(U, U + nsolve);
    rq.shift.resize(nsolve);
    for (int s = 0; s < nsolve; ++s) rq.shift[s] = -mu[s] * (double)h->n;
    Stream st;
    SolveResult r = block_lanczos(op64_of(h), op32_of(h), rq, st);
    std::memcpy(evals, r.evals.data(), r.evals.size() * sizeof(double));
    if (resid) std::memcpy(resid, r.resid.data(), r.resid.size() * sizeof(double));
    if (nconv) std::memcpy(nconv, r.nconv.data(), nsolve * sizeof(int));
    if (status)
        for (int s = 0; s < nsolve; ++s)
            status[s] = r.status[s] != BH_OK ? r.status[s] : (r.nconv[s] < o->nev ? BH_ERR_NOCONV : BH_OK);
    if (evecs) write_vectors(h, r, nsolve, o->nev, o->order, evecs);
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    fill_info(info, r, o->nev, secs);
}

int bh_eigsh_batch(const bh_hamiltonian* h, int nsolve, const double* J, const double* U,
                   const double* mu, const bh_solver_opts* o, double* evals, double* resid,
                   int* nconv, bh_solve_info* info) {
    return guard([&] { batch_solve(h, nsolve, J, U, mu, o, evals, resid, nconv, nullptr, nullptr, info); });
}

int bh_eigsh_batch_status(const bh_hamiltonian* h, int nsolve, const double* J, const double* U,
                          const double* mu, const bh_solver_opts* o, double* evals, double* resid,
                          int* nconv, int* status, bh_solve_info* info) {
    return guard([&] {
        BH_REQUIRE(status != nullptr, "null argument");
        batch_solve(h, nsolve, J, U, mu, o, evals, resid, nconv, status, nullptr, info);
    });
}

int bh_eigsh_batch_vectors(const bh_hamiltonian* h, int nsolve, const double* J, const double* U,
                           const double* mu, const bh_solver_opts* o, double* evals, double* resid,
                           int* nconv, double* evecs, bh_solve_info* info) {
    return guard([&] {
        BH_REQUIRE(evecs != nullptr, "null argument");
        batch_solve(h, nsolve, J, U, mu, o, evals, resid, nconv, nullptr, evecs, info);
    });
}

int bh_eigsh_batch_sectors(int nh, const bh_hamiltonian* const* hs, int nsolve, const double* J,
                           const double* U, const double* mu, const bh_solver_opts* o, double* evals,
                           double* resid, int* nconv, bh_solve_info* info) {
    return guard([&] {
        const auto t0 = std::chrono::steady_clock::now();
        BH_REQUIRE(nh >= 1 && hs && J && U && mu && evals, "null argument or nh < 1");
        BH_REQUIRE(nsolve >= 1, "nsolve must be >= 1");
        check_solver_opts(o);
        require_finite(J, nsolve, "J");
        require_finite(U, nsolve, "U");
        require_finite(mu, nsolve, "mu");
        for (int k = 0; k < nh; ++k) BH_REQUIRE(hs[k] != nullptr, "null Hamiltonian");
        int dev = 0;
        BH_CUDA(cudaGetDevice(&dev));
        const int nev = o->nev;
        std::vector<SolveResult> res(nh);
        std::vector<int> codes(nh, BH_OK);
        std::vector<std::string> msgs(nh);
        // one host thread per sector, each with its own stream: the sectors'
        // kernels overlap on the device, and one sector's restart work on the
        // host (or its slowest last solve) leaves the GPU to the others
        auto work = [&](int k) {
            try {
                BH_CUDA(cudaSetDevice(dev));
                const bh_hamiltonian* h = hs[k];
                SolveRequest rq = make_request(o, h->D, nsolve);
                rq.want_vectors = false;
                rq.d_perm = h->basis->d_col_of_lex.p;
                rq.J.assign(J, J + nsolve);
                rq.U.assign(U, U + nsolve);
                rq.shift.resize(nsolve);
                for (int s = 0; s < nsolve; ++s) rq.shift[s] = -mu[s] * (double)h->n;
                Stream st;
                res[k] = block_lanczos(op64_of(h), op32_of(h), rq, st);
            } catch (const Error& e) {
                codes[k] = e.code;
                msgs[k] = e.what();
            } catch (const std::bad_alloc&) {
                codes[k] = BH_ERR_NOMEM;
                msgs[k] = "host allocation failed";
            } catch (const std::exception& e) {
                codes[k] = BH_ERR_CUDA;
                msgs[k] = e.what();
            }
        };
        if (nh == 1 || profile_on()) {
            for (int k = 0; k < nh; ++k) work(k);  // per-kernel timing wants no overlap
        } else {
            std::vector<std::thread> th;
            for (int k = 0; k < nh; ++k) th.emplace_back(work, k);
            for (auto& t : th) t.join();
        }
        for (int k = 0; k < nh; ++k)
            if (codes[k] != BH_OK) throw Error(codes[k], "sector " + std::to_string(k) + ": " + msgs[k]);
        SolveResult agg;
        for (int k = 0; k < nh; ++k) {
            const SolveResult& r = res[k];
            std::memcpy(evals + (size_t)k * nsolve * nev, r.evals.data(), r.evals.size() * sizeof(double));
            if (resid) std::memcpy(resid + (size_t)k * nsolve * nev, r.resid.data(), r.resid.size() * sizeof(double));
            if (nconv) std::memcpy(nconv + (size_t)k * nsolve, r.nconv.data(), nsolve * sizeof(int));
            agg.nconv.insert(agg.nconv.end(), r.nconv.begin(), r.nconv.end());
            agg.resid.insert(agg.resid.end(), r.resid.begin(), r.resid.end());
            agg.restarts = std::max(agg.restarts, r.restarts);
            agg.matvecs += r.matvecs;
            agg.launches += r.launches;
        }
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        fill_info(info, agg, nev, secs);
    });
}

int bh_eigsh(const bh_hamiltonian* h, double J, double U, double mu, const bh_solver_opts* o,
             double* evals, double* resid, double* evecs, bh_solve_info* info) {
    return guard([&] {
        const auto t0 = std::chrono::steady_clock::now();
        BH_REQUIRE(h != nullptr && evals, "null argument");
        check_solver_opts(o);
        require_finite_params(J, U, mu);
        SolveRequest rq = make_request(o, h->D, 1);
        rq.want_vectors = evecs != nullptr;
        rq.d_perm = h->basis->d_col_of_lex.p;
        rq.J = {J};
        rq.U = {U};
        rq.shift = {-mu * (double)h->n};
        Stream st;
        SolveResult r = block_lanczos(op64_of(h), op32_of(h), rq, st);
        std::memcpy(evals, r.evals.data(), o->nev * sizeof(double));
        if (resid) std::memcpy(resid, r.resid.data(), o->nev * sizeof(double));
        write_vectors(h, r, 1, o->nev, o->order, evecs);
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        fill_info(info, r, o->nev, secs);
        throw_if_failed(r, o->nev);
    });
}

int bh_eigsh_csr(int64_t dim, const int64_t* row_ptr, const int32_t* col, const double* val,
                 const bh_solver_opts* o, double* evals, double* resid, double* evecs,
                 bh_solve_info* info) {
    return guard([&] {
        const auto t0 = std::chrono::steady_clock::now();
        BH_REQUIRE(dim >= 1 && dim <= 2147483647LL, "dimension out of range");
        BH_REQUIRE(row_ptr && col && val && evals, "null argument");
        BH_REQUIRE(row_ptr[0] == 0, "row_ptr[0] must be 0");
        check_solver_opts(o);
        const int64_t nnz = row_ptr[dim];
        for (int64_t r = 0; r < dim; ++r) BH_REQUIRE(row_ptr[r + 1] >= row_ptr[r], "row_ptr must be non-decreasing");
        for (int64_t e = 0; e < nnz; ++e) BH_REQUIRE(col[e] >= 0 && col[e] < dim, "column index out of range");
        require_finite(val, nnz, "matrix values");
        Stream st;
        DevBuf<int64_t> rp(dim + 1);
        DevBuf<int32_t> ci(nnz);
        DevBuf<double> v64(nnz);
        DevBuf<float> v32;
        std::vector<float> hv32;
        BH_CUDA(cudaMemcpyAsync(rp.p, row_ptr, (dim + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        if (nnz) {
            BH_CUDA(cudaMemcpyAsync(ci.p, col, nnz * sizeof(int32_t), cudaMemcpyHostToDevice, st));
            BH_CUDA(cudaMemcpyAsync(v64.p, val, nnz * sizeof(double), cudaMemcpyHostToDevice, st));
        }
        if (o->precision == BH_PREC_MIXED) {
            hv32.resize(nnz);
            for (int64_t e = 0; e < nnz; ++e) hv32[e] = (float)val[e];
            v32.alloc(nnz);
            if (nnz) BH_CUDA(cudaMemcpyAsync(v32.p, hv32.data(), nnz * sizeof(float), cudaMemcpyHostToDevice, st));
        }
        OpView<double> a64;
        a64.rp = rp.p;
        a64.ci = ci.p;
        a64.tv = v64.p;
        a64.D = dim;
        a64.rp_nnz = nnz;
        OpView<float> a32;
        a32.rp = rp.p;
        a32.ci = ci.p;
        a32.tv = v32.p;
        a32.D = dim;
        a32.rp_nnz = nnz;
        SolveRequest rq = make_request(o, dim, 1);
        rq.want_vectors = evecs != nullptr;
        rq.J = {1.0};
        rq.U = {0.0};
        rq.shift = {0.0};
        SolveResult r = block_lanczos(a64, a32, rq, st);
        std::memcpy(evals, r.evals.data(), o->nev * sizeof(double));
        if (resid) std::memcpy(resid, r.resid.data(), o->nev * sizeof(double));
        if (evecs) std::memcpy(evecs, r.vecs.data(), (size_t)o->nev * dim * sizeof(double));
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        fill_info(info, r, o->nev, secs);
        throw_if_failed(r, o->nev);
    });
}

int bh_folm_diag_csr(int64_t dim, const int64_t* row_ptr, const int32_t* col, const double* val, int nb_iter,
                     double* v0, double* T, double* V, int* steps) {
    return guard([&] {
        BH_REQUIRE(dim >= 1 && dim <= 2147483647LL, "dimension out of range");
        BH_REQUIRE(row_ptr && col && val && v0 && T && V, "null argument");
        BH_REQUIRE(nb_iter >= 1 && nb_iter <= dim, "nb_iter must be in [1, dimension]");
        BH_REQUIRE(row_ptr[0] == 0, "row_ptr[0] must be 0");
        const int64_t nnz = row_ptr[dim];
        for (int64_t r = 0; r < dim; ++r) BH_REQUIRE(row_ptr[r + 1] >= row_ptr[r], "row_ptr must be non-decreasing");
        for (int64_t e = 0; e < nnz; ++e) BH_REQUIRE(col[e] >= 0 && col[e] < dim, "column index out of range");
        require_finite(val, nnz, "matrix values");
        require_finite(v0, dim, "start vector");
        double n2 = 0.0;
        for (int64_t r = 0; r < dim; ++r) n2 += v0[r] * v0[r];
        BH_REQUIRE(n2 > 0.0, "start vector is zero");
        // the reference normalises the caller's v_0 in place (operator.cpp:43)
        const double inv = 1.0 / std::sqrt(n2);
        for (int64_t r = 0; r < dim; ++r) v0[r] *= inv;
        Stream st;
        DevBuf<int64_t> rp(dim + 1);
        DevBuf<int32_t> ci(nnz);
        DevBuf<double> v64(nnz);
        BH_CUDA(cudaMemcpyAsync(rp.p, row_ptr, (dim + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        if (nnz) {
            BH_CUDA(cudaMemcpyAsync(ci.p, col, nnz * sizeof(int32_t), cudaMemcpyHostToDevice, st));
            BH_CUDA(cudaMemcpyAsync(v64.p, val, nnz * sizeof(double), cudaMemcpyHostToDevice, st));
        }
        OpView<double> a64;
        a64.rp = rp.p;
        a64.ci = ci.p;
        a64.tv = v64.p;
        a64.D = dim;
        a64.rp_nnz = nnz;
        const int k = folm_diag(a64, nb_iter, v0, T, V, st);
        if (steps) *steps = k;
    });
}

int bh_dense_eigh(int64_t n, const double* a, double* w, double* z) {
    return guard([&] {
        BH_REQUIRE(a && w, "null argument");
        dense_eigh(n, a, w, z);
    });
}

// ---- observables ----
int bh_gap_ratios(int nev, const double* evals, double* ratios, double* mean) {
    return guard([&] {
        BH_REQUIRE(nev >= 0 && (nev == 0 || evals), "null argument");
        std::vector<double> s(evals, evals + nev);
        std::sort(s.begin(), s.end());
        double sum = 0.0;
        for (int i = 1; i + 1 < nev; ++i) {
            const double up = s[i + 1] - s[i], dn = s[i] - s[i - 1];
            const double mn = std::min(up, dn), mx = std::max(up, dn);
            const double r = mx != 0.0 ? mn / mx : 0.0;
            if (ratios) ratios[i - 1] = r;
            sum += r;
        }
        if (mean) *mean = nev > 2 ? sum / (nev - 2) : 0.0;
    });
}

int bh_spdm(const bh_hamiltonian* h, int order, const double* phi, double* rho) {
    return guard([&] {
        BH_REQUIRE(h != nullptr && phi && rho, "null argument");
        const int64_t D = h->D;
        Stream st;
        DevBuf<double> dp(D), dl(D), dr((size_t)h->m * h->m);
        BH_CUDA(cudaMemcpyAsync(dp.p, phi, D * sizeof(double), cudaMemcpyHostToDevice, st));
        const double* lex = dp.p;
        if (order == BH_ORDER_REFERENCE) {
            gather_rows(D, 1, h->basis->d_col_of_lex.p, dp.p, dl.p, st);
            lex = dl.p;
        }
        spdm_device(h, lex, dr.p, st);
        BH_CUDA(cudaMemcpyAsync(rho, dr.p, (size_t)h->m * h->m * sizeof(double), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaStreamSynchronize(st));
    });
}

int bh_phase_map(int m, int n_lo, int nsec, int nJ, const double* e0, int nmu, const double* mu,
                 double* density, double* compressibility) {
    return guard([&] {
        BH_REQUIRE(m >= 1 && nsec >= 1 && nJ >= 1 && nmu >= 1, "empty grid");
        BH_REQUIRE(e0 && mu && density && compressibility, "null argument");
        require_finite(e0, (int64_t)nsec * nJ, "e0");
        require_finite(mu, nmu, "mu");
        Stream st;
        DevBuf<double> de((size_t)nsec * nJ), dm(nmu), dd((size_t)nJ * nmu), dk((size_t)nJ * nmu);
        BH_CUDA(cudaMemcpyAsync(de.p, e0, (size_t)nsec * nJ * sizeof(double), cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaMemcpyAsync(dm.p, mu, nmu * sizeof(double), cudaMemcpyHostToDevice, st));
        phase_map_device(m, n_lo, nsec, nJ, de.p, nmu, dm.p, dd.p, dk.p, st);
        BH_CUDA(cudaMemcpyAsync(density, dd.p, (size_t)nJ * nmu * sizeof(double), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaMemcpyAsync(compressibility, dk.p, (size_t)nJ * nmu * sizeof(double), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaStreamSynchronize(st));
    });
}

// ---- launch shapes of the sparse product and the autotuner ----
// cols_per_lane < 0 in the C ABI: -VW adjacent columns per lane (the
// contiguous-column product)
static SpmmShape shape_in(const bh_spmm_shape& s) {
    SpmmShape o;
    o.L = s.lanes;
    o.CW = s.cols_per_lane > 0 ? s.cols_per_lane : 0;
    o.VW = s.cols_per_lane < 0 ? -s.cols_per_lane : 0;
    o.grid = s.grid;
    return o;
}

static bh_spmm_shape shape_out(const SpmmShape& s) {
    bh_spmm_shape o;
    o.lanes = s.L;
    o.cols_per_lane = s.VW > 0 ? -s.VW : s.CW;
    o.grid = s.grid;
    return o;
}

int bh_spmm_candidates(int nvec, int matrix_free, bh_spmm_shape* out, int cap, int* count) {
    return guard([&] {
        BH_REQUIRE(nvec >= 1 && count, "null argument or nvec < 1");
        const bool mf = matrix_free != 0;
        const std::vector<SpmmChoice> c = spmm_candidates(nvec, mf);
        BH_REQUIRE(cap >= (int)c.size() && out, "output capacity too small");
        for (size_t i = 0; i < c.size(); ++i) out[i] = shape_out(spmm_resolve(c[i], nvec, mf));
        *count = (int)c.size();
    });
}

int bh_hamiltonian_apply_shape(const bh_hamiltonian* h, int precision, double J, double U,
                               double mu, int nvec, const bh_spmm_shape* shape, const double* x,
                               double* y) {
    return guard([&] {
        BH_REQUIRE(h != nullptr && x && y && nvec >= 1, "null argument");
        BH_REQUIRE(precision == BH_PREC_FP64 || precision == BH_PREC_MIXED, "unknown precision mode");
        require_finite_params(J, U, mu);
        const SpmmShape s = shape ? shape_in(*shape) : spmm_resolve(SpmmChoice{}, nvec, h->matrix_free);
        BH_REQUIRE(spmm_shape_valid(s, nvec, h->matrix_free),
                   "launch shape: lanes must be a power of two <= 32 dividing nvec (32 at any nvec "
                   "for a matrix-free operator), columns per lane 1 or 4 (or 2 with 32 lanes), "
                   "grid >= -1");
        const int64_t D = h->D, n = D * nvec;
        Stream st;
        DevBuf<double> dx(n), dy(n), prm(3);
        const double hp[3] = {J, U, -mu * (double)h->n};
        BH_CUDA(cudaMemcpyAsync(prm.p, hp, sizeof hp, cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaMemcpyAsync(dx.p, x, n * sizeof(double), cudaMemcpyHostToDevice, st));
        if (precision == BH_PREC_FP64) {
            launch_spmm_shape<double>(op64_of(h), nvec, nvec, prm.p, dx.p, dy.p, st, s);
        } else {
            DevBuf<float> fx(n), fy(n);
            cast_f64_f32(n, dx.p, fx.p, st);
            launch_spmm_shape<float>(op32_of(h), nvec, nvec, prm.p, fx.p, fy.p, st, s);
            cast_f32_f64(n, fy.p, dy.p, st);
        }
        BH_CUDA(cudaGetLastError());
        BH_CUDA(cudaMemcpyAsync(y, dy.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaStreamSynchronize(st));
    });
}

int bh_spmm_autotune(const bh_hamiltonian* h, int nvec, int precision, bh_spmm_shape* chosen,
                     float* ms, float* ms_default) {
    return guard([&] {
        BH_REQUIRE(h != nullptr && nvec >= 1, "null argument or nvec < 1");
        BH_REQUIRE(precision == BH_PREC_FP64 || precision == BH_PREC_MIXED, "unknown precision mode");
        const int64_t D = h->D, n = D * nvec;
        Stream st;
        DevBuf<double> prm(3);
        const double hp[3] = {1.0, 1.0, 0.0};
        BH_CUDA(cudaMemcpyAsync(prm.p, hp, sizeof hp, cudaMemcpyHostToDevice, st));
        TuneEntry e;
        if (precision == BH_PREC_FP64) {
            DevBuf<double> X(n), Y(n);
            BH_CUDA(cudaMemsetAsync(X.p, 0, n * sizeof(double), st));
            tune_spmm<double>(op64_of(h), nvec, nvec, prm.p, X.p, Y.p, st, false, true, &e);
            BH_CUDA(cudaStreamSynchronize(st));
        } else {
            DevBuf<float> X(n), Y(n);
            BH_CUDA(cudaMemsetAsync(X.p, 0, n * sizeof(float), st));
            tune_spmm<float>(op32_of(h), nvec, nvec, prm.p, X.p, Y.p, st, false, true, &e);
            BH_CUDA(cudaStreamSynchronize(st));
        }
        if (chosen) *chosen = shape_out(e.shape);
        if (ms) *ms = e.ms;
        if (ms_default) *ms_default = e.ms_default;
    });
}

int bh_spmm_tuning_count(int* n) {
    return guard([&] {
        BH_REQUIRE(n != nullptr, "null argument");
        *n = (int)tune_table().size();
    });
}

int bh_spmm_tuning_get(int i, bh_spmm_tuning* out) {
    return guard([&] {
        BH_REQUIRE(out != nullptr, "null argument");
        const auto t = tune_table();
        BH_REQUIRE(i >= 0 && i < (int)t.size(), "tuning entry index out of range");
        const TuneKey& k = t[(size_t)i].first;
        const TuneEntry& e = t[(size_t)i].second;
        out->matrix_free = k.mf;
        out->elem_bytes = k.elem;
        out->dim = k.D;
        out->nnz = k.nnz;
        out->ncols = e.ncols;
        out->shape = shape_out(e.shape);
        out->ms = e.ms;
        out->ms_default = e.ms_default;
        out->candidates = e.candidates;
    });
}

int bh_spmm_tuning_reset(void) {
    return guard([&] { tune_reset(); });
}

}  // extern "C"


// ---- mean field ----
int bh_scmf(int npts, const double* mu, const double* J, int q, const double* psi0, int precision,
            double* psi, int* iters) {
    return guard([&] {
        BH_REQUIRE(npts >= 0, "npts must be >= 0");
        BH_REQUIRE(npts == 0 || (mu && J && psi0 && psi), "null argument");
        BH_REQUIRE(q >= 0 && precision >= 0 && precision <= 15, "q must be >= 0 and precision in [0, 15]");
        if (npts == 0) return;
        Stream st;
        DevBuf<double> dm(npts), dj(npts), dp0(npts), dp(npts);
        DevBuf<int> di(npts);
        BH_CUDA(cudaMemcpyAsync(dm.p, mu, npts * sizeof(double), cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaMemcpyAsync(dj.p, J, npts * sizeof(double), cudaMemcpyHostToDevice, st));
        BH_CUDA(cudaMemcpyAsync(dp0.p, psi0, npts * sizeof(double), cudaMemcpyHostToDevice, st));
        scmf_device(npts, dm.p, dj.p, q, dp0.p, precision, 20000, dp.p, di.p, st);
        BH_CUDA(cudaMemcpyAsync(psi, dp.p, npts * sizeof(double), cudaMemcpyDeviceToHost, st));
        std::vector<int> hi(npts);
        BH_CUDA(cudaMemcpyAsync(hi.data(), di.p, npts * sizeof(int), cudaMemcpyDeviceToHost, st));
        BH_CUDA(cudaStreamSynchronize(st));
        if (iters) std::memcpy(iters, hi.data(), npts * sizeof(int));
    });
}

// uniform [0, 1) from splitmix64 of (seed, k)
static double mf_seed_value(uint64_t seed, uint64_t k) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ull * (k + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

int bh_mean_field_grid(int n, int precision, int q, uint64_t seed, int* nmu, int* nJ,
                       double* mu_out, double* J_out, double* psi_out) {
    return guard([&] {
        BH_REQUIRE(n >= 1 && nmu && nJ && mu_out && J_out && psi_out, "null argument or n < 1");
        // the reference's loops: x = x_min, x += dx while x < x_max (analysis.cpp:60-79)
        const double J_min = 0.0, J_max = 0.25, mu_min = 0.0, mu_max = 4.0;
        const double dJ = (J_max - J_min) / n, dmu = (mu_max - mu_min) / n;
        std::vector<double> mus, Js;
        for (double x = mu_min; x < mu_max; x += dmu) mus.push_back(x);
        for (double x = J_min; x < J_max; x += dJ) Js.push_back(x);
        BH_REQUIRE((int)mus.size() <= n + 1 && (int)Js.size() <= n + 1, "grid longer than n + 1");
        const int a = (int)mus.size(), b = (int)Js.size();
        std::vector<double> pm((size_t)a * b), pj((size_t)a * b), p0((size_t)a * b);
        for (int i = 0; i < a; ++i)
            for (int k = 0; k < b; ++k) {
                const size_t idx = (size_t)i * b + k;
                pm[idx] = mus[i];
                pj[idx] = Js[k];
                p0[idx] = mf_seed_value(seed, idx);
            }
        std::vector<int> it((size_t)a * b);
        const int rc = bh_scmf(a * b, pm.data(), pj.data(), q, p0.data(), precision, psi_out, it.data());
        if (rc != BH_OK) throw Error(rc, bh_last_error());
        std::memcpy(mu_out, mus.data(), a * sizeof(double));
        std::memcpy(J_out, Js.data(), b * sizeof(double));
        *nmu = a;
        *nJ = b;
    });
}
