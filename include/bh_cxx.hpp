// bh_cxx.hpp -- Eigen-free C++ layer over the C ABI (bh_gb300.h): owning
// handles, the reference's exception conventions, and the eigensolve of a
// symmetric CSR matrix with the result order of Op::IRLM_eigen.
//
// bh_reference_api.hpp (the Eigen-typed drop-in for the reference's
// hamiltonian.cpp / neighbours.cpp / operator.cpp) is built on these pieces;
// they are usable on their own by C++ callers without Eigen.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "bh_gb300.h"

namespace bhgb {

// Status code -> the exception the reference throws: std::runtime_error(
// "Eigenvalue computation failed.") for a solve that does not converge
// (operator.cpp:28), std::invalid_argument for invalid arguments
// (neighbours.cpp:43, Spectra GenEigsBase.h:335-339), std::runtime_error
// (the library's message) otherwise.
inline void check(int rc) {
    if (rc == BH_OK) return;
    const std::string msg = bh_last_error();
    if (rc == BH_ERR_NOCONV) throw std::runtime_error("Eigenvalue computation failed.");
    if (rc == BH_ERR_ARG) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

inline void flatten(const std::vector<std::vector<int>>& nb, std::vector<int32_t>& off,
                    std::vector<int32_t>& flat) {
    off.assign(nb.size() + 1, 0);
    flat.clear();
    for (size_t i = 0; i < nb.size(); ++i) {
        for (int j : nb[i]) flat.push_back(j);
        off[i + 1] = (int32_t)flat.size();
    }
    if (flat.empty()) flat.push_back(0);
}

// Neighbour lists from one of bh_neighbours_chain / _square / _cube.
template <class F>
std::vector<std::vector<int>> lattice(int m, bool closed, F fn) {
    std::vector<int32_t> off(m + 1);
    int count = 0;
    check(fn(m, closed ? 1 : 0, off.data(), nullptr, 0, &count));
    std::vector<int32_t> flat(count > 0 ? count : 1);
    check(fn(m, closed ? 1 : 0, off.data(), flat.data(), (int)flat.size(), &count));
    std::vector<std::vector<int>> out(m);
    for (int i = 0; i < m; ++i) out[i].assign(flat.begin() + off[i], flat.begin() + off[i + 1]);
    return out;
}

// owning wrappers of the C handles
struct Basis {
    bh_basis* p = nullptr;
    Basis(int m, int n) { check(bh_basis_create(m, n, &p)); }
    ~Basis() { bh_basis_destroy(p); }
    Basis(const Basis&) = delete;
    Basis& operator=(const Basis&) = delete;
    int64_t dim() const {
        int64_t d = 0;
        check(bh_basis_info(p, nullptr, nullptr, &d));
        return d;
    }
};

struct Hamiltonian {
    bh_hamiltonian* p = nullptr;
    Hamiltonian(const Basis& b, const std::vector<std::vector<int>>& nb) {
        std::vector<int32_t> off, flat;
        flatten(nb, off, flat);
        check(bh_hamiltonian_create(b.p, off.data(), flat.data(), &p));
    }
    ~Hamiltonian() { bh_hamiltonian_destroy(p); }
    Hamiltonian(const Hamiltonian&) = delete;
    Hamiltonian& operator=(const Hamiltonian&) = delete;
};

// A symmetric matrix in compressed rows (for a symmetric matrix the same
// arrays as Eigen's compressed columns).
struct Csr {
    int64_t dim = 0;
    std::vector<int64_t> rp;
    std::vector<int32_t> ci;
    std::vector<double> val;
};

// H = J T + U V - mu N of a built Hamiltonian, in the reference's column order.
inline Csr hamiltonian_csr(const Basis& b, const Hamiltonian& h, double J, double U, double mu) {
    Csr c;
    c.dim = b.dim();
    int64_t nnz = 0;
    check(bh_hamiltonian_nnz(h.p, &nnz));
    c.rp.resize(c.dim + 1);
    c.ci.resize(nnz + c.dim);
    c.val.resize(nnz + c.dim);
    check(bh_hamiltonian_csr(h.p, BH_ORDER_REFERENCE, J, U, mu, c.rp.data(), c.ci.data(), c.val.data()));
    return c;
}

// Lowest nev eigenpairs of a symmetric CSR matrix (FP64, the plain method),
// ascending; vec[k * dim + r] is component r of vector k.  max_restarts and
// ncv: 0 = the library's defaults.
inline void eigsh(const Csr& O, int nev, std::vector<double>& ev, std::vector<double>& vec,
                  int max_restarts = 0, int ncv = 0) {
    bh_solver_opts o;
    bh_solver_opts_default(&o);
    o.nev = nev;
    o.want_vectors = 1;
    o.order = BH_ORDER_LEX;  // the caller's own order (identity map)
    if (max_restarts > 0) o.max_restarts = max_restarts;
    if (ncv > 0) o.ncv = ncv;
    ev.assign(nev, 0.0);
    vec.assign((size_t)nev * O.dim, 0.0);
    bh_solve_info info;
    std::vector<int32_t> ci(O.ci);
    std::vector<double> val(O.val);
    if (ci.empty()) {
        ci.push_back(0);
        val.push_back(0.0);
    }
    check(bh_eigsh_csr(O.dim, O.rp.data(), ci.data(), val.data(), &o, ev.data(), nullptr, vec.data(), &info));
}

// Op::IRLM_eigen's result convention (operator.cpp:22-33 with Spectra's
// LargestMagn output order, GenEigsBase.h:417, 466-483): the nev lowest
// eigenvalues ordered by descending magnitude, ties kept in ascending order;
// vec rows follow the same order.  Throws like the reference:
// std::invalid_argument for nev outside [1, n - 2], std::runtime_error(
// "Eigenvalue computation failed.") when the solve does not converge.
inline void irlm_eigen(const Csr& O, int nev, std::vector<double>& vals, std::vector<double>& vec,
                       int max_restarts = 0, int ncv = 0) {
    if (nev < 1 || nev > O.dim - 2)
        throw std::invalid_argument("nev must satisfy 1 <= nev <= n - 2, n is the size of matrix");
    std::vector<double> ev, v;
    eigsh(O, nev, ev, v, max_restarts, ncv);
    std::vector<int> ord(nev);
    for (int i = 0; i < nev; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return std::fabs(ev[a]) > std::fabs(ev[b]); });
    vals.resize(nev);
    vec.resize((size_t)nev * O.dim);
    for (int k = 0; k < nev; ++k) {
        vals[k] = ev[ord[k]];
        std::copy(v.begin() + (size_t)ord[k] * O.dim, v.begin() + (size_t)(ord[k] + 1) * O.dim,
                  vec.begin() + (size_t)k * O.dim);
    }
}

// Op::FOLM_diag (operator.cpp:39-71): nb_iter Lanczos steps of O from v0
// (normalised in place) with full re-orthogonalisation; T (nb_iter x nb_iter)
// and V (O.dim x nb_iter), both column-major, receive the tridiagonal matrix
// and the Krylov vectors.  Returns the number of vectors.
inline int folm_diag(const Csr& O, int nb_iter, std::vector<double>& v0, std::vector<double>& T,
                     std::vector<double>& V) {
    if (nb_iter < 1 || nb_iter > O.dim) throw std::invalid_argument("nb_iter must satisfy 1 <= nb_iter <= n");
    if ((int64_t)v0.size() != O.dim) throw std::invalid_argument("v_0 must have the size of the matrix");
    T.assign((size_t)nb_iter * nb_iter, 0.0);
    V.assign((size_t)nb_iter * O.dim, 0.0);
    std::vector<int32_t> ci(O.ci);
    std::vector<double> val(O.val);
    if (ci.empty()) {
        ci.push_back(0);
        val.push_back(0.0);
    }
    int steps = 0;
    check(bh_folm_diag_csr(O.dim, O.rp.data(), ci.data(), val.data(), nb_iter, v0.data(), T.data(), V.data(),
                           &steps));
    return steps;
}

}  // namespace bhgb
