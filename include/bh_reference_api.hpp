// bh_reference_api.hpp -- C++ drop-in for the exact path of
// Maximilien-Hantonne/Bose-Hubbard-Phase-Transition, over the C ABI of
// libbhgb300.so (bh_gb300.h).
//
// It defines, with the reference's own signatures (include/hamiltonian.hpp,
// include/neighbours.hpp, include/operator.hpp), the functions that
// src/hamiltonian.cpp, src/neighbours.cpp and src/operator.cpp implement, so a
// build of the reference can drop those three files and compile instead one
// translation unit:
//
//     #include "hamiltonian.hpp"
//     #include "neighbours.hpp"
//     #include "operator.hpp"
//     #define BH_GB300_IMPLEMENTATION
//     #include "bh_reference_api.hpp"
//
// and link -lbhgb300.  Errors are rethrown as the reference throws them:
// std::runtime_error("Eigenvalue computation failed.") for a solve that does
// not converge (operator.cpp:28), std::invalid_argument for invalid arguments
// (neighbours.cpp:43, Spectra's argument checks), std::runtime_error for CUDA
// errors.  The physics is the model's (U/2 n(n-1), one entry per directed
// bond); see the header of bh_gb300.h.  Requires Eigen (the reference vendors
// 3.4.0).
#pragma once

#include <Eigen/Dense>
#include <Eigen/SparseCore>
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <iostream>
#include <limits>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "bh_cxx.hpp"
#include "bh_gb300.h"

namespace bhgb {

// CSR (symmetric matrix) -> Eigen::SparseMatrix<double> (ColMajor): for a
// symmetric matrix the row-compressed arrays are the column-compressed ones.
inline Eigen::SparseMatrix<double> from_csr(int64_t D, const std::vector<int64_t>& rp,
                                            const std::vector<int32_t>& ci,
                                            const std::vector<double>& val, bool keep_diag,
                                            bool keep_off) {
    std::vector<Eigen::Triplet<double>> t;
    t.reserve((size_t)rp[D]);
    for (int64_t r = 0; r < D; ++r)
        for (int64_t e = rp[r]; e < rp[r + 1]; ++e) {
            const bool diag = ci[e] == r;
            if ((diag && keep_diag) || (!diag && keep_off)) t.emplace_back((int)ci[e], (int)r, val[e]);
        }
    Eigen::SparseMatrix<double> H(D, D);
    H.setFromTriplets(t.begin(), t.end());
    return H;
}

inline Eigen::SparseMatrix<double> term(const std::vector<std::vector<int>>& nb, int m, int n,
                                        double J, double U, double mu, bool keep_diag,
                                        bool keep_off) {
    Basis b(m, n);
    Hamiltonian h(b, nb);
    const Csr c = hamiltonian_csr(b, h, J, U, mu);
    return from_csr(c.dim, c.rp, c.ci, c.val, keep_diag, keep_off);
}

// the reference's sort_basis (hamiltonian.cpp:109-123): argsort by tag, then
// the cycle loop, which applies the inverse of the argsort permutation
inline void sort_like_reference(Eigen::VectorXd& tags, Eigen::MatrixXd& basis) {
    std::vector<int> idx(tags.size());
    for (int i = 0; i < (int)idx.size(); ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return tags[a] < tags[b]; });
    for (int i = 0; i < (int)idx.size(); ++i)
        while (idx[i] != i) {
            const int j = idx[i];
            std::swap(tags[i], tags[j]);
            basis.col(i).swap(basis.col(j));
            std::swap(idx[i], idx[j]);
        }
}

inline Csr csr_of(Eigen::SparseMatrix<double>& O) {
    O.makeCompressed();
    Csr c;
    c.dim = O.rows();
    c.rp.resize(c.dim + 1);
    for (int64_t k = 0; k <= c.dim; ++k) c.rp[k] = O.outerIndexPtr()[k];
    c.ci.assign(O.innerIndexPtr(), O.innerIndexPtr() + O.nonZeros());
    c.val.assign(O.valuePtr(), O.valuePtr() + O.nonZeros());
    return c;
}

}  // namespace bhgb

#ifdef BH_GB300_IMPLEMENTATION

// ---- Neighbours (neighbours.hpp:20-58) ----
Neighbours::Neighbours(int m) : m(m), neighbours(m) {}
Neighbours::~Neighbours() {}

void Neighbours::chain_neighbours(bool closed) { neighbours = bhgb::lattice(m, closed, bh_neighbours_chain); }
void Neighbours::square_neighbours(bool closed) { neighbours = bhgb::lattice(m, closed, bh_neighbours_square); }
void Neighbours::cube_neighbours(bool closed) { neighbours = bhgb::lattice(m, closed, bh_neighbours_cube); }
std::vector<std::vector<int>> Neighbours::getNeighbours() const { return neighbours; }

// ---- BH (hamiltonian.hpp:33-112) ----
double BH::calculate_tag(const Eigen::MatrixXd& basis, const std::vector<int>& primes, int k) {
    double tag = 0;
    for (int i = 0; i < basis.rows(); i++) tag += basis.coeff(i, k) * std::log((double)primes[i]);
    return tag;
}

Eigen::VectorXd BH::calculate_tags(const Eigen::MatrixXd& basis, const std::vector<int>& primes) {
    Eigen::VectorXd tags(basis.cols());
    for (int i = 0; i < basis.cols(); i++) tags[i] = calculate_tag(basis, primes, i);
    return tags;
}

// Index of the tag closest to x (the reference's binary search assumes sorted
// tags, which fixed_set_basis does not produce; the closest-tag scan is exact
// for any order because distinct states have tags at least 1e-14 apart).
int BH::search_tag(const Eigen::VectorXd& tags, double x) {
    int best = 0;
    double bd = std::numeric_limits<double>::infinity();
    for (int i = 0; i < tags.size(); ++i) {
        const double d = std::fabs(tags[i] - x);
        if (d < bd) {
            bd = d;
            best = i;
        }
    }
    return best;
}

std::pair<Eigen::VectorXd, Eigen::MatrixXd> BH::fixed_set_basis(int m, int n) {
    bhgb::Basis b(m, n);
    const int64_t D = b.dim();
    Eigen::VectorXd tags(D);
    Eigen::MatrixXd basis(m, D);
    bhgb::check(bh_basis_copy(b.p, tags.data(), basis.data(), nullptr, nullptr));
    return std::make_pair(tags, basis);
}

std::pair<Eigen::VectorXd, Eigen::MatrixXd> BH::max_set_basis(int m, int n) {
    Eigen::VectorXd tags;
    Eigen::MatrixXd basis(m, 0);
    for (int bosons = 1; bosons <= n; ++bosons) {
        auto [t, b] = fixed_set_basis(m, bosons);
        const Eigen::Index o = tags.size();
        tags.conservativeResize(o + t.size());
        tags.segment(o, t.size()) = t;
        basis.conservativeResize(Eigen::NoChange, o + b.cols());
        basis.block(0, o, m, b.cols()) = b;
    }
    bhgb::sort_like_reference(tags, basis);
    return std::make_pair(tags, basis);
}

// One term, selected as the reference selects it (hamiltonian.cpp:238-256).
Eigen::SparseMatrix<double> BH::fixed_bosons_hamiltonian(const std::vector<std::vector<int>>& neighbours,
                                                         const Eigen::MatrixXd& basis,
                                                         const Eigen::VectorXd& tags, int m, int n,
                                                         double J, double U, double mu) {
    (void)basis;
    (void)tags;
    const double eps = std::numeric_limits<double>::epsilon();
    if (std::abs(J - 0.0) > eps) return bhgb::term(neighbours, m, n, J, 0.0, 0.0, false, true);
    if (std::abs(U - 0.0) > eps) return bhgb::term(neighbours, m, n, 0.0, U, 0.0, true, false);
    if (std::abs(mu - 0.0) > eps) return bhgb::term(neighbours, m, n, 0.0, 0.0, mu, true, false);
    std::cerr << "Error: At least one of the parameters J, U, mu must be different from zero." << std::endl;
    int64_t D = 0;
    bhgb::check(bh_dimension(m, n, &D));
    return Eigen::SparseMatrix<double>(D, D);
}

// Block-diagonal concatenation of the sectors n_min..n_max (hamiltonian.cpp:260-288).
Eigen::SparseMatrix<double> BH::max_bosons_hamiltonian(const std::vector<std::vector<int>>& neighbours,
                                                       int m, int n_min, int n_max, double J,
                                                       double U, double mu) {
    if (n_min < 0) n_min = 0;
    if (n_max < n_min) n_max = n_min;
    std::vector<Eigen::Triplet<double>> t;
    int64_t offset = 0;
    for (int bosons = n_min; bosons <= n_max; ++bosons) {
        auto [tags, basis] = fixed_set_basis(m, bosons);
        Eigen::SparseMatrix<double> h = fixed_bosons_hamiltonian(neighbours, basis, tags, m, bosons, J, U, mu);
        for (int k = 0; k < h.outerSize(); ++k)
            for (Eigen::SparseMatrix<double>::InnerIterator it(h, k); it; ++it)
                t.emplace_back((int)(it.row() + offset), (int)(it.col() + offset), it.value());
        offset += h.rows();
    }
    Eigen::SparseMatrix<double> H(offset, offset);
    H.setFromTriplets(t.begin(), t.end());
    return H;
}

// Mean-field single-site Hamiltonian (hamiltonian.cpp:290-309), same entries.
void BH::h_MF(double psi, int p, double mu, double J, int q, Eigen::MatrixXd& h) {
    for (int i = 0; i < 2 * p + 1; i++) h(i, i) = -mu * i + 0.5 * i * (i - 1) + q * J * psi * psi;
    for (int j = 0; j < 2 * p + 1; j++) {
        if (j == 0) {
            h(1, 0) = -q * J * psi * std::sqrt(1.0);
        } else if (j == 2 * p) {
            h(2 * p - 1, 2 * p) = -q * J * psi * std::sqrt(2.0 * p);
        } else {
            h(j + 1, j) = -q * J * psi * std::sqrt(j + 1.0);
            h(j - 1, j) = -q * J * psi * std::sqrt((double)j);
        }
    }
}

// ---- Op (operator.hpp:17-55) ----
// Lowest nb_eigen eigenpairs of the symmetric O, ordered like Spectra's
// LargestMagn output (GenEigsBase.h:417, 466-483), as complex vectors
// (bhgb::irlm_eigen, bh_cxx.hpp).
Eigen::VectorXcd Op::IRLM_eigen(Eigen::SparseMatrix<double> O, int nb_eigen, Eigen::MatrixXcd& eigenvectors) {
    std::vector<double> ev, vec;
    bhgb::irlm_eigen(bhgb::csr_of(O), nb_eigen, ev, vec);
    Eigen::VectorXcd vals(nb_eigen);
    eigenvectors.resize(O.rows(), nb_eigen);
    for (int k = 0; k < nb_eigen; ++k) {
        vals[k] = std::complex<double>(ev[k], 0.0);
        for (Eigen::Index r = 0; r < O.rows(); ++r)
            eigenvectors(r, k) = std::complex<double>(vec[(size_t)k * O.rows() + r], 0.0);
    }
    return vals;
}

// The intended full-orthogonalisation Lanczos: the lowest
// min(nb_iter, n - 2, 32) eigenpairs, ascending, FP64.
void Op::FOLM_diag(Eigen::SparseMatrix<double> O, int nb_iter, Eigen::VectorXd& v_0, Eigen::MatrixXd& T,
                   Eigen::MatrixXd& V) {
    std::vector<double> v0(v_0.data(), v_0.data() + v_0.size()), t, vv;
    bhgb::folm_diag(bhgb::csr_of(O), nb_iter, v0, t, vv);
    for (Eigen::Index r = 0; r < v_0.size(); ++r) v_0[r] = v0[(size_t)r];  // normalised, as the reference's
    T = Eigen::Map<Eigen::MatrixXd>(t.data(), nb_iter, nb_iter);
    V = Eigen::Map<Eigen::MatrixXd>(vv.data(), O.rows(), nb_iter);
}

Eigen::VectorXd Op::FOLM_eigen(Eigen::SparseMatrix<double> O, int nb_iter, Eigen::MatrixXd& eigenvectors) {
    const int nev = std::max(1, std::min<int>({nb_iter, (int)O.rows() - 2, 32}));
    std::vector<double> ev, vec;
    bhgb::eigsh(bhgb::csr_of(O), nev, ev, vec);
    Eigen::VectorXd vals(nev);
    eigenvectors.resize(O.rows(), nev);
    for (int k = 0; k < nev; ++k) {
        vals[k] = ev[k];
        for (Eigen::Index r = 0; r < O.rows(); ++r) eigenvectors(r, k) = vec[(size_t)k * O.rows() + r];
    }
    return vals;
}

Eigen::VectorXd Op::exact_eigen(Eigen::SparseMatrix<double> O, Eigen::MatrixXd& eigenvectors) {
    Eigen::MatrixXd dense = Eigen::MatrixXd(O);
    const int64_t n = dense.rows();
    Eigen::VectorXd vals(n);
    eigenvectors.resize(n, n);
    bhgb::check(bh_dense_eigh(n, dense.data(), vals.data(), eigenvectors.data()));
    return vals;
}

#endif  // BH_GB300_IMPLEMENTATION
