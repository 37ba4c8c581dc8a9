// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference's own exact-path sources (Maximilien-Hantonne/
// Bose-Hubbard-Phase-Transition: src/hamiltonian.cpp, src/neighbours.cpp,
// src/operator.cpp, src/analysis.cpp, src/resource.cpp, against its vendored
// Eigen 3.4.0 and Spectra 1.1.0) into oracle/_ref/libbhref.so and exposes a
// few C entry points so that tests/golden/make_golden.py can record golden
// vectors from the reference itself.  The sources are #included from the
// reference tree (never copied) because the helpers used here have internal
// linkage in the reference's headers (hamiltonian.hpp:14-53,
// analysis.hpp:13-87).  Built by oracle/Makefile, only where the reference
// tree is present.
#include "hamiltonian.cpp"
#include "neighbours.cpp"
#include "operator.cpp"
#include "resource.cpp"
#include "analysis.cpp"

#include <cstdint>
#include <cstring>
#include <exception>

extern "C" {

// BH::dimension (hamiltonian.cpp:52-54)
int ref_dimension(int m, int n) { return BH::dimension(m, n); }

// BH::fixed_set_basis (hamiltonian.cpp:143-149): tags (D) and basis (m x D,
// column-major) exactly as the reference returns them.
int ref_fixed_set_basis(int m, int n, double* tags, double* basis) {
    auto [t, b] = BH::fixed_set_basis(m, n);
    std::memcpy(tags, t.data(), sizeof(double) * t.size());
    std::memcpy(basis, b.data(), sizeof(double) * b.size());
    return static_cast<int>(t.size());
}

// BH::init_lexicographic (hamiltonian.cpp:75-85)
int ref_init_lexicographic(int m, int n, double* basis) {
    Eigen::MatrixXd b = BH::init_lexicographic(m, n);
    std::memcpy(basis, b.data(), sizeof(double) * b.size());
    return static_cast<int>(b.cols());
}

// Neighbours::chain_neighbours / square_neighbours / cube_neighbours
// (neighbours.cpp:21-120); kind 1 = chain, 2 = square, 3 = cube.
// Writes offsets (m+1) and the flattened lists (capacity cap); returns the
// total count or -1 on an exception.
int ref_neighbours(int kind, int m, int closed, int* off, int* nbr, int cap) {
    try {
        Neighbours nb(m);
        if (kind == 1) nb.chain_neighbours(closed != 0);
        else if (kind == 2) nb.square_neighbours(closed != 0);
        else nb.cube_neighbours(closed != 0);
        auto lists = nb.getNeighbours();
        int c = 0;
        off[0] = 0;
        for (int i = 0; i < m; ++i) {
            for (int j : lists[i]) {
                if (c < cap) nbr[c] = j;
                ++c;
            }
            off[i + 1] = c;
        }
        return c;
    } catch (const std::exception&) {
        return -1;
    }
}

// Op::IRLM_eigen (operator.cpp:22-33) on a symmetric matrix given as
// compressed columns (for a symmetric matrix, CSR and CSC coincide).
// Returns nconv (the number of values written, in the reference's order),
// or -1 if the reference threw ("Eigenvalue computation failed.").
int ref_irlm(int64_t D, const int64_t* outer, const int32_t* inner, const double* val,
             int nev, double* evals_re, double* evals_im, double* evecs_re) {
    std::vector<Eigen::Triplet<double>> trip;
    trip.reserve(static_cast<size_t>(outer[D]));
    for (int64_t c = 0; c < D; ++c)
        for (int64_t e = outer[c]; e < outer[c + 1]; ++e)
            trip.emplace_back(static_cast<int>(inner[e]), static_cast<int>(c), val[e]);
    Eigen::SparseMatrix<double> H(D, D);
    H.setFromTriplets(trip.begin(), trip.end());
    Eigen::MatrixXcd vecs;
    try {
        Eigen::VectorXcd ev = Op::IRLM_eigen(H, nev, vecs);
        for (int i = 0; i < ev.size(); ++i) {
            evals_re[i] = ev[i].real();
            evals_im[i] = ev[i].imag();
        }
        if (evecs_re)
            for (int j = 0; j < vecs.cols(); ++j)
                for (int64_t r = 0; r < D; ++r) evecs_re[j * D + r] = vecs(r, j).real();
        return static_cast<int>(ev.size());
    } catch (const std::exception&) {
        return -1;
    }
}

// Op::exact_eigen (operator.cpp:92-101): all eigenvalues, ascending.
int ref_exact_eigen(int64_t D, const int64_t* outer, const int32_t* inner, const double* val,
                    double* evals) {
    std::vector<Eigen::Triplet<double>> trip;
    for (int64_t c = 0; c < D; ++c)
        for (int64_t e = outer[c]; e < outer[c + 1]; ++e)
            trip.emplace_back(static_cast<int>(inner[e]), static_cast<int>(c), val[e]);
    Eigen::SparseMatrix<double> H(D, D);
    H.setFromTriplets(trip.begin(), trip.end());
    Eigen::MatrixXd vecs;
    try {
        Eigen::VectorXd ev = Op::exact_eigen(H, vecs);
        for (int i = 0; i < ev.size(); ++i) evals[i] = ev[i];
        return static_cast<int>(ev.size());
    } catch (const std::exception&) {
        return -1;
    }
}

// Analysis::gap_ratios (analysis.cpp:433-454) on real eigenvalues.
int ref_gap_ratios(int nev, const double* evals, double* ratios) {
    Eigen::VectorXcd ev(nev);
    for (int i = 0; i < nev; ++i) ev[i] = std::complex<double>(evals[i], 0.0);
    Eigen::VectorXd r = Analysis::gap_ratios(ev, nev);
    for (int i = 0; i < r.size(); ++i) ratios[i] = r[i];
    return static_cast<int>(r.size());
}

// Analysis::coherence (analysis.cpp:542-556) on a real m x m matrix (row-major).
double ref_coherence(int m, const double* rho) {
    Eigen::MatrixXcd s(m, m);
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) s(i, j) = rho[i * m + j];
    return Analysis::coherence(s);
}

// Analysis::SCMF (analysis.cpp:111-178): the self-consistent mean-field order
// parameter at (mu, J) from the seed psi0, eps = 10^-precision.
double ref_scmf(double mu, double J, int q, double psi0, int precision) {
    try {
        return Analysis::SCMF(mu, J, q, psi0, precision);
    } catch (const std::exception&) {
        return std::nan("");
    }
}

}  // extern "C"
