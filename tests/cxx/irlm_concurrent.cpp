// irlm_concurrent.cpp -- GPU test driver of the C++ layer (bh_cxx.hpp), the
// code under the Eigen-typed drop-in's Op::IRLM_eigen.  It does what the
// reference's grid loop does (src/analysis.cpp:302-314): several OpenMP
// threads call IRLM_eigen at once on Hamiltonians of the m = n = 8 chain.
//
//   irlm_concurrent <nthreads>
//
// Output lines:
//   point <k> <J> <mu> <value_0> ... <value_9>     (concurrent run, reference order)
//   same <k> <0|1>      1 if the concurrent values equal a sequential re-run bit for bit
//   noconv <k> <what>   the exception text of a solve capped at 1 restart of a 22-vector basis
//   badarg <what>       the exception text of nev = n - 1
//   folm <steps> <max|V^T V - I|> <alpha_0..alpha_k-1> <beta_0..beta_k-2>
//                       Op::FOLM_diag through the C++ layer: 30 Lanczos steps of
//                       point 0 from v0[r] = sin(0.37 (r + 1))
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "bh_cxx.hpp"

int main(int argc, char** argv) {
    const int nthreads = argc > 1 ? std::atoi(argv[1]) : 8;
    const int m = 8, n = 8, nev = 10;
    const auto nb = bhgb::lattice(m, true, bh_neighbours_chain);
    bhgb::Basis b(m, n);
    bhgb::Hamiltonian h(b, nb);
    // point 0 is the golden case J = 0.1, U = 1, mu = 0.5
    std::vector<double> Js, mus;
    for (int k = 0; k < 2 * nthreads; ++k) {
        Js.push_back(k == 0 ? 0.1 : 0.02 + 0.015 * k);
        mus.push_back(k == 0 ? 0.5 : 0.1 * (k % 5));
    }
    const int np = (int)Js.size();
    std::vector<bhgb::Csr> ops;
    for (int k = 0; k < np; ++k) ops.push_back(bhgb::hamiltonian_csr(b, h, Js[k], 1.0, mus[k]));

    std::vector<std::vector<double>> conc(np), seq(np);
    std::vector<std::string> err(np);
#pragma omp parallel for schedule(dynamic) num_threads(nthreads)
    for (int k = 0; k < np; ++k) {
        try {
            std::vector<double> vec;
            bhgb::irlm_eigen(ops[k], nev, conc[k], vec);
        } catch (const std::exception& e) {
            err[k] = e.what();
        }
    }
    for (int k = 0; k < np; ++k) {
        if (!err[k].empty()) {
            std::printf("error %d %s\n", k, err[k].c_str());
            return 2;
        }
        std::vector<double> vec;
        bhgb::irlm_eigen(ops[k], nev, seq[k], vec);
        std::printf("point %d %.17g %.17g", k, Js[k], mus[k]);
        for (double v : conc[k]) std::printf(" %.17g", v);
        std::printf("\n");
        bool same = conc[k].size() == seq[k].size();
        for (size_t i = 0; same && i < conc[k].size(); ++i) same = conc[k][i] == seq[k][i];
        std::printf("same %d %d\n", k, same ? 1 : 0);
    }
    // non-convergence, from every thread at once
    std::vector<std::string> nc(nthreads);
#pragma omp parallel for num_threads(nthreads)
    for (int k = 0; k < nthreads; ++k) {
        try {
            std::vector<double> vals, vec;
            bhgb::irlm_eigen(ops[k], nev, vals, vec, /*max_restarts=*/1, /*ncv=*/22);
            nc[k] = "no exception";
        } catch (const std::runtime_error& e) {
            nc[k] = e.what();
        } catch (const std::exception& e) {
            nc[k] = std::string("other: ") + e.what();
        }
    }
    for (int k = 0; k < nthreads; ++k) std::printf("noconv %d %s\n", k, nc[k].c_str());
    try {
        std::vector<double> vals, vec;
        bhgb::irlm_eigen(ops[0], (int)ops[0].dim - 1, vals, vec);
        std::printf("badarg no exception\n");
    } catch (const std::invalid_argument& e) {
        std::printf("badarg %s\n", e.what());
    }
    {
        const bhgb::Csr& O = ops[0];
        const int k = 30;
        std::vector<double> v0((size_t)O.dim), T, V;
        for (int64_t r = 0; r < O.dim; ++r) v0[(size_t)r] = std::sin(0.37 * (double)(r + 1));
        const int steps = bhgb::folm_diag(O, k, v0, T, V);
        double orth = 0.0;
        for (int a = 0; a < steps; ++a)
            for (int c = 0; c < steps; ++c) {
                double d = 0.0;
                for (int64_t r = 0; r < O.dim; ++r) d += V[(size_t)a * O.dim + r] * V[(size_t)c * O.dim + r];
                orth = std::max(orth, std::fabs(d - (a == c ? 1.0 : 0.0)));
            }
        std::printf("folm %d %.3e", steps, orth);
        for (int i = 0; i < k; ++i) std::printf(" %.17g", T[(size_t)i * k + i]);
        for (int i = 0; i + 1 < k; ++i) std::printf(" %.17g", T[(size_t)i * k + i + 1]);
        std::printf("\n");
    }
    return 0;
}
