// bh_symeig.cpp -- FP64 dense symmetric eigensolver for the small projected
// problems of the Krylov solver (the role Spectra's UpperHessenbergEigen and
// Eigen's SelfAdjointEigenSolver play for the reference, operator.cpp:79).
//
// Householder reduction to tridiagonal form, then the implicit symmetric QR
// iteration with Wilkinson shifts (Golub & Van Loan, Matrix Computations,
// algorithms 8.3.1 and 8.3.3), accumulating all transformations.
#include <algorithm>
#include <cmath>
#include <vector>

#include "bh_internal.h"

namespace bh {

bool symeig(int n, double* a, double* w) {
    if (n <= 0) return true;
    if (n == 1) {
        w[0] = a[0];
        a[0] = 1.0;
        return true;
    }
    auto A = [&](int i, int j) -> double& { return a[(size_t)j * n + i]; };
    std::vector<double> Q((size_t)n * n, 0.0);
    auto Qm = [&](int i, int j) -> double& { return Q[(size_t)j * n + i]; };
    for (int i = 0; i < n; ++i) Qm(i, i) = 1.0;
    std::vector<double> v(n), p(n), wv(n);

    // 1. tridiagonalisation: A <- H_k A H_k, Q <- Q H_k
    for (int k = 0; k + 2 < n; ++k) {
        const int m = n - k - 1;  // length of the reflected part (rows k+1..n-1)
        double alpha = 0.0;
        for (int i = 0; i < m; ++i) alpha = std::max(alpha, std::fabs(A(k + 1 + i, k)));
        if (alpha == 0.0) continue;
        double sig = 0.0;
        for (int i = 0; i < m; ++i) {
            v[i] = A(k + 1 + i, k) / alpha;
            sig += v[i] * v[i];
        }
        double nx = std::sqrt(sig);
        const double x0 = v[0];
        const double mu = x0 >= 0.0 ? x0 + nx : x0 - nx;  // v = x + sign(x0) |x| e1
        if (mu == 0.0) continue;
        v[0] = mu;
        double vv = 0.0;
        for (int i = 0; i < m; ++i) vv += v[i] * v[i];
        const double beta = 2.0 / vv;
        // p = beta * A_sub v
        for (int i = 0; i < m; ++i) {
            double s = 0.0;
            for (int j = 0; j < m; ++j) s += A(k + 1 + i, k + 1 + j) * v[j];
            p[i] = beta * s;
        }
        double pv = 0.0;
        for (int i = 0; i < m; ++i) pv += p[i] * v[i];
        const double c = 0.5 * beta * pv;
        for (int i = 0; i < m; ++i) wv[i] = p[i] - c * v[i];
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < m; ++i) A(k + 1 + i, k + 1 + j) -= v[i] * wv[j] + wv[i] * v[j];
        // column k below the subdiagonal becomes (-sign(x0) |x|, 0, ...)
        const double newsub = (x0 >= 0.0 ? -nx : nx) * alpha;
        A(k + 1, k) = newsub;
        A(k, k + 1) = newsub;
        for (int i = 1; i < m; ++i) {
            A(k + 1 + i, k) = 0.0;
            A(k, k + 1 + i) = 0.0;
        }
        // Q <- Q (I - beta v v^T) on columns k+1..n-1
        for (int r = 0; r < n; ++r) {
            double s = 0.0;
            for (int j = 0; j < m; ++j) s += Qm(r, k + 1 + j) * v[j];
            s *= beta;
            for (int j = 0; j < m; ++j) Qm(r, k + 1 + j) -= s * v[j];
        }
    }
    std::vector<double> d(n), e(n, 0.0);
    for (int i = 0; i < n; ++i) d[i] = A(i, i);
    for (int i = 0; i + 1 < n; ++i) e[i] = A(i + 1, i);

    // 2. implicit symmetric QR with Wilkinson shift on (d, e)
    const double eps = 2.220446049250313e-16;
    int hi = n - 1;
    int iter = 0;
    const int max_iter = 60 * n;
    while (hi > 0) {
        // deflate converged trailing off-diagonals
        if (std::fabs(e[hi - 1]) <= eps * (std::fabs(d[hi - 1]) + std::fabs(d[hi])) ||
            std::fabs(e[hi - 1]) < 1e-300) {
            e[hi - 1] = 0.0;
            --hi;
            continue;
        }
        int lo = hi - 1;
        while (lo > 0 && std::fabs(e[lo - 1]) > eps * (std::fabs(d[lo - 1]) + std::fabs(d[lo])) &&
               std::fabs(e[lo - 1]) >= 1e-300)
            --lo;
        if (lo > 0) e[lo - 1] = 0.0;
        if (++iter > max_iter) return false;
        // Wilkinson shift from the trailing 2x2 block
        const double dd = 0.5 * (d[hi - 1] - d[hi]);
        const double eh = e[hi - 1];
        const double den = dd + (dd >= 0.0 ? 1.0 : -1.0) * std::hypot(dd, eh);
        const double shift = den != 0.0 ? d[hi] - eh * eh / den : d[hi] - std::fabs(eh);
        double x = d[lo] - shift, z = e[lo];
        for (int k = lo; k < hi; ++k) {
            // Givens rotation zeroing z against x
            double c, s;
            if (z == 0.0) {
                c = 1.0;
                s = 0.0;
            } else {
                const double r = std::hypot(x, z);
                c = x / r;
                s = -z / r;
            }
            if (k > lo) e[k - 1] = c * e[k - 1] - s * z;
            const double dk = d[k], dk1 = d[k + 1], ek = e[k];
            // [d_k e_k; e_k d_k1] <- G^T [..] G with G = [c s; -s c]
            d[k] = c * c * dk - 2.0 * c * s * ek + s * s * dk1;
            d[k + 1] = s * s * dk + 2.0 * c * s * ek + c * c * dk1;
            e[k] = c * s * (dk - dk1) + (c * c - s * s) * ek;
            if (k + 1 < hi) {
                x = e[k];
                z = -s * e[k + 1];
                e[k + 1] = c * e[k + 1];
            }
            for (int r = 0; r < n; ++r) {
                const double q0 = Qm(r, k), q1 = Qm(r, k + 1);
                Qm(r, k) = c * q0 - s * q1;
                Qm(r, k + 1) = s * q0 + c * q1;
            }
        }
    }
    // 3. sort ascending
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](int x1, int x2) { return d[x1] < d[x2]; });
    for (int i = 0; i < n; ++i) {
        w[i] = d[ord[i]];
        for (int r = 0; r < n; ++r) a[(size_t)i * n + r] = Qm(r, ord[i]);
    }
    return true;
}

}  // namespace bh
