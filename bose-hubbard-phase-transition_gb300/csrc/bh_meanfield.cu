// bh_meanfield.cu -- the self-consistent mean-field (SCMF) sweep on the device.
//
// Replaces Analysis::mean_field_parameters / SCMF / SF_density
// (src/analysis.cpp:58-178) and BH::h_MF (src/hamiltonian.cpp:290-309).  The
// reference solves, for every (mu, J) grid point, a double fixed-point
// iteration: grow the truncation p from 1 until the ground energy of the
// (2p+1) x (2p+1) single-site matrix
//     h = diag(-mu i + i (i-1) / 2 + q J psi^2),  h(i, i+1) = -q J psi sqrt(i+1)
// moves by at most eps = 10^-precision, then replace psi by
// sum_{i=1}^{2p} sqrt(i) phi_i phi_{i-1} of its ground vector phi, until psi
// moves by at most eps.  Each eigensolve there is a Spectra Lanczos run on a
// dense block carved out of a 1000 x 1000 matrix.
//
// Here one thread owns one grid point.  h is symmetric tridiagonal and
// generated on the fly from (mu, J, q, psi, p).  From 7 levels on its ground
// state comes from Rayleigh-quotient iteration started at the previous
// truncation's ground vector, certified by Sturm counts; the first
// truncations (and any uncertified case) use Sturm-count bisection, bracketed
// by the Gershgorin lower bound and min_i h_ii (and, for p > 1, by the
// previous truncation's energy: the smallest eigenvalue cannot rise when a
// level is added), the ground vector from two inverse-iteration sweeps, and
// the energy from its Rayleigh quotient.  For psi = 0 or J = 0 h is diagonal; its ground vector is taken
// as the unit vector of the first smallest diagonal entry, so psi = 0 is a
// fixed point (the reference's Lanczos returns an arbitrary mixture when two
// diagonal entries tie, at integer mu).
#include <algorithm>
#include <cmath>

#include "bh_internal.h"

namespace bh {

constexpr int kScmfPmax = 48;                 // truncation limit: 2 p + 1 <= 97 levels
constexpr int kScmfN = 2 * kScmfPmax + 1;

__device__ __forceinline__ double mf_diag(int i, double mu, double c2) {
    return -mu * i + 0.5 * i * (i - 1) + c2;
}

// Number of eigenvalues of h below x: sign changes of the Sturm sequence
// P_0 = 1, P_1 = d_0 - x, P_{i+1} = (d_i - x) P_i - e_{i-1}^2 P_{i-1}
// (P_i = det of the leading i x i block of h - x I), without divisions; the
// pair (P_i, P_{i-1}) is rescaled by powers of two to stay in range.  A zero
// P_i takes the sign opposite to P_{i-1}.
__device__ __forceinline__ int mf_sturm(int N, double mu, double c1sq, double c2, double x) {
    double pm = 1.0, pc = mf_diag(0, mu, c2) - x;
    int cnt = (pc < 0.0) || (pc == 0.0);
    bool prev_neg = pc < 0.0 || pc == 0.0;
    for (int i = 1; i < N; ++i) {
        const double pn = (mf_diag(i, mu, c2) - x) * pc - (c1sq * i) * pm;
        pm = pc;
        pc = pn;
        const bool neg = pc == 0.0 ? !prev_neg : pc < 0.0;
        cnt += neg != prev_neg;
        prev_neg = neg;
        const double a = fabs(pc);
        if (a > 0x1p+500) {
            pc *= 0x1p-500;
            pm *= 0x1p-500;
        } else if (a < 0x1p-500 && a > 0.0) {
            pc *= 0x1p+500;
            pm *= 0x1p+500;
        }
    }
    return cnt;
}

// Ground state of h(psi, p): energy, and the normalised vector in x.
// hi_in: an upper bound of the smallest eigenvalue (+inf if none).  The
// bracket [Gershgorin lower bound, min(min_i h_ii, hi_in)] is bisected to a
// relative width of 2^-34; two inverse-iteration sweeps at its lower end
// (where h - sigma I is positive definite, so the LDL^T pivots stay positive)
// give the vector, and its Rayleigh quotient the energy (error ~ width^2).
__device__ double mf_ground(int N, double mu, double c1, double c2, double hi_in, double* x,
                            double* piv, const double* __restrict__ sq) {
    // c1 = -q J psi (off-diagonal factor), c2 = q J psi^2 (diagonal shift)
    if (c1 == 0.0) {
        int imin = 0;
        double dmin = mf_diag(0, mu, c2);
        for (int i = 1; i < N; ++i) {
            const double di = mf_diag(i, mu, c2);
            if (di < dmin) {
                dmin = di;
                imin = i;
            }
        }
        for (int i = 0; i < N; ++i) x[i] = i == imin ? 1.0 : 0.0;
        return dmin;
    }
    const double c1sq = c1 * c1;
    double lo = INFINITY, hi = hi_in;
    for (int i = 0; i < N; ++i) {
        const double di = mf_diag(i, mu, c2);
        const double r = fabs(c1) * ((i > 0 ? sq[i] : 0.0) + (i + 1 < N ? sq[i + 1] : 0.0));
        lo = fmin(lo, di - r);
        hi = fmin(hi, di);
    }
    const double scale = fmax(fabs(lo), fabs(hi)) + fabs(c1);
    for (int it = 0; it < 200; ++it) {
        if (hi - lo <= 0x1p-34 * scale) break;
        const double mid = 0.5 * (lo + hi);
        if (!(mid > lo && mid < hi)) break;
        if (mf_sturm(N, mu, c1sq, c2, mid) >= 1) hi = mid;
        else lo = mid;
    }
    // inverse iteration at sigma = lo: (h - sigma I) y = x, LDL^T without
    // pivoting; pivots are kept >= a rounding-level floor relative to the
    // matrix scale, so a nearly singular last pivot cannot overflow y
    const double sigma = lo;
    const double tiny = 1e-15 * (fabs(sigma) + fabs(c1) * sq[N] + 1.0);
    // factor once (piv holds the inverse pivots), then two solves
    {
        double p0 = mf_diag(0, mu, c2) - sigma;
        if (p0 < tiny) p0 = tiny;
        piv[0] = 1.0 / p0;
        for (int i = 1; i < N; ++i) {
            const double e = c1 * sq[i];  // h(i-1, i)
            double pi = mf_diag(i, mu, c2) - sigma - e * e * piv[i - 1];
            if (pi < tiny) pi = tiny;
            piv[i] = 1.0 / pi;
        }
    }
    for (int i = 0; i < N; ++i) x[i] = 1.0;
    for (int sweep = 0; sweep < 2; ++sweep) {
        for (int i = 1; i < N; ++i) x[i] -= c1 * sq[i] * piv[i - 1] * x[i - 1];
        x[N - 1] *= piv[N - 1];
        for (int i = N - 2; i >= 0; --i) x[i] = (x[i] - c1 * sq[i + 1] * x[i + 1]) * piv[i];
        double nrm = 0.0;
        for (int i = 0; i < N; ++i) nrm += x[i] * x[i];
        const double s = rsqrt(nrm);
        for (int i = 0; i < N; ++i) x[i] *= s;
    }
    // Rayleigh quotient x^T h x
    double rq = 0.0;
    for (int i = 0; i < N; ++i) {
        rq += mf_diag(i, mu, c2) * x[i] * x[i];
        if (i + 1 < N) rq += 2.0 * c1 * sq[i + 1] * x[i] * x[i + 1];
    }
    return rq;
}

// Ground state by Rayleigh-quotient iteration from x (the previous
// truncation's ground vector padded with zeros, an excellent start: adding
// two levels barely moves it): at most four steps of x <- (h - rho I)^-1 x,
// rho = x^T h x, then a certificate by two Sturm counts -- exactly one
// eigenvalue below rho + delta and none below rho - delta.  Returns false
// (x destroyed) when the certificate fails; the caller then bisects.
__device__ bool mf_ground_rqi(int N, double mu, double c1, double c2, double* x, double* piv,
                              const double* __restrict__ sq, double& e0) {
    auto rayleigh = [&]() {
        double r = 0.0;
        for (int i = 0; i < N; ++i) {
            r += mf_diag(i, mu, c2) * x[i] * x[i];
            if (i + 1 < N) r += 2.0 * c1 * sq[i + 1] * x[i] * x[i + 1];
        }
        return r;
    };
    auto normalise = [&]() {
        double nrm = 0.0;
        for (int i = 0; i < N; ++i) nrm += x[i] * x[i];
        if (!(nrm > 0.0) || !isfinite(nrm)) return false;
        const double s = rsqrt(nrm);
        for (int i = 0; i < N; ++i) x[i] *= s;
        return true;
    };
    if (!normalise()) return false;
    double rho = rayleigh();
    const double tiny = 1e-15 * (fabs(rho) + fabs(c1) * sq[N] + 1.0);
    for (int it = 0; it < 4; ++it) {
        // (h - rho I) y = x in place, LDL^T without pivoting, |pivots| >= tiny
        double p0 = mf_diag(0, mu, c2) - rho;
        if (fabs(p0) < tiny) p0 = p0 < 0.0 ? -tiny : tiny;
        piv[0] = 1.0 / p0;
        for (int i = 1; i < N; ++i) {
            const double e = c1 * sq[i];
            double pi = mf_diag(i, mu, c2) - rho - e * e * piv[i - 1];
            if (fabs(pi) < tiny) pi = pi < 0.0 ? -tiny : tiny;
            piv[i] = 1.0 / pi;
            x[i] -= e * piv[i - 1] * x[i - 1];
        }
        x[N - 1] *= piv[N - 1];
        for (int i = N - 2; i >= 0; --i) x[i] = (x[i] - c1 * sq[i + 1] * x[i + 1]) * piv[i];
        if (!normalise()) return false;
        const double rn = rayleigh();
        const bool done = fabs(rn - rho) <= 1e-15 * (fabs(rn) + 1.0);
        rho = rn;
        if (done) break;
    }
    const double delta = 1e-9 * (fabs(rho) + fabs(c1) + 1.0);
    const double c1sq = c1 * c1;
    if (mf_sturm(N, mu, c1sq, c2, rho + delta) != 1 || mf_sturm(N, mu, c1sq, c2, rho - delta) != 0) return false;
    e0 = rho;
    return true;
}

// Persistent threads: each thread takes the next grid point from *next
// (points differ by orders of magnitude in their number of psi updates, so
// static assignment would leave most lanes idle behind the slowest point).
// psi_out[k], outer iterations in iters[k] (-1 if the truncation needed more
// than kScmfPmax, -2 if psi still moved after max_outer updates).
__global__ void __launch_bounds__(128)
k_scmf(int npts, const double* __restrict__ mu, const double* __restrict__ J, int q,
       const double* __restrict__ psi0, double eps, int max_outer, double* __restrict__ psi_out,
       int* __restrict__ iters, int* __restrict__ next) {
    __shared__ double sq[kScmfN + 1];  // sqrt(i)
    for (int i = threadIdx.x; i <= kScmfN; i += blockDim.x) sq[i] = sqrt((double)i);
    __syncthreads();
    double x[kScmfN], piv[kScmfN];
    for (;;) {
        const int k = atomicAdd(next, 1);
        if (k >= npts) break;
        const double m = mu[k], j = J[k];
        double psi = psi0[k], tmp = 0.0;
        int outer = 0;
        bool ok = true;
        do {
            const double c1 = -q * j * psi, c2 = q * j * psi * psi;
            int p = 1;
            double e0 = mf_ground(2 * p + 1, m, c1, c2, INFINITY, x, piv, sq);
            do {
                ++p;
                if (p > kScmfPmax) {
                    ok = false;
                    break;
                }
                // from 7 levels on: Rayleigh-quotient iteration from the previous
                // ground vector; else (or if it cannot certify) bisection, whose
                // bracket uses interlacing: the smallest eigenvalue cannot rise with p
                const int N = 2 * p + 1;
                double e1;
                bool ok1 = false;
                if (N >= 7 && c1 != 0.0) {
                    x[N - 2] = 0.0;
                    x[N - 1] = 0.0;
                    ok1 = mf_ground_rqi(N, m, c1, c2, x, piv, sq, e1);
                }
                if (!ok1) e1 = mf_ground(N, m, c1, c2, e0 + 1e-12 * (fabs(e0) + 1.0), x, piv, sq);
                tmp = fabs(e0 - e1);
                e0 = e1;
            } while (tmp > eps);
            if (!ok) break;
            double a = 0.0;
            for (int i = 1; i < 2 * p + 1; ++i) a += sq[i] * x[i] * x[i - 1];
            ++outer;
            tmp = fabs(a - psi);
            psi = a;
        } while (tmp > eps && outer < max_outer);
        psi_out[k] = ok ? psi : NAN;
        if (iters) iters[k] = !ok ? -1 : (tmp > eps ? -2 : outer);
    }
}

void scmf_device(int npts, const double* d_mu, const double* d_J, int q, const double* d_psi0,
                 int precision, int max_outer, double* d_psi, int* d_iters, cudaStream_t st) {
    const double eps = std::pow(10.0, -precision);
    DevBuf<int> next(1);
    BH_CUDA(cudaMemsetAsync(next.p, 0, sizeof(int), st));
    int64_t g = (npts + 127) / 128;
    g = std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)sm_count() * 16));
    k_scmf<<<(unsigned)g, 128, 0, st>>>(npts, d_mu, d_J, q, d_psi0, eps, max_outer, d_psi, d_iters,
                                        next.p);
    BH_CUDA(cudaGetLastError());
    BH_CUDA(cudaStreamSynchronize(st));
}

}  // namespace bh
