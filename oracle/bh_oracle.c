/*
 * bh_oracle.c -- CPU ORACLE for the Bose-Hubbard exact-diagonalisation path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library and its
 * host mirror) links, loads or calls this file.  tests/ and
 * __graft_entry__.smoke() compare the device results with it, and bench.py's
 * CPU baseline leg / reference arm times it as the CPU restatement ("port")
 * of the reference's exact path.
 *
 * It restates, in plain C, the reference's algorithms for this path
 * (Maximilien-Hantonne/Bose-Hubbard-Phase-Transition):
 *   - BH::binomial / BH::dimension            src/hamiltonian.cpp:39-54
 *   - BH::next_lexicographic / init_lexicographic  src/hamiltonian.cpp:60-85
 *   - BH::calculate_tag(s)                    src/hamiltonian.cpp:91-106
 *   - BH::sort_basis (inverse-permutation cycle sort) src/hamiltonian.cpp:109-123
 *   - BH::fixed_set_basis                     src/hamiltonian.cpp:143-149
 *   - BH::fill_hopping / fill_interaction / fill_chemical and
 *     BH::fixed_bosons_hamiltonian            src/hamiltonian.cpp:170-256
 *     with the physics of H = -J sum_<ij> b+_i b_j + U/2 sum n(n-1) - mu sum n
 *     (the reference's own builder loops over neighbour *slots*, reads out of
 *     bounds and doubles each hop; this restatement keeps its structure --
 *     three terms T, V, N combined as src/analysis.cpp:311 -- but with the
 *     correct neighbour loop, an exact integer rank instead of the float
 *     tag search, one entry per directed bond and U/2 n(n-1)).
 *   - Op::IRLM_eigen                          src/operator.cpp:22-33, i.e.
 *     Spectra 1.1.0 GenEigsSolver<SparseGenMatProd> with nev, ncv = 2 nev + 1,
 *     SimpleRandom(0) start vector (Util/SimpleRandom.h:30-123), Arnoldi
 *     factorisation with DGKS re-orthogonalisation (LinAlg/Arnoldi.h:132-280),
 *     shifted-QR implicit restarts (GenEigsBase.h:86-138), convergence test
 *     and nev adjustment (GenEigsBase.h:141-193), SmallestReal selection and
 *     LargestMagn final ordering (GenEigsBase.h:417-441).  For a symmetric
 *     matrix all Ritz values are real, so only the real-shift branch is
 *     restated and the Ritz pairs come from a symmetric eigensolve of the
 *     (symmetrised) Hessenberg matrix.
 *   - Analysis::gap_ratios                    src/analysis.cpp:433-454
 *   - Analysis::coherence                     src/analysis.cpp:542-556
 *   - single-particle density matrix <phi|b+_i b_j|phi> (the quantity that
 *     Analysis::SPDM / braket, src/analysis.cpp:497-528 and 562-594, intend).
 *   - the self-consistent mean-field order parameter: BH::h_MF
 *     (src/hamiltonian.cpp:290-309), Analysis::SF_density and Analysis::SCMF
 *     (src/analysis.cpp:93-178), with the smallest eigenpair of each
 *     (2p+1) x (2p+1) matrix from a dense symmetric eigensolve (the reference
 *     asks Spectra's SymEigsSolver for the same pair).
 *
 * Floating-point note: the tag sum is evaluated without contraction
 * (compile with -ffp-contract=off) so that it is the plain multiply-then-add
 * sequence of src/hamiltonian.cpp:91-97.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

static const int BHO_PRIMES[25] = {2,  3,  5,  7,  11, 13, 17, 19, 23, 29, 31, 37, 41,
                                   43, 47, 53, 59, 61, 67, 71, 73, 79, 83, 89, 97};

#define BHO_MAXM 25

/* ------------------------------------------------------------------ */
/* dimension                                                          */
/* ------------------------------------------------------------------ */

/* C(n, k) exactly in 64-bit (the reference's recursive int form,
 * src/hamiltonian.cpp:39-49, gives the same values for the sizes used). */
int64_t bho_binomial(int n, int k) {
    if (k < 0 || n < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    u128 r = 1;
    for (int i = 1; i <= k; ++i) r = r * (u128)(n - k + i) / (u128)i;
    return (int64_t)r;
}

int64_t bho_dimension(int m, int n) { return bho_binomial(m + n - 1, n); }

/* ------------------------------------------------------------------ */
/* lexicographic enumeration (src/hamiltonian.cpp:60-85)               */
/* ------------------------------------------------------------------ */

static int next_lexicographic(uint8_t* s, int m, int n) {
    for (int k = m - 2; k > -1; --k) {
        if (s[k] != 0) {
            s[k] -= 1;
            int part = 0;
            for (int i = 0; i <= k; ++i) part += s[i];
            s[k + 1] = (uint8_t)(n - part);
            for (int i = k + 2; i < m; ++i) s[i] = 0;
            return 1;
        }
    }
    return 0;
}

/* occ: D x m, row r = occupation of lexicographic state r. */
int bho_lex_states(int m, int n, int64_t D, uint8_t* occ) {
    if (m < 1 || m > BHO_MAXM || n < 0 || n > 255) return 1;
    uint8_t s[BHO_MAXM];
    memset(s, 0, sizeof s);
    s[0] = (uint8_t)n;
    int64_t r = 0;
    do {
        if (r >= D) return 2;
        memcpy(occ + r * m, s, (size_t)m);
        ++r;
    } while (next_lexicographic(s, m, n));
    return r == D ? 0 : 3;
}

/* Combinadic rank of an occupation in the enumeration above:
 * r = sum_{i=0}^{m-2} C(s_i + m - i - 2, m - i - 1), s_i = sum_{j>i} n_j. */
int64_t bho_rank(int m, const uint8_t* o) {
    int64_t r = 0;
    int suffix = 0;
    for (int i = m - 2; i >= 0; --i) {
        suffix += o[i + 1];
        r += bho_binomial(suffix + m - i - 2, m - i - 1);
    }
    return r;
}

/* ------------------------------------------------------------------ */
/* tags and the reference's column order                               */
/* ------------------------------------------------------------------ */

void bho_tags(int m, int64_t D, const uint8_t* occ, double* tags) {
    double lp[BHO_MAXM];
    for (int i = 0; i < m; ++i) lp[i] = log((double)BHO_PRIMES[i]);
    for (int64_t r = 0; r < D; ++r) {
        double t = 0.0;
        for (int i = 0; i < m; ++i) {
            double prod = (double)occ[r * m + i] * lp[i];
            t = t + prod;
        }
        tags[r] = t;
    }
}

static u128* g_sort_keys;
static int cmp_key(const void* a, const void* b) {
    u128 ka = g_sort_keys[*(const int32_t*)a], kb = g_sort_keys[*(const int32_t*)b];
    return ka < kb ? -1 : (ka > kb ? 1 : 0);
}

/* Reference column order of fixed_set_basis: argsort of the lexicographic
 * states by the exact prime product P = prod p_i^{n_i} (order-equivalent to
 * the double tags at every size checked), followed by the inverse
 * permutation that sort_basis's cycle loop applies (hamiltonian.cpp:109-123):
 * column argsort[r] holds lexicographic state r.
 * col_of_lex[r] = column of lex state r; lex_of_col[c] = lex state at column c. */
int bho_reference_order(int m, int64_t D, const uint8_t* occ, int32_t* col_of_lex,
                        int32_t* lex_of_col) {
    u128* keys = (u128*)malloc(sizeof(u128) * (size_t)D);
    int32_t* idx = (int32_t*)malloc(sizeof(int32_t) * (size_t)D);
    if (!keys || !idx) { free(keys); free(idx); return 1; }
    for (int64_t r = 0; r < D; ++r) {
        u128 p = 1;
        for (int i = 0; i < m; ++i)
            for (int k = 0; k < occ[r * m + i]; ++k) p *= (u128)BHO_PRIMES[i];
        keys[r] = p;
        idx[r] = (int32_t)r;
    }
    g_sort_keys = keys;
    qsort(idx, (size_t)D, sizeof(int32_t), cmp_key); /* keys are unique */
    for (int64_t r = 0; r < D; ++r) {
        col_of_lex[r] = idx[r];
        lex_of_col[idx[r]] = (int32_t)r;
    }
    free(keys);
    free(idx);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Hamiltonian terms                                                   */
/* ------------------------------------------------------------------ */

typedef struct { int32_t col; double val; } bho_entry;

static int cmp_entry(const void* a, const void* b) {
    int32_t ca = ((const bho_entry*)a)->col, cb = ((const bho_entry*)b)->col;
    return ca < cb ? -1 : (ca > cb ? 1 : 0);
}

/* Off-diagonal hopping term T = -sum_i sum_{j in nbr[i]} b+_i b_j as CSR with
 * sorted, de-duplicated columns.  Row c is the state lex_of_row[c]; the
 * column of lexicographic state r is col_of_lex[r] (pass NULL for both to use
 * lexicographic order).  Self-bonds (j == i) are rejected.
 * Call with col == NULL to obtain only row_ptr (nnz = row_ptr[D]). */
int bho_build_T(int m, int n, int64_t D, const uint8_t* occ, const int32_t* nbr_off,
                const int32_t* nbr, const int32_t* lex_of_row, const int32_t* col_of_lex,
                int64_t* row_ptr, int32_t* col, double* val) {
    (void)n;
    int maxdeg = nbr_off[m];
    bho_entry* buf = (bho_entry*)malloc(sizeof(bho_entry) * (size_t)(maxdeg > 0 ? maxdeg : 1));
    if (!buf) return 1;
    uint8_t s[BHO_MAXM];
    int64_t nz = 0;
    row_ptr[0] = 0;
    for (int64_t c = 0; c < D; ++c) {
        int64_t lr = lex_of_row ? lex_of_row[c] : c;
        const uint8_t* o = occ + lr * m;
        int cnt = 0;
        for (int i = 0; i < m; ++i) {
            if (o[i] == 0) continue;
            for (int k = nbr_off[i]; k < nbr_off[i + 1]; ++k) {
                int j = nbr[k];
                if (j == i) { free(buf); return 2; }
                memcpy(s, o, (size_t)m);
                s[i] -= 1;
                s[j] += 1;
                int64_t tr = bho_rank(m, s);
                buf[cnt].col = col_of_lex ? col_of_lex[tr] : (int32_t)tr;
                buf[cnt].val = -sqrt((double)o[i] * (double)(o[j] + 1));
                ++cnt;
            }
        }
        qsort(buf, (size_t)cnt, sizeof(bho_entry), cmp_entry);
        int w = 0;
        for (int e = 0; e < cnt; ++e) {
            if (w > 0 && buf[w - 1].col == buf[e].col)
                buf[w - 1].val += buf[e].val;
            else
                buf[w++] = buf[e];
        }
        if (col) {
            for (int e = 0; e < w; ++e) {
                col[nz + e] = buf[e].col;
                val[nz + e] = buf[e].val;
            }
        }
        nz += w;
        row_ptr[c + 1] = nz;
    }
    free(buf);
    return 0;
}

/* Diagonal interaction term V_r = 1/2 sum_i n_i (n_i - 1), row order as above. */
void bho_diag_V(int m, int64_t D, const uint8_t* occ, const int32_t* lex_of_row, double* v) {
    for (int64_t c = 0; c < D; ++c) {
        int64_t lr = lex_of_row ? lex_of_row[c] : c;
        double a = 0.0;
        for (int i = 0; i < m; ++i) {
            double ni = occ[lr * m + i];
            a += 0.5 * ni * (ni - 1.0);
        }
        v[c] = a;
    }
}

/* y = J T x + (U V - mu n) x */
typedef struct {
    int64_t D;
    const int64_t* rp;
    const int32_t* ci;
    const double* tv;
    const double* vd;
    double J, U, mu;
    int n;
} bho_op;

/* Threads of the row loops inside one IRLM solve (0 = serial, the default).
 * Row loops (the product, axpy-like updates, V Q) give the same bits with any
 * thread count; inner products are then summed in fixed 8192-row chunks, so
 * their value depends on neither the thread count nor the schedule, though it
 * differs from the serial sum in the last bits.  Used by the timed CPU
 * baseline, which must use every host core on a few large solves, the way the
 * reference's grid loop would on many (src/analysis.cpp:302). */
static int g_inner_threads = 0;

void bho_set_inner_threads(int t) { g_inner_threads = t > 0 ? t : 0; }

#define BHO_ROWS_PARALLEL _Pragma("omp parallel for schedule(static) num_threads(g_inner_threads) if (g_inner_threads > 1 && D > 65536)")

static void op_apply(const bho_op* A, const double* x, double* y) {
    const double sh = -A->mu * (double)A->n;
#pragma omp parallel for schedule(static) num_threads(g_inner_threads) if (g_inner_threads > 1 && A->D > 65536)
    for (int64_t r = 0; r < A->D; ++r) {
        double acc = 0.0;
        for (int64_t e = A->rp[r]; e < A->rp[r + 1]; ++e) acc += A->tv[e] * x[A->ci[e]];
        y[r] = A->J * acc + (A->U * A->vd[r] + sh) * x[r];
    }
}

void bho_spmv(int64_t D, const int64_t* rp, const int32_t* ci, const double* tv,
              const double* vd, int n, double J, double U, double mu, const double* x,
              double* y) {
    bho_op A = {D, rp, ci, tv, vd, J, U, mu, n};
    op_apply(&A, x, y);
}

/* ------------------------------------------------------------------ */
/* dense symmetric eigensolver (Householder + implicit-shift QL)       */
/* ------------------------------------------------------------------ */

/* Eigen-decomposition of the symmetric n x n matrix a (column-major,
 * overwritten by the eigenvectors, columns), eigenvalues ascending in w.
 * Householder tridiagonalisation followed by the implicit QL iteration with
 * Wilkinson-type shifts (Golub & Van Loan, "Matrix Computations", 8.3). */
static int sym_eig(int n, double* a, double* w) {
    if (n <= 0) return 0;
    double* d = w;
    double* e = (double*)calloc((size_t)n, sizeof(double));
    if (!e) return 1;
#define A_(i, j) a[(size_t)(j) * n + (i)]
    /* tridiagonalise: for k = n-1 .. 1 eliminate row k left of the subdiagonal */
    for (int k = n - 1; k > 0; --k) {
        int l = k - 1;
        double scale = 0.0, h = 0.0;
        for (int j = 0; j <= l; ++j) scale += fabs(A_(k, j));
        if (l == 0 || scale == 0.0) {
            e[k] = A_(k, l);
            d[k] = 0.0;
            continue;
        }
        for (int j = 0; j <= l; ++j) {
            A_(k, j) /= scale;
            h += A_(k, j) * A_(k, j);
        }
        double f = A_(k, l);
        double g = f >= 0.0 ? -sqrt(h) : sqrt(h);
        e[k] = scale * g;
        h -= f * g;
        A_(k, l) = f - g;
        f = 0.0;
        for (int j = 0; j <= l; ++j) {
            A_(j, k) = A_(k, j) / h;
            g = 0.0;
            for (int i = 0; i <= j; ++i) g += A_(j, i) * A_(k, i);
            for (int i = j + 1; i <= l; ++i) g += A_(i, j) * A_(k, i);
            e[j] = g / h;
            f += e[j] * A_(k, j);
        }
        double hh = f / (h + h);
        for (int j = 0; j <= l; ++j) {
            f = A_(k, j);
            e[j] = g = e[j] - hh * f;
            for (int i = 0; i <= j; ++i) A_(j, i) -= (f * e[i] + g * A_(k, i));
        }
        d[k] = h;
    }
    d[0] = 0.0;
    e[0] = 0.0;
    /* accumulate the transformations */
    for (int k = 0; k < n; ++k) {
        if (d[k] != 0.0) {
            for (int j = 0; j < k; ++j) {
                double g = 0.0;
                for (int i = 0; i < k; ++i) g += A_(k, i) * A_(i, j);
                for (int i = 0; i < k; ++i) A_(i, j) -= g * A_(i, k);
            }
        }
        d[k] = A_(k, k);
        A_(k, k) = 1.0;
        for (int j = 0; j < k; ++j) A_(j, k) = A_(k, j) = 0.0;
    }
    /* implicit QL on (d, e) */
    for (int i = 1; i < n; ++i) e[i - 1] = e[i];
    e[n - 1] = 0.0;
    for (int l = 0; l < n; ++l) {
        int iter = 0, mm;
        do {
            for (mm = l; mm < n - 1; ++mm) {
                double dd = fabs(d[mm]) + fabs(d[mm + 1]);
                if (fabs(e[mm]) <= 1e-300 + 2.2e-16 * dd) break;
            }
            if (mm != l) {
                if (iter++ == 60) { free(e); return 2; }
                double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
                double r = hypot(g, 1.0);
                g = d[mm] - d[l] + e[l] / (g + (g >= 0.0 ? fabs(r) : -fabs(r)));
                double s = 1.0, c = 1.0, p = 0.0;
                int i;
                for (i = mm - 1; i >= l; --i) {
                    double f = s * e[i], b = c * e[i];
                    r = hypot(f, g);
                    e[i + 1] = r;
                    if (r == 0.0) {
                        d[i + 1] -= p;
                        e[mm] = 0.0;
                        break;
                    }
                    s = f / r;
                    c = g / r;
                    g = d[i + 1] - p;
                    r = (d[i] - g) * s + 2.0 * c * b;
                    p = s * r;
                    d[i + 1] = g + p;
                    g = c * r - b;
                    for (int k = 0; k < n; ++k) {
                        f = A_(k, i + 1);
                        A_(k, i + 1) = s * A_(k, i) + c * f;
                        A_(k, i) = c * A_(k, i) - s * f;
                    }
                }
                if (r == 0.0 && i >= l) continue;
                d[l] -= p;
                e[l] = g;
                e[mm] = 0.0;
            }
        } while (mm != l);
    }
    /* sort ascending */
    for (int i = 0; i < n - 1; ++i) {
        int k = i;
        for (int j = i + 1; j < n; ++j)
            if (d[j] < d[k]) k = j;
        if (k != i) {
            double t = d[i];
            d[i] = d[k];
            d[k] = t;
            for (int r = 0; r < n; ++r) {
                t = A_(r, i);
                A_(r, i) = A_(r, k);
                A_(r, k) = t;
            }
        }
    }
#undef A_
    free(e);
    return 0;
}

int bho_sym_eig(int n, double* a, double* w) { return sym_eig(n, a, w); }

/* ------------------------------------------------------------------ */
/* IRLM restatement (Spectra GenEigsSolver, real-shift branch)         */
/* ------------------------------------------------------------------ */

/* Park-Miller minimal standard LCG as in Spectra's SimpleRandom (seed 0 is
 * mapped to 1); returns values in (-0.5, 0.5). */
void bho_start_vector(uint64_t seed, int64_t D, double* v) {
    const uint64_t M = 2147483647ULL;
    uint64_t s = seed ? (seed & M) : 1;
    for (int64_t i = 0; i < D; ++i) {
        s = (s * 16807ULL) % M;
        v[i] = (double)s / (double)M - 0.5;
    }
}

static double dotp(int64_t D, const double* a, const double* b) {
    if (g_inner_threads > 1 && D > 65536) {
        const int64_t CH = 8192;
        int64_t nch = (D + CH - 1) / CH;
        double* part = (double*)malloc(sizeof(double) * (size_t)nch);
        BHO_ROWS_PARALLEL
        for (int64_t c = 0; c < nch; ++c) {
            int64_t e = (c + 1) * CH < D ? (c + 1) * CH : D;
            double s = 0.0;
            for (int64_t i = c * CH; i < e; ++i) s += a[i] * b[i];
            part[c] = s;
        }
        double s = 0.0;
        for (int64_t c = 0; c < nch; ++c) s += part[c];
        free(part);
        return s;
    }
    double s = 0.0;
    for (int64_t i = 0; i < D; ++i) s += a[i] * b[i];
    return s;
}

/* out[j] = <V_j, w> for j < nc (V column-major, D x nc): dotp for each
 * column, or with inner threads one pass over fixed 8192-row chunks whose
 * partial sums are added in chunk order (the same value as dotp's chunked
 * form, for any thread count). */
static void gemv_t(int64_t D, const double* V, int nc, const double* w, double* out) {
    if (!(g_inner_threads > 1 && D > 65536)) {
        for (int j = 0; j < nc; ++j) out[j] = dotp(D, V + (size_t)j * D, w);
        return;
    }
    const int64_t CH = 8192;
    int64_t nch = (D + CH - 1) / CH;
    double* part = (double*)malloc(sizeof(double) * (size_t)nch * (size_t)nc);
    BHO_ROWS_PARALLEL
    for (int64_t c = 0; c < nch; ++c) {
        int64_t e = (c + 1) * CH < D ? (c + 1) * CH : D;
        for (int j = 0; j < nc; ++j) {
            const double* a = V + (size_t)j * D;
            double s = 0.0;
            for (int64_t i = c * CH; i < e; ++i) s += a[i] * w[i];
            part[(size_t)c * nc + j] = s;
        }
    }
    for (int j = 0; j < nc; ++j) {
        double s = 0.0;
        for (int64_t c = 0; c < nch; ++c) s += part[(size_t)c * nc + j];
        out[j] = s;
    }
    free(part);
}

typedef struct {
    const bho_op* A;
    int64_t D;
    int ncv;
    double* V;  /* D x ncv */
    double* H;  /* ncv x ncv, column-major */
    double* f;  /* D */
    double beta;
    int k;
    long nmatop;
} arnoldi;

#define HH(i, j) ar->H[(size_t)(j) * ar->ncv + (i)]

/* new residual orthogonal to the first i columns (Arnoldi.h expand_basis) */
static void expand_basis(arnoldi* ar, int i, uint64_t seed) {
    double* v = (double*)malloc(sizeof(double) * (size_t)ar->D);
    bho_start_vector(seed, ar->D, v);
    for (int pass = 0; pass < 3; ++pass)
        for (int j = 0; j < i; ++j) {
            double c = dotp(ar->D, ar->V + (size_t)j * ar->D, v);
            for (int64_t r = 0; r < ar->D; ++r) v[r] -= c * ar->V[(size_t)j * ar->D + r];
        }
    double nv = sqrt(dotp(ar->D, v, v));
    for (int64_t r = 0; r < ar->D; ++r) ar->f[r] = v[r] / nv;
    ar->beta = 1.0;
    free(v);
}

static void factorize_from(arnoldi* ar, int from_k, int to_m) {
    const double eps = 2.220446049250313e-16;
    const double near0 = 2.2250738585072014e-308 * 10.0;
    const double beta_thresh = eps * sqrt((double)ar->D);
    int64_t D = ar->D;
    double* w = (double*)malloc(sizeof(double) * (size_t)D);
    double* h = (double*)malloc(sizeof(double) * (size_t)to_m);
    double* vf = (double*)malloc(sizeof(double) * (size_t)to_m);
    for (int j = from_k; j < ar->ncv; ++j)
        for (int i = 0; i < ar->ncv; ++i) HH(i, j) = 0.0;
    for (int j = 0; j < from_k; ++j)
        for (int i = from_k; i < ar->ncv; ++i) HH(i, j) = 0.0;
    for (int i = from_k; i <= to_m - 1; ++i) {
        int restart = 0;
        if (ar->beta < near0) {
            expand_basis(ar, i, 2u * (unsigned)i);
            restart = 1;
        }
        double* vi = ar->V + (size_t)i * D;
        BHO_ROWS_PARALLEL
        for (int64_t r = 0; r < D; ++r) vi[r] = ar->f[r] / ar->beta;
        HH(i, i - 1) = restart ? 0.0 : ar->beta;
        op_apply(ar->A, vi, w);
        ar->nmatop++;
        int i1 = i + 1;
        gemv_t(D, ar->V, i1, w, h);
        BHO_ROWS_PARALLEL
        for (int64_t r = 0; r < D; ++r) {
            double acc = w[r];
            for (int j = 0; j < i1; ++j) acc -= ar->V[(size_t)j * D + r] * h[j];
            ar->f[r] = acc;
        }
        ar->beta = sqrt(dotp(D, ar->f, ar->f));
        double hn = sqrt(dotp(i1, h, h));
        if (ar->beta > 0.717 * hn) {
            for (int j = 0; j < i1; ++j) HH(j, i) = h[j];
            continue;
        }
        gemv_t(D, ar->V, i1, ar->f, vf);
        double oe = 0.0;
        for (int j = 0; j < i1; ++j) oe = fmax(oe, fabs(vf[j]));
        int count = 0;
        while (count < 5 && oe > eps * ar->beta) {
            if (ar->beta < beta_thresh) {
                memset(ar->f, 0, sizeof(double) * (size_t)D);
                ar->beta = 0.0;
                break;
            }
            BHO_ROWS_PARALLEL
            for (int64_t r = 0; r < D; ++r) {
                double acc = ar->f[r];
                for (int j = 0; j < i1; ++j) acc -= ar->V[(size_t)j * D + r] * vf[j];
                ar->f[r] = acc;
            }
            for (int j = 0; j < i1; ++j) h[j] += vf[j];
            ar->beta = sqrt(dotp(D, ar->f, ar->f));
            gemv_t(D, ar->V, i1, ar->f, vf);
            oe = 0.0;
            for (int j = 0; j < i1; ++j) oe = fmax(oe, fabs(vf[j]));
            ++count;
        }
        for (int j = 0; j < i1; ++j) HH(j, i) = h[j];
    }
    ar->k = to_m;
    free(w);
    free(h);
    free(vf);
}

typedef struct {
    double* val; /* ncv, ascending (SmallestReal selection) */
    double* vec; /* ncv x ncv */
    double* est; /* last row of vec */
} ritz;

static void retrieve_ritz(arnoldi* ar, ritz* rz) {
    int n = ar->ncv;
    double* S = rz->vec;
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) S[(size_t)j * n + i] = 0.5 * (HH(i, j) + HH(j, i));
    sym_eig(n, S, rz->val);
    for (int i = 0; i < n; ++i) rz->est[i] = S[(size_t)i * n + (n - 1)];
}

/* one explicit shifted QR step  H - mu I = QR,  H <- RQ + mu I,  Qacc <- Qacc Q,
 * with Givens rotations (Spectra LinAlg/UpperHessenbergQR.h semantics) */
static void shifted_qr(arnoldi* ar, double mu, double* Qacc) {
    int n = ar->ncv;
    double* c = (double*)malloc(sizeof(double) * (size_t)n);
    double* s = (double*)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; ++i) HH(i, i) -= mu;
    for (int i = 0; i < n - 1; ++i) {
        double a = HH(i, i), b = HH(i + 1, i);
        double r = hypot(a, b);
        double ci = r == 0.0 ? 1.0 : a / r, si = r == 0.0 ? 0.0 : -b / r;
        c[i] = ci;
        s[i] = si;
        /* rows i, i+1 <- G^T rows */
        for (int j = 0; j < n; ++j) {
            double x = HH(i, j), y = HH(i + 1, j);
            HH(i, j) = ci * x - si * y;
            HH(i + 1, j) = si * x + ci * y;
        }
    }
    for (int i = 0; i < n - 1; ++i) {
        double ci = c[i], si = s[i];
        for (int r = 0; r < n; ++r) {
            double x = HH(r, i), y = HH(r, i + 1);
            HH(r, i) = ci * x - si * y;
            HH(r, i + 1) = si * x + ci * y;
        }
        for (int r = 0; r < n; ++r) {
            double x = Qacc[(size_t)i * n + r], y = Qacc[(size_t)(i + 1) * n + r];
            Qacc[(size_t)i * n + r] = ci * x - si * y;
            Qacc[(size_t)(i + 1) * n + r] = si * x + ci * y;
        }
    }
    for (int i = 0; i < n; ++i) HH(i, i) += mu;
    free(c);
    free(s);
}

static void irlm_restart(arnoldi* ar, ritz* rz, int k) {
    int n = ar->ncv;
    int64_t D = ar->D;
    if (k >= n) return;
    double* Q = (double*)calloc((size_t)n * n, sizeof(double));
    for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;
    for (int i = k; i < n; ++i) shifted_qr(ar, rz->val[i], Q);
    /* V <- V Q(:, 0:k), f <- V Q(:,k) H(k,k-1) + f Q(n-1,k-1) */
    double* Vn = (double*)malloc(sizeof(double) * (size_t)D * (size_t)(k + 1));
    /* per row, the same t-ascending accumulation as a column-by-column pass */
    const int64_t RB = 4096;
    BHO_ROWS_PARALLEL
    for (int64_t r0 = 0; r0 < D; r0 += RB) {
        int64_t r1 = r0 + RB < D ? r0 + RB : D;
        for (int j = 0; j <= k; ++j) {
            double* out = Vn + (size_t)j * D;
            for (int64_t r = r0; r < r1; ++r) out[r] = 0.0;
            for (int t = 0; t < n; ++t) {
                double q = Q[(size_t)j * n + t];
                if (q == 0.0) continue;
                const double* vt = ar->V + (size_t)t * D;
                for (int64_t r = r0; r < r1; ++r) out[r] += q * vt[r];
            }
        }
    }
    double qf = Q[(size_t)(k - 1) * n + (n - 1)];
    double hk = HH(k, k - 1);
    BHO_ROWS_PARALLEL
    for (int64_t r = 0; r < D; ++r) ar->f[r] = Vn[(size_t)k * D + r] * hk + ar->f[r] * qf;
    memcpy(ar->V, Vn, sizeof(double) * (size_t)D * (size_t)k);
    ar->beta = sqrt(dotp(D, ar->f, ar->f));
    ar->k = k;
    free(Vn);
    free(Q);
    factorize_from(ar, k, n);
    retrieve_ritz(ar, rz);
}

/* Returns the number of converged eigenvalues (<= nev).  evals receives the
 * converged Ritz values in the reference's output order (descending |lambda|,
 * GenEigsBase.h:417,466-483); evecs (optional, D x nev column-major) the
 * matching Ritz vectors; *niter the restart count; *nop the operator count. */
int bho_irlm(int64_t D, const int64_t* rp, const int32_t* ci, const double* tv,
             const double* vd, int n_bosons, double J, double U, double mu, int nev,
             int maxit, double tol, double* evals, double* evecs, int* niter, long* nop) {
    int ncv = 2 * nev + 1;
    if (nev < 1 || nev > D - 2 || ncv > D) return -1;
    bho_op A = {D, rp, ci, tv, vd, J, U, mu, n_bosons};
    arnoldi ar;
    ar.A = &A;
    ar.D = D;
    ar.ncv = ncv;
    ar.V = (double*)calloc((size_t)D * ncv, sizeof(double));
    ar.H = (double*)calloc((size_t)ncv * ncv, sizeof(double));
    ar.f = (double*)calloc((size_t)D, sizeof(double));
    ar.nmatop = 0;
    double* v0 = (double*)malloc(sizeof(double) * (size_t)D);
    double* w = (double*)malloc(sizeof(double) * (size_t)D);
    ritz rz;
    rz.val = (double*)malloc(sizeof(double) * ncv);
    rz.vec = (double*)malloc(sizeof(double) * (size_t)ncv * ncv);
    rz.est = (double*)malloc(sizeof(double) * ncv);
    const double eps = 2.220446049250313e-16;
    const double eps23 = pow(eps, 2.0 / 3.0);

    /* Arnoldi init (Arnoldi.h:132-180) */
    bho_start_vector(0, D, v0);
    op_apply(&A, v0, ar.V);
    ar.nmatop++;
    double vn = sqrt(dotp(D, ar.V, ar.V));
    for (int64_t r = 0; r < D; ++r) ar.V[r] /= vn;
    op_apply(&A, ar.V, w);
    ar.nmatop++;
    ar.H[0] = dotp(D, ar.V, w);
    double fmax_ = 0.0;
    for (int64_t r = 0; r < D; ++r) {
        ar.f[r] = w[r] - ar.V[r] * ar.H[0];
        fmax_ = fmax(fmax_, fabs(ar.f[r]));
    }
    if (fmax_ < eps * fabs(ar.H[0])) {
        memset(ar.f, 0, sizeof(double) * (size_t)D);
        ar.beta = 0.0;
    } else {
        ar.beta = sqrt(dotp(D, ar.f, ar.f));
    }
    ar.k = 1;

    factorize_from(&ar, 1, ncv);
    retrieve_ritz(&ar, &rz);
    int it, nconv = 0;
    int* conv = (int*)calloc((size_t)ncv, sizeof(int));
    for (it = 0; it < maxit; ++it) {
        nconv = 0;
        for (int i = 0; i < nev; ++i) {
            double thr = tol * fmax(eps23, fabs(rz.val[i]));
            double res = fabs(rz.est[i]) * ar.beta;
            conv[i] = res < thr;
            nconv += conv[i];
        }
        if (nconv >= nev) break;
        /* nev_adjusted (GenEigsBase.h:161-193) */
        const double near0 = 2.2250738585072014e-308 * 10.0;
        int nev_new = nev;
        for (int i = nev; i < ncv; ++i)
            if (fabs(rz.est[i]) < near0) nev_new++;
        int add = (ncv - nev_new) / 2;
        nev_new += nconv < add ? nconv : add;
        if (nev_new == 1 && ncv >= 6)
            nev_new = ncv / 2;
        else if (nev_new == 1 && ncv > 3)
            nev_new = 2;
        if (nev_new > ncv - 2) nev_new = ncv - 2;
        irlm_restart(&ar, &rz, nev_new);
    }
    /* final ordering: converged wanted values sorted by descending magnitude */
    int* ord = (int*)malloc(sizeof(int) * nev);
    for (int i = 0; i < nev; ++i) ord[i] = i;
    for (int i = 0; i < nev; ++i)
        for (int j = i + 1; j < nev; ++j)
            if (fabs(rz.val[ord[j]]) > fabs(rz.val[ord[i]])) {
                int t = ord[i];
                ord[i] = ord[j];
                ord[j] = t;
            }
    int outc = 0;
    for (int q = 0; q < nev; ++q) {
        int i = ord[q];
        if (!conv[i]) continue;
        evals[outc] = rz.val[i];
        if (evecs) {
            double* out = evecs + (size_t)outc * D;
            for (int64_t r = 0; r < D; ++r) out[r] = 0.0;
            for (int t = 0; t < ncv; ++t) {
                double y = rz.vec[(size_t)i * ncv + t];
                const double* vt = ar.V + (size_t)t * D;
                for (int64_t r = 0; r < D; ++r) out[r] += y * vt[r];
            }
        }
        ++outc;
    }
    if (niter) *niter = it + 1;
    if (nop) *nop = ar.nmatop;
    free(ord);
    free(conv);
    free(ar.V);
    free(ar.H);
    free(ar.f);
    free(v0);
    free(w);
    free(rz.val);
    free(rz.vec);
    free(rz.est);
    return outc;
}

/* Many independent IRLM solves sharing one (T, V) pattern, one per thread
 * (the reference's OpenMP grid loop, src/analysis.cpp:302-314).  evals is
 * nsolve x nev (reference order per solve), nconv_out per solve. */
int bho_irlm_batch(int64_t D, const int64_t* rp, const int32_t* ci, const double* tv,
                   const double* vd, int n_bosons, int nsolve, const double* J,
                   const double* U, const double* mu, int nev, int maxit, double tol,
                   int nthreads, double* evals, int* nconv_out) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
#endif
    for (int s = 0; s < nsolve; ++s) {
        nconv_out[s] = bho_irlm(D, rp, ci, tv, vd, n_bosons, J[s], U[s], mu[s], nev, maxit, tol,
                                evals + (size_t)s * nev, NULL, NULL, NULL);
    }
    (void)nthreads;
    return 0;
}

/* One wave of the reference's grid loop (src/analysis.cpp:302): nsolve
 * independent IRLM solves of one operator run `groups` at a time (OpenMP,
 * dynamic schedule), each solve's row loops on `inner` threads (nested
 * parallelism; inner = 1 is the reference's own one-solve-per-thread form).
 * evals nsolve x nev (reference order), nconv_out per solve. */
int bho_irlm_wave(int64_t D, const int64_t* rp, const int32_t* ci, const double* tv,
                  const double* vd, int n_bosons, int nsolve, const double* J,
                  const double* U, const double* mu, int nev, int maxit, double tol,
                  int groups, int inner, double* evals, int* nconv_out) {
    const int saved = g_inner_threads;
    g_inner_threads = inner > 1 ? inner : 0;
#ifdef _OPENMP
    if (inner > 1) omp_set_max_active_levels(2);
#pragma omp parallel for schedule(dynamic) num_threads(groups > 0 ? groups : 1)
#endif
    for (int s = 0; s < nsolve; ++s) {
        nconv_out[s] = bho_irlm(D, rp, ci, tv, vd, n_bosons, J[s], U[s], mu[s], nev, maxit, tol,
                                evals + (size_t)s * nev, NULL, NULL, NULL);
    }
    g_inner_threads = saved;
    return 0;
}

int bho_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* observables                                                         */
/* ------------------------------------------------------------------ */

/* gap ratios r_i = min(gap)/max(gap) over the sorted values (analysis.cpp:433-454);
 * returns the mean over the nev-2 ratios. */
double bho_gap_ratio(int nev, const double* evals, double* ratios) {
    double* s = (double*)malloc(sizeof(double) * nev);
    memcpy(s, evals, sizeof(double) * nev);
    for (int i = 0; i < nev; ++i)
        for (int j = i + 1; j < nev; ++j)
            if (s[j] < s[i]) {
                double t = s[i];
                s[i] = s[j];
                s[j] = t;
            }
    double sum = 0.0;
    for (int i = 1; i < nev - 1; ++i) {
        double a = s[i + 1] - s[i], b = s[i] - s[i - 1];
        double mn = a < b ? a : b, mx = a < b ? b : a;
        double r = mx != 0.0 ? mn / mx : 0.0;
        if (ratios) ratios[i - 1] = r;
        sum += r;
    }
    free(s);
    return nev > 2 ? sum / (nev - 2) : 0.0;
}

/* rho_ij = <phi| b+_i b_j |phi> for a real phi in lexicographic order. */
void bho_spdm(int m, int n, int64_t D, const uint8_t* occ, const double* phi, double* rho) {
    (void)n;
    uint8_t s[BHO_MAXM];
    for (int i = 0; i < m * m; ++i) rho[i] = 0.0;
    for (int64_t r = 0; r < D; ++r) {
        const uint8_t* o = occ + r * m;
        if (phi[r] == 0.0) continue;
        for (int i = 0; i < m; ++i) {
            rho[i * m + i] += phi[r] * phi[r] * o[i];
            for (int j = 0; j < m; ++j) {
                if (j == i || o[j] == 0) continue;
                memcpy(s, o, (size_t)m);
                s[j] -= 1;
                s[i] += 1;
                int64_t t = bho_rank(m, s);
                /* <t| b+_i b_j |r> = sqrt((n_i+1) n_j) */
                rho[i * m + j] += phi[t] * phi[r] * sqrt((double)(o[i] + 1) * (double)o[j]);
            }
        }
    }
}

/* coherence K = sum_{i!=j} |rho_ij|^2 / sum |rho_ij|^2 (analysis.cpp:542-556) */
double bho_coherence(int m, const double* rho) {
    double all = 0.0, diag = 0.0;
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) {
            double v = rho[i * m + j] * rho[j * m + i];
            all += v;
            if (i == j) diag += v;
        }
    return (all - diag) / all;
}

/* condensate fraction: largest eigenvalue of rho over its trace
 * (analysis.cpp:331-334) */
double bho_condensate_fraction(int m, const double* rho) {
    double* a = (double*)malloc(sizeof(double) * m * m);
    double* w = (double*)malloc(sizeof(double) * m);
    memcpy(a, rho, sizeof(double) * m * m);
    sym_eig(m, a, w);
    double tr = 0.0, mx = 0.0;
    for (int i = 0; i < m; ++i) {
        tr += rho[i * m + i];
        if (fabs(w[i]) > fabs(mx)) mx = w[i];
    }
    free(a);
    free(w);
    return fabs(mx / tr);
}

/* ------------------------------------------------------------------ */
/* self-consistent mean field (src/analysis.cpp:93-178)               */
/* ------------------------------------------------------------------ */

/* Smallest eigenpair of the (2p+1) x (2p+1) matrix of BH::h_MF
 * (src/hamiltonian.cpp:290-309): diagonal -mu i + i (i-1) / 2 + q J psi^2,
 * entries (i+1, i) = (i, i+1) = -q J psi sqrt(i+1).  phi gets the vector. */
static int scmf_ground(double psi, int p, double mu, double J, int q, double* phi, double* e0) {
    const int N = 2 * p + 1;
    double* a = (double*)calloc((size_t)N * N, sizeof(double));
    double* w = (double*)malloc(sizeof(double) * N);
    if (!a || !w) {
        free(a);
        free(w);
        return 1;
    }
    for (int i = 0; i < N; ++i) a[(size_t)i * N + i] = -mu * i + 0.5 * i * (i - 1) + q * J * psi * psi;
    for (int i = 0; i + 1 < N; ++i) {
        const double v = -q * J * psi * sqrt((double)(i + 1));
        a[(size_t)i * N + i + 1] = v;
        a[(size_t)(i + 1) * N + i] = v;
    }
    const int rc = sym_eig(N, a, w);
    *e0 = w[0];
    for (int i = 0; i < N; ++i) phi[i] = a[i]; /* column 0 */
    free(a);
    free(w);
    return rc;
}

/* Analysis::SCMF: grow the truncation p from 1 until the ground energy moves
 * by at most eps = 10^-precision, set psi = sum_{i=1}^{2p} sqrt(i) phi_i
 * phi_{i-1} (Analysis::SF_density), repeat until psi moves by at most eps.
 * Returns psi (NaN if p would exceed pmax); *outer gets the psi updates. */
double bho_scmf(double mu, double J, int q, double psi0, int precision, int pmax, int* outer) {
    const double eps = pow(10.0, -precision);
    double psi = psi0, tmp;
    double* phi = (double*)malloc(sizeof(double) * (2 * pmax + 1));
    int it = 0;
    if (!phi) return NAN;
    do {
        int p = 1;
        double e0, e1;
        if (scmf_ground(psi, p, mu, J, q, phi, &e0)) {
            free(phi);
            return NAN;
        }
        do {
            ++p;
            if (p > pmax || scmf_ground(psi, p, mu, J, q, phi, &e1)) {
                free(phi);
                return NAN;
            }
            tmp = fabs(e0 - e1);
            e0 = e1;
        } while (tmp > eps);
        double a = 0.0;
        for (int i = 1; i < 2 * p + 1; ++i) a += sqrt((double)i) * phi[i] * phi[i - 1];
        ++it;
        tmp = fabs(a - psi);
        psi = a;
    } while (tmp > eps);
    free(phi);
    if (outer) *outer = it;
    return psi;
}

/* bho_scmf over npts points in parallel (OpenMP); psi[k], outer[k]. */
void bho_scmf_batch(int npts, const double* mu, const double* J, int q, const double* psi0,
                    int precision, int pmax, int nthreads, double* psi, int* outer) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
#endif
    for (int k = 0; k < npts; ++k) psi[k] = bho_scmf(mu[k], J[k], q, psi0[k], precision, pmax, outer ? &outer[k] : 0);
}
