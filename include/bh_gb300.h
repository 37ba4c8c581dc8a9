/*
 * bh_gb300.h -- C ABI of the GB300-native exact-diagonalisation engine for the
 * Bose-Hubbard model.
 *
 * Every entry point is a plain C function over plain pointers and sizes.  The
 * library owns device memory behind opaque handles (bh_basis, bh_hamiltonian)
 * and writes results into caller-allocated HOST buffers.  Every function
 * returns a status code (BH_OK on success); bh_last_error() gives the message
 * of the last failure on the calling thread.
 *
 * The comment above each declaration names the reference interface it
 * replaces (Maximilien-Hantonne/Bose-Hubbard-Phase-Transition, file:line).
 *
 * Conventions
 *  - Hamiltonian  H = J T + U V - mu N,  T = -sum_i sum_{j in nbr(i)} b+_i b_j,
 *    V = 1/2 sum_i n_i (n_i - 1), N = sum_i n_i (= n in a fixed-n sector).
 *  - "reference order" is the column order of BH::fixed_set_basis
 *    (hamiltonian.cpp:143-149); "lexicographic order" is the order of
 *    BH::init_lexicographic (hamiltonian.cpp:75-85).
 *  - Neighbour lists are CSR-like: nbr[off[i] .. off[i+1]) are the neighbours
 *    of site i, as std::vector<std::vector<int>> Neighbours::getNeighbours()
 *    (neighbours.cpp:126-128) holds them.
 */
#ifndef BH_GB300_H
#define BH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference throws; see bh_reference_api.hpp) ---- */
#define BH_OK 0
#define BH_ERR_ARG 1       /* invalid argument (std::invalid_argument)            */
#define BH_ERR_NOCONV 2    /* not converged ("Eigenvalue computation failed.")    */
#define BH_ERR_BREAKDOWN 3 /* Krylov breakdown that could not be recovered        */
#define BH_ERR_TIMEOUT 4   /* a bounded device wait ran out                        */
#define BH_ERR_CUDA 5      /* CUDA runtime error                                   */
#define BH_ERR_NOMEM 6     /* device or host allocation failed                     */

#define BH_ORDER_REFERENCE 0
#define BH_ORDER_LEX 1

#define BH_PREC_FP64 0  /* vectors, SpMV and recurrence in FP64 (the plain method) */
#define BH_PREC_MIXED 1 /* FP32 vectors/SpMM, FP64 coefficients + FP64 refinement  */

typedef struct bh_basis bh_basis;
typedef struct bh_hamiltonian bh_hamiltonian;

/* Message of the last failing call on this thread ("" if none). */
const char* bh_last_error(void);
/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
int bh_version(void);

/* ---------------------------------------------------------------------- */
/* Lattice (host)                                                          */
/* ---------------------------------------------------------------------- */

/* Replaces Neighbours::chain_neighbours (neighbours.cpp:21-34): 1D chain,
 * periodic when closed != 0.  Writes off[m+1] and up to cap entries of nbr;
 * *count receives the total number of entries. */
int bh_neighbours_chain(int m, int closed, int32_t* off, int32_t* nbr, int cap, int* count);
/* Replaces Neighbours::square_neighbours (neighbours.cpp:40-71) with the
 * lists that function intends (the reference fills a shadowing local and
 * returns empty lists).  m must be a perfect square (else BH_ERR_ARG, the
 * reference's std::invalid_argument). */
int bh_neighbours_square(int m, int closed, int32_t* off, int32_t* nbr, int cap, int* count);
/* Replaces Neighbours::cube_neighbours (neighbours.cpp:77-120), as above;
 * m must be a perfect cube. */
int bh_neighbours_cube(int m, int closed, int32_t* off, int32_t* nbr, int cap, int* count);

/* ---------------------------------------------------------------------- */
/* Fock basis                                                              */
/* ---------------------------------------------------------------------- */

/* Replaces BH::dimension / BH::binomial (hamiltonian.cpp:39-54). */
int bh_dimension(int m, int n, int64_t* dim);

/* Replaces BH::fixed_set_basis (hamiltonian.cpp:143-149): builds the basis
 * on the device (combinadic unranking, exact 128-bit prime-product keys,
 * device radix sort).  m <= 25 (the reference's primes table). */
int bh_basis_create(int m, int n, bh_basis** out);
int bh_basis_destroy(bh_basis* b);
int bh_basis_info(const bh_basis* b, int* m, int* n, int64_t* dim);
/* Copies the basis out in the reference's representation.  Any pointer may
 * be NULL.  tags[D] and basis[m*D] (column-major, column c = occupation of
 * the state at reference column c) equal the pair fixed_set_basis returns;
 * col_of_lex[D] maps lexicographic index -> reference column and
 * lex_of_col[D] the inverse. */
int bh_basis_copy(const bh_basis* b, double* tags, double* basis, int32_t* col_of_lex,
                  int32_t* lex_of_col);
/* Replaces BH::search_tag on the exact state (hamiltonian.cpp:126-140):
 * reference column of each of nq occupations occ[nq*m] (uint8, row-major);
 * -1 where the occupation is not in the sector. */
int bh_basis_index(const bh_basis* b, int64_t nq, const uint8_t* occ, int32_t* col);

/* ---------------------------------------------------------------------- */
/* Hamiltonian                                                             */
/* ---------------------------------------------------------------------- */

/* Replaces BH::fixed_bosons_hamiltonian / fill_hopping / fill_interaction /
 * fill_chemical (hamiltonian.cpp:170-256): assembles the hopping term T
 * (warp per row CSR, sorted columns, duplicate bonds merged) and the
 * diagonal V on the device, once, for all (J, U, mu).  The neighbour lists
 * must be symmetric and free of self-bonds. */
int bh_hamiltonian_create(const bh_basis* b, const int32_t* nbr_off, const int32_t* nbr,
                          bh_hamiltonian** out);
/* The same operator without stored matrix entries (replaces the same
 * reference functions as bh_hamiltonian_create): every product regenerates
 * the rows of T and V from the states' occupations packed into one uint64
 * each (ceil(log2(n+1)) bits per site, so m * bits <= 64 is required), with
 * combinadic ranking of each hopped state; at most 128 directed bonds.
 * Device memory: 8 bytes per state instead of about 12 per stored entry.
 * Every entry point that takes a Hamiltonian accepts either kind;
 * bh_hamiltonian_csr assembles the stored form on request. */
int bh_hamiltonian_create_matrix_free(const bh_basis* b, const int32_t* nbr_off,
                                      const int32_t* nbr, bh_hamiltonian** out);
/* *matrix_free = 1 for a Hamiltonian made by bh_hamiltonian_create_matrix_free. */
int bh_hamiltonian_is_matrix_free(const bh_hamiltonian* h, int* matrix_free);
int bh_hamiltonian_destroy(bh_hamiltonian* h);
/* Number of off-diagonal entries of T (stored, or of the equivalent stored
 * form for a matrix-free Hamiltonian). */
int bh_hamiltonian_nnz(const bh_hamiltonian* h, int64_t* nnz_offdiag);
/* Writes H = J T + U V - mu N as CSR into host buffers, rows and columns in
 * `order`, with one (explicit, possibly zero) diagonal entry per row and
 * sorted columns: row_ptr[D+1], col[nnz_offdiag + D], val[nnz_offdiag + D]. */
int bh_hamiltonian_csr(const bh_hamiltonian* h, int order, double J, double U, double mu,
                       int64_t* row_ptr, int32_t* col, double* val);
/* Replaces BH::max_bosons_hamiltonian (hamiltonian.cpp:260-288): the
 * block-diagonal H = J T + U V - mu N of nh sectors (usually n_min..n_max of
 * one lattice), assembled on the device, sector k's rows and columns offset
 * by the dimensions of sectors 0..k-1, each block in `order`, one explicit
 * diagonal entry per row: row_ptr[sum D_k + 1], col/val[sum (nnz_k + D_k)]. */
int bh_hamiltonian_multi_csr(int nh, const bh_hamiltonian* const* hs, int order, double J, double U,
                             double mu, int64_t* row_ptr, int32_t* col, double* val);
/* y = H x for nvec vectors (x, y: host, row-major [D][nvec], `order`). */
int bh_hamiltonian_apply(const bh_hamiltonian* h, int order, double J, double U, double mu,
                         int nvec, const double* x, double* y);
/* No counterpart in the reference.  y = H x like bh_hamiltonian_apply, for
 * callers that cannot allocate device memory while they run (a host
 * application that hands out device memory once from its own pool, or many
 * host threads sharing one GPU, where cudaMalloc/cudaFree serialise against
 * all other device work): x and y are DEVICE pointers [D][nvec] in `order`,
 * the work is queued on `stream` (a cudaStream_t, NULL = legacy default
 * stream) and the call returns when it has finished.  It allocates nothing:
 * its working memory is a fixed 32 MiB device array inside the library
 * (4 Mi doubles), shared by all calls and kept by every GPU that loads the
 * library until exit, so 2 * D * nvec must not exceed 4 Mi - 32 doubles in
 * the reference order (BH_ERR_ARG otherwise; the lexicographic order needs no
 * vector scratch, but there x and y must not overlap: BH_ERR_ARG).  The first
 * call on each device looks up that array's device address and should come
 * before any stream capture; the address is kept for the device's context, so
 * after a cudaDeviceReset the process must not call this entry point again on
 * that device.  Calls that overlap on the GPU race on the shared array:
 * serialise them. */
int bh_hamiltonian_apply_noalloc(const bh_hamiltonian* h, int order, double J, double U,
                                 double mu, int nvec, const double* x, double* y, void* stream);

/* ---------------------------------------------------------------------- */
/* Eigensolver                                                             */
/* ---------------------------------------------------------------------- */

typedef struct bh_solver_opts {
    int nev;          /* wanted lowest eigenvalues (the reference's nb_eigen)         */
    int ncv;          /* max Krylov basis size per solve; 0 = max(7 nev, nev + 8 block) */
    int block;        /* block size p (>= degeneracy to resolve); 0 = automatic       */
    int precision;    /* BH_PREC_FP64 or BH_PREC_MIXED                                 */
    int max_restarts; /* restart cap (the reference's maxit = 1000)                    */
    double tol;       /* relative residual tolerance; 0 = 1e-10 (FP64) / auto (mixed) */
    uint64_t seed;    /* start block seed (Spectra SimpleRandom seed; 0 == 1)          */
    int want_vectors; /* nonzero: return Ritz vectors                                  */
    int order;        /* order of returned vectors: BH_ORDER_REFERENCE or BH_ORDER_LEX */
} bh_solver_opts;

typedef struct bh_solve_info {
    int nconv;         /* converged eigenvalues (per solve, minimum over a batch) */
    int restarts;      /* thick restarts performed                                */
    int64_t matvecs;   /* H x products per solve                                  */
    double max_resid;  /* max relative residual of the returned pairs             */
    double seconds;    /* wall time of the call                                   */
    int64_t launches;  /* kernels launched by the call                            */
} bh_solve_info;

void bh_solver_opts_default(bh_solver_opts* o);

/* Replaces Op::IRLM_eigen (operator.cpp:22-33) for one (J, U, mu) point of a
 * built Hamiltonian: the nev lowest eigenvalues, ascending, in evals[nev];
 * per-pair relative residuals in resid[nev] (may be NULL); Ritz vectors in
 * evecs[nev*D] (row i = vector i, in opts->order; may be NULL).  Returns
 * BH_ERR_NOCONV ("Eigenvalue computation failed.") when fewer than nev pairs
 * converged and BH_ERR_BREAKDOWN when the Krylov space was exhausted first.
 * Every entry point rejects non-finite J, U, mu (and tol, matrix values)
 * with BH_ERR_ARG before any device work. */
int bh_eigsh(const bh_hamiltonian* h, double J, double U, double mu, const bh_solver_opts* o,
             double* evals, double* resid, double* evecs, bh_solve_info* info);

/* Replaces Op::IRLM_eigen (operator.cpp:22-33) on an arbitrary symmetric
 * matrix given as CSR in host memory (Eigen's compressed storage of a
 * symmetric matrix can be passed as is).  Same outputs as bh_eigsh. */
int bh_eigsh_csr(int64_t dim, const int64_t* row_ptr, const int32_t* col, const double* val,
                 const bh_solver_opts* o, double* evals, double* resid, double* evecs,
                 bh_solve_info* info);

/* Replaces the OpenMP grid loop of Analysis::calculate_and_save
 * (analysis.cpp:302-314): nsolve (J, U, mu) points of one Hamiltonian solved
 * together as one batch (shared-pattern SpMM, device-resident Krylov loop).
 * evals[nsolve*nev] ascending per solve; resid[nsolve*nev] (may be NULL);
 * nconv[nsolve] (may be NULL). */
int bh_eigsh_batch(const bh_hamiltonian* h, int nsolve, const double* J, const double* U,
                   const double* mu, const bh_solver_opts* o, double* evals, double* resid,
                   int* nconv, bh_solve_info* info);
/* bh_eigsh_batch with a status per point (the reference's grid loop calls
 * Op::IRLM_eigen per point, which throws std::runtime_error("Eigenvalue
 * computation failed.") on non-convergence, operator.cpp:27-29, and Spectra
 * throws on an exhausted Krylov space, GenEigsBase.h:335-339):
 * status[nsolve] receives BH_OK, BH_ERR_NOCONV (fewer than nev pairs
 * converged within max_restarts, or Ritz vectors not independent in the final
 * FP64 refinement) or BH_ERR_BREAKDOWN (the point's Krylov space held fewer
 * than nev directions: an invariant start block, e.g. H a multiple of the
 * identity; its evals hold the values it found, NaN beyond them).  The call
 * itself returns BH_OK when it ran; one failing point does not stop the
 * others.  bh_eigsh_batch is this call without status (nconv[s] < nev marks a
 * failed point there). */
int bh_eigsh_batch_status(const bh_hamiltonian* h, int nsolve, const double* J, const double* U,
                          const double* mu, const bh_solver_opts* o, double* evals, double* resid,
                          int* nconv, int* status, bh_solve_info* info);
/* bh_eigsh_batch with the eigenvectors: evecs[(s*nev + i)*D + r] (host,
 * D*nev doubles per solve, rows in o->order), the i-th lowest eigenvector of
 * solve s (FP64 Rayleigh-Ritz vectors of either precision). */
int bh_eigsh_batch_vectors(const bh_hamiltonian* h, int nsolve, const double* J, const double* U,
                           const double* mu, const bh_solver_opts* o, double* evals, double* resid,
                           int* nconv, double* evecs, bh_solve_info* info);
/* The same batch over nh Hamiltonians (the particle-number sectors of a
 * phase diagram, of uneven dimension) in one call: the sectors run
 * concurrently on the device, each on its own stream driven by its own host
 * thread (sequentially while per-kernel timing is on).  mu is applied as
 * -mu[s] * n_k in sector k.  evals[(k*nsolve + s)*nev + i], resid likewise,
 * nconv[k*nsolve + s]; info aggregates (matvecs and launches summed,
 * restarts = the largest of the sectors). */
int bh_eigsh_batch_sectors(int nh, const bh_hamiltonian* const* hs, int nsolve, const double* J,
                           const double* U, const double* mu, const bh_solver_opts* o,
                           double* evals, double* resid, int* nconv, bh_solve_info* info);

/* Replaces Op::FOLM_diag (operator.cpp:39-71): nb_iter Lanczos steps of the
 * symmetric CSR matrix (host arrays, as bh_eigsh_csr) from the start vector
 * v0[dim] (normalised in place, as the reference does), FP64 with full
 * re-orthogonalisation of every new vector against all earlier ones.
 * T[nb_iter * nb_iter] receives the tridiagonal matrix (T_ii = alpha_i,
 * T_{i,i+1} = T_{i+1,i} = beta_i, zeros beyond the steps taken) and
 * V[nb_iter * dim] the Krylov vectors as columns (V[j * dim + r], column-major
 * like Eigen::MatrixXd); *steps (optional) the number of vectors: fewer than
 * nb_iter once beta_i < 1e-6 (the reference's breakdown test).  The
 * reference's own loop leaves v_i out of the orthogonalisation and stores
 * beta_i one row late; this gives the matrix the method defines. */
int bh_folm_diag_csr(int64_t dim, const int64_t* row_ptr, const int32_t* col, const double* val, int nb_iter,
                     double* v0, double* T, double* V, int* steps);

/* Replaces Op::exact_eigen (operator.cpp:92-101): all eigenvalues (ascending)
 * and, if z != NULL, eigenvectors (columns of z, column-major n x n) of the
 * dense symmetric matrix a (column-major, host).  n <= 32768. */
int bh_dense_eigh(int64_t n, const double* a, double* w, double* z);

/* ---------------------------------------------------------------------- */
/* Observables                                                             */
/* ---------------------------------------------------------------------- */

/* Replaces Analysis::gap_ratios (analysis.cpp:433-454): ratios[nev-2] of the
 * sorted values; returns the mean in *mean. */
int bh_gap_ratios(int nev, const double* evals, double* ratios, double* mean);

/* Replaces Analysis::SPDM / braket (analysis.cpp:497-528, 562-594) with the
 * single-particle density matrix they intend: rho[m*m] (row-major) =
 * <phi| b+_i b_j |phi> for a real vector phi[D] given in `order`. */
int bh_spdm(const bh_hamiltonian* h, int order, const double* phi, double* rho);

/* Phase-map composition over particle-number sectors (the exact path's
 * boson density / compressibility, with mu applied as the -mu n shift):
 * e0[nsec*nJ] ground energies at mu = 0 for sectors n_lo..n_lo+nsec-1,
 * mu[nmu]; outputs density[nJ*nmu] = nbest / m with
 * nbest = argmin_n E0(n) - mu n, and compressibility[nJ*nmu] = d density / d mu
 * (central differences, one-sided at the ends of the mu grid). */
int bh_phase_map(int m, int n_lo, int nsec, int nJ, const double* e0, int nmu, const double* mu,
                 double* density, double* compressibility);

/* ---------------------------------------------------------------------- */
/* Mean field                                                              */
/* ---------------------------------------------------------------------- */

/* Replaces Analysis::SCMF / SF_density (analysis.cpp:93-178) with BH::h_MF
 * (hamiltonian.cpp:290-309) for npts points at once, one device thread per
 * point: psi[k] is the self-consistent order parameter at (mu[k], J[k]) with
 * q neighbours from the seed psi0[k], to eps = 10^-precision (precision in
 * [0, 15]).  iters[k] (optional) = psi updates, -1 where the truncation would
 * exceed 2p+1 = 97 levels (psi NaN), -2 where psi still moved after 20000
 * updates.  Where psi = 0 or J = 0 the single-site matrix is diagonal and its
 * ground vector is the first lowest level, so psi = 0 stays 0 (the
 * reference's Lanczos mixes tied levels there, at integer mu). */
int bh_scmf(int npts, const double* mu, const double* J, int q, const double* psi0, int precision,
            double* psi, int* iters);
/* Replaces Analysis::mean_field_parameters (analysis.cpp:58-89): the grid
 * mu = 0, dmu, ... < 4 and J = 0, dJ, ... < 0.25 (dmu = 4/n, dJ = 0.25/n,
 * built by repeated addition as the reference's range loops are, so up to
 * n + 1 values each), seeds psi0 uniform in [0, 1) from splitmix64(seed, k)
 * (the reference draws them from std::random_device).  mu_out and J_out need
 * n + 1 entries, psi_out (n + 1)^2; on return psi_out[i * nJ + k] belongs to
 * (mu_out[i], J_out[k]). */
int bh_mean_field_grid(int n, int precision, int q, uint64_t seed, int* nmu, int* nJ,
                       double* mu_out, double* J_out, double* psi_out);

/* ---------------------------------------------------------------------- */
/* Tracing (no counterpart in the reference beyond Resource::timer,        */
/* src/resource.cpp:55-71): per-kernel device time from CUDA events.       */
/* ---------------------------------------------------------------------- */

/* Turns per-kernel event timing on or off (process-wide; off by default). */
int bh_profile_enable(int on);
/* Clears the accumulated totals. */
int bh_profile_reset(void);
/* Number of distinct kernels with totals. */
int bh_profile_count(int* n);
/* Totals of kernel i: name, launches, device milliseconds and algorithmic
 * bytes (every operand read once and every result written once). */
int bh_profile_get(int i, char* name, int name_cap, int64_t* launches, double* ms, double* bytes);

/* ---------------------------------------------------------------------- */
/* Launch shapes of the sparse product and their autotuner (no counterpart */
/* in the reference, whose product is Eigen's serial SparseMatrix * vector */
/* in Spectra's SparseGenMatProd::perform_op, SparseGenMatProd.h:81-86).   */
/*                                                                         */
/* The product Y = H X over nvec columns runs `lanes` threads per row      */
/* (a power of two <= 32 dividing nvec; 256 / lanes rows per CTA; the      */
/* matrix-free product also runs one warp per row, lanes = 32, at any      */
/* nvec, its default),                                                     */
/* `cols_per_lane` columns per thread per pass (1 or 4, also 2 with 32     */
/* lanes; for stored CSR also -4 or -2: that many ADJACENT columns per     */
/* lane, read as one vector, on 2..32 lanes per row, columns masked, any   */
/* width that is a multiple of 4 or 2)                                     */
/* on `grid` CTAs of 256 threads striding over the rows (0: the            */
/* default min(rows / (256 / lanes), 16 per SM); -1: one resident wave).   */
/* Every shape gives the same y bit for bit.  The solvers time the         */
/* candidate shapes the first time a width class of an operator is seen    */
/* (outside any stream capture) and use the fastest from then on; the      */
/* environment variable BH_AUTOTUNE=0 turns that off.                      */
/* ---------------------------------------------------------------------- */

typedef struct bh_spmm_shape {
    int lanes;
    int cols_per_lane;
    int64_t grid;
} bh_spmm_shape;

typedef struct bh_spmm_tuning {
    int matrix_free;       /* operator kind                                  */
    int elem_bytes;        /* 4: FP32 vectors (mixed), 8: FP64               */
    int64_t dim;           /* D                                              */
    int64_t nnz;           /* off-diagonal entries of T                      */
    int ncols;             /* width the class was timed at                   */
    bh_spmm_shape shape;   /* chosen shape at that width                     */
    float ms;              /* its time per product                           */
    float ms_default;      /* the default shape's                            */
    int candidates;        /* shapes timed                                   */
} bh_spmm_tuning;

/* Candidate shapes for nvec columns of a stored-CSR (matrix_free = 0) or
 * matrix-free operator, the default first: *count of them are written to
 * out[0..cap). */
int bh_spmm_candidates(int nvec, int matrix_free, bh_spmm_shape* out, int cap, int* count);
/* y = H x (lexicographic order, host arrays [D][nvec]) with a given shape
 * (NULL: the default), in FP64 (BH_PREC_FP64) or with FP32 vectors and
 * values (BH_PREC_MIXED: x rounded to FP32, y widened back). */
int bh_hamiltonian_apply_shape(const bh_hamiltonian* h, int precision, double J, double U,
                               double mu, int nvec, const bh_spmm_shape* shape, const double* x,
                               double* y);
/* Times the candidate shapes of products of nvec columns (batches of
 * nvec / block solves) now, on scratch vectors it allocates, and records the
 * fastest for this operator's width class (replacing an earlier entry); for
 * callers that capture their own graphs.  A width whose solver product fuses
 * the block coefficient (CSR, block 2 or 4, one pass per row) has a single
 * shape there, but is tuned here all the same for bh_hamiltonian_apply. */
int bh_spmm_autotune(const bh_hamiltonian* h, int nvec, int precision, bh_spmm_shape* chosen,
                     float* ms, float* ms_default);
/* Entries of the process-wide tuning table. */
int bh_spmm_tuning_count(int* n);
int bh_spmm_tuning_get(int i, bh_spmm_tuning* out);
/* Forgets every entry (the next products time their shapes again). */
int bh_spmm_tuning_reset(void);

#ifdef __cplusplus
}
#endif

#endif /* BH_GB300_H */
