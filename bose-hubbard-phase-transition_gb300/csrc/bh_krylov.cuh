// bh_krylov.cuh -- block thick-restart Lanczos on the device (declarations).
#pragma once

#include <utility>

#include "bh_internal.h"

namespace bh {

// Sparse operator  y_t = J_s (T x)_t + (U_s vd + shift_s) x_t  for column t of
// solve s = t / group.  vd may be null (plain CSR of a full matrix, U = 0).
template <class T>
struct OpView {
    const int64_t* rp = nullptr;
    const int32_t* ci = nullptr;
    const T* tv = nullptr;
    const T* vd = nullptr;
    int64_t D = 0;
    int64_t rp_nnz = 0;  // stored entries (for the algorithmic byte count)
    // matrix-free operator (occ != nullptr): the rows of T and V are
    // regenerated in every product from the packed occupation strings
    const uint64_t* occ = nullptr;   // D strings, `bits` bits per site, site 0 in the low bits
    const uint32_t* rt = nullptr;    // rank table (m-1) x (n+1)
    const uint8_t* bonds = nullptr;  // directed bonds: bonds[2k] = i, bonds[2k+1] = j
    const T* sq = nullptr;           // sq[a] = -sqrt(a), a <= n (n + 1)
    int m = 0, n = 0, bits = 0, nbonds = 0;
};

// Lets kern take more than 48 KB of dynamic shared memory.  The attribute is
// per function and process-wide, and solves of other sectors set it from
// other host threads: it is therefore only ever set to the device's opt-in
// maximum (never to a launch's own size, which another thread could lower
// between this thread's setting and its launch).
template <class K>
inline void allow_large_smem(K kern, size_t smem) {
    if (smem <= 48 * 1024) return;
    int dev = 0, mx = 0;
    BH_CUDA(cudaGetDevice(&dev));
    BH_CUDA(cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    BH_REQUIRE(smem <= (size_t)mx, "shared memory of a launch exceeds the device limit");
    BH_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
}

// CTAs of kern resident on one SM at this block size and dynamic shared memory.
template <class K>
inline int resident_ctas(K kern, int threads, size_t smem) {
    int n = 0;
    BH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, threads, smem));
    return n;
}

// Operator views of a built Hamiltonian (CSR or matrix-free).
template <class T>
inline OpView<T> op_view(const bh_hamiltonian* h) {
    OpView<T> o;
    o.D = h->D;
    o.rp_nnz = h->nnz;
    if (h->matrix_free) {
        o.occ = h->d_occ.p;
        o.rt = h->basis->d_rt.p;
        o.bonds = h->d_bonds.p;
        if constexpr (sizeof(T) == 8) o.sq = reinterpret_cast<const T*>(h->d_sq64.p);
        else o.sq = reinterpret_cast<const T*>(h->d_sq32.p);
        o.m = h->m;
        o.n = h->n;
        o.bits = h->occ_bits;
        o.nbonds = h->nbonds;
        return o;
    }
    o.rp = h->d_rp.p;
    o.ci = h->d_ci.p;
    if constexpr (sizeof(T) == 8) {
        o.tv = reinterpret_cast<const T*>(h->d_tv64.p);
        o.vd = reinterpret_cast<const T*>(h->d_vd64.p);
    } else {
        o.tv = reinterpret_cast<const T*>(h->d_tv32.p);
        o.vd = reinterpret_cast<const T*>(h->d_vd32.p);
    }
    return o;
}

struct SolveRequest {
    int S = 1;                 // solves in the batch (share the operator pattern)
    int nev = 10;
    int p = 2;                 // block size
    int kmax = 0;              // basis size (multiple of p)
    int max_restarts = 1000;
    double tol = 1e-10;
    int precision = BH_PREC_FP64;
    uint64_t seed = 0;
    const int32_t* d_perm = nullptr;  // start-vector index map (row -> reference index)
    std::vector<double> J, U, shift;  // per solve
    bool want_vectors = false;
};

struct SolveResult {
    std::vector<double> evals;   // S x nev, ascending
    std::vector<double> resid;   // S x nev, relative residual norms
    std::vector<int> nconv;      // S
    std::vector<int> conv_at;    // S: restart count at which the solve converged (-1: never)
    std::vector<double> scale;   // S: spectral radius estimate (largest |Ritz value|)
    std::vector<double> vecs;    // S x nev x D (lexicographic/operator order), if requested
    std::vector<int> status;     // S: BH_OK, or BH_ERR_BREAKDOWN where the solve's Krylov
                                 // space held fewer than nev directions (an invariant start
                                 // block), or BH_ERR_NOCONV where its Ritz vectors were not
                                 // independent in the final Rayleigh-Ritz
    std::vector<int> live;       // S: Krylov directions the solve held at its last restart
    int restarts = 0;
    int64_t matvecs = 0;
    int64_t launches = 0;        // kernels launched by the solve
    bool breakdown = false;
};

// ---------------------------------------------------------------------------
// Launch shape of the sparse product and its autotuner (bh_spmm_tune.cu).
//
// The product runs L lanes per row over the columns (L a power of two <= 32
// dividing ncols: the row tile is 256 / L rows per CTA), CW columns per lane
// per pass (the vector block: 1 or 4, also 2 when L = 32; further passes
// cover the rest of the row's columns), on `grid` CTAs of 256 threads that
// stride over the rows (0: min(rows / (256 / L), 16 per SM); -1: one
// resident wave; > 0: that many).  Every shape gives the same Y bit for bit:
// each column's sum runs over the row's entries (or bonds) in storage order
// with the same operations, only the thread that computes it changes.  The
// one exception is the fused CSR product that also yields the partials of
// V_j^T H V_j, whose CTA partial sums depend on the grid: it keeps its one
// shape and is never tuned.
// ---------------------------------------------------------------------------
struct SpmmShape {
    int L = 0, CW = 0;
    int64_t grid = 0;
    int VW = 0;  // > 0: L lanes per row, each VW adjacent columns per pass (k_spmm_v)
};

// The matrix-free product also has a warp-per-row kernel (L = 32 at any
// ncols, columns t = lane + 32 u masked by t < ncols), its default shape.
//
// A shape relative to the column count, kept by the tuner for a class of
// widths: L = lmax(ncols) >> dl (matrix-free: dl = 0 is the warp kernel,
// dl >= 1 the per-lane kernels from lmax, or 16 when lmax = 32, down), CW = 1
// if narrow (else the widest that covers the lane's columns in few passes),
// grid default or one wave.
// vec = 1 (stored CSR, even ncols): the contiguous-column product k_spmm_v,
// VW = 4 adjacent columns per lane (2 when ncols is not a multiple of 4) on
// L = (the power of two >= ncols / VW, at most 32) >> dl lanes per row.
struct SpmmChoice {
    int dl = 0, narrow = 0, wave = 0, vec = 0;
};

// Largest power of two <= 32 dividing ncols (the default lanes per row).
int spmm_lmax(int ncols);
// Concrete shape of a relative choice at ncols ({0, 0, 0} is the default).
SpmmShape spmm_resolve(const SpmmChoice& c, int ncols, bool matrix_free = false);
// Shapes the tuner times at ncols, the default first, without duplicates.
std::vector<SpmmChoice> spmm_candidates(int ncols, bool matrix_free = false);
// Whether shape s can run a product of ncols columns.
bool spmm_shape_valid(const SpmmShape& s, int ncols, bool matrix_free = false);
// Whether the default product fuses the local coefficient (CSR with dpart,
// block 2 or 4, one pass over the row's columns).
bool spmm_fuses(bool matrix_free, bool has_dpart, int ncols, int group);
// Columns per lane of the contiguous-column product at ncols (4, 2, or 0 when
// ncols is odd), and whether the fused product uses it (one pass, whole
// solves in every lane's columns).
int spmm_vec_width(int ncols);
bool spmm_fuses_vec(int ncols, int group);
// Automatic tuning at first use (off with BH_AUTOTUNE=0).
bool autotune_on();

// One entry of the tuning table: an operator (kind, element size, D, entries)
// and a class of widths (lmax, passes), the choice and its timings.
struct TuneKey {
    int mf = 0, elem = 0, lmax = 0, cls = 0, aux = 0;
    int64_t D = 0, nnz = 0;
    bool operator<(const TuneKey& o) const;
};
struct TuneEntry {
    SpmmChoice choice;
    int ncols = 0;         // width it was timed at
    SpmmShape shape;       // the choice resolved at that width
    float ms = 0.f, ms_default = 0.f;
    int candidates = 0;    // shapes timed
};
template <class T>
TuneKey tune_key(const OpView<T>& op, int ncols) {
    TuneKey k;
    k.mf = op.occ ? 1 : 0;
    k.elem = (int)sizeof(T);
    k.lmax = spmm_lmax(ncols);
    auto bucket = [](int c) { return c <= 1 ? 0 : c == 2 ? 1 : c <= 4 ? 2 : c <= 8 ? 3 : c <= 16 ? 4 : 5; };
    k.cls = bucket(ncols / k.lmax) + (op.occ ? 8 * bucket((ncols + 31) / 32) : 0);
    k.aux = op.occ ? op.nbonds * 64 + op.m : 0;
    k.D = op.D;
    k.nnz = op.rp_nnz;
    return k;
}
bool tune_lookup(const TuneKey& k, SpmmChoice* c);
void tune_store(const TuneKey& k, const TuneEntry& e);
std::vector<std::pair<TuneKey, TuneEntry>> tune_table();
void tune_reset();

// Y = H X for ncols columns of T (CSR operator: MF = false; matrix-free:
// MF = true), solve of column t = t / group, prm[3 s..] = (J, U, shift);
// returns the algorithmic bytes.  Instantiated for float and double in
// bh_spmm_{csr,mf}_{f32,f64}.cu.
// With dpart (CSR operators, block size group = 2 or 4, at most one pass over
// the row's columns) the product also writes the partial sums of X_s^T Y_s,
// dpart[(chunk group + q) ncols + t] for chunk < *dparts; *dparts = 0 when
// the product could not fuse them.  A product that does not fuse takes the
// tuning table's shape for its operator and width class when `tuned` and
// the table has one, else the default shape.
template <class T, bool MF>
double launch_spmm_kind(const OpView<T>& op, int ncols, int group, const double* prm, const T* X,
                        T* Y, cudaStream_t st, double* dpart, int* dparts, bool tuned);

// The product (never fused) with a given shape; BH_ERR_ARG if it cannot run.
template <class T, bool MF>
double launch_spmm_shape_kind(const OpView<T>& op, int ncols, int group, const double* prm,
                              const T* X, T* Y, cudaStream_t st, const SpmmShape& s);

// Times the candidate shapes of this operator's width class on the caller's
// stream and records the fastest, unless the table has the class already
// (force: time again), the default product fuses (has_dpart), tuning is off
// (force overrides), or the stream is capturing.  Y is overwritten with H X
// (the same values as the product itself); X and Y must not overlap.
// Returns the kernels launched; *out (if given) receives the entry.
template <class T, bool MF>
int tune_spmm_kind(const OpView<T>& op, int ncols, int group, const double* prm, const T* X, T* Y,
                   cudaStream_t st, bool has_dpart, bool force, TuneEntry* out);

template <class T>
inline double launch_spmm(const OpView<T>& op, int ncols, int group, const double* prm, const T* X,
                          T* Y, cudaStream_t st, double* dpart = nullptr, int* dparts = nullptr,
                          bool tuned = true) {
    return op.occ ? launch_spmm_kind<T, true>(op, ncols, group, prm, X, Y, st, dpart, dparts, tuned)
                  : launch_spmm_kind<T, false>(op, ncols, group, prm, X, Y, st, dpart, dparts, tuned);
}

template <class T>
inline int tune_spmm(const OpView<T>& op, int ncols, int group, const double* prm, const T* X, T* Y,
                     cudaStream_t st, bool has_dpart, bool force = false, TuneEntry* out = nullptr) {
    return op.occ ? tune_spmm_kind<T, true>(op, ncols, group, prm, X, Y, st, has_dpart, force, out)
                  : tune_spmm_kind<T, false>(op, ncols, group, prm, X, Y, st, has_dpart, force, out);
}

template <class T>
inline double launch_spmm_shape(const OpView<T>& op, int ncols, int group, const double* prm,
                                const T* X, T* Y, cudaStream_t st, const SpmmShape& s) {
    return op.occ ? launch_spmm_shape_kind<T, true>(op, ncols, group, prm, X, Y, st, s)
                  : launch_spmm_shape_kind<T, false>(op, ncols, group, prm, X, Y, st, s);
}

// out[i] = in[i] converted, i < n (FP64 <-> FP32 vectors of the shape-forced product).
void cast_f64_f32(int64_t n, const double* in, float* out, cudaStream_t st);
void cast_f32_f64(int64_t n, const float* in, double* out, cudaStream_t st);

// Y = H X (FP64) for ncols columns, solve of column t = t / group, prm[3 s..] = (J, U, shift).
void apply_operator(const OpView<double>& op, int ncols, int group, const double* d_prm,
                    const double* d_X, double* d_Y, cudaStream_t st);

// The same product with no profiling events and no allocation.
void apply_operator_raw(const OpView<double>& op, int ncols, int group, const double* d_prm,
                        const double* d_X, double* d_Y, cudaStream_t st);

// op64 must be set; op32 must be set for BH_PREC_MIXED (same pattern).
// The thick-restart rotation of an FP32 basis on the tensor cores
// (bh_rotate_tc.cu), same arguments and result as the SIMT rotation; false
// (nothing launched) where its shapes do not fit (more than 256 outputs, block
// size above 4, shared memory); *d_status (device) is set if a bounded wait
// of a CTA ran out.
bool rotate_tc(int64_t D, int Sproc, int ld_in, int p, int kc, int nout, int64_t bstride, const float* V,
               const float* Yg, const int* in_idx, const int* out_idx, float* Vout, int64_t ostride,
               int ld_out, int single, int* d_status, cudaStream_t st);
// The same rotation streamed by TMA with warp-specialised TF32 tensor-core
// products (bh_rotate_tma.cu), for a batch whose solves all continue (input
// and output solve indices the identity, not the single-array layout).
// Returns false, launching nothing, when the shapes or alignments do not fit.
bool rotate_tma(int64_t D, int Sproc, int ld_in, int p, int kc, int nout, int64_t bstride, const float* V,
                const float* Yg, float* Vout, int64_t ostride, int ld_out, int* d_status, cudaStream_t st,
                bool a_in_tmem);

// Op::FOLM_diag: k Lanczos steps of the FP64 operator from v0 (unit norm, host)
// with full re-orthogonalisation; T (k x k, host) and V (D x k column-major,
// host) receive the tridiagonal matrix and the Krylov vectors.  Returns the
// number of vectors (fewer than k after a breakdown, beta < 1e-6).
int folm_diag(const OpView<double>& op, int k, const double* v0, double* T, double* V, cudaStream_t st);

SolveResult block_lanczos(const OpView<double>& op64, const OpView<float>& op32,
                          const SolveRequest& rq, cudaStream_t st);

}  // namespace bh
