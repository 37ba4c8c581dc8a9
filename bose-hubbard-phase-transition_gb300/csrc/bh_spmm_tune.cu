// bh_spmm_tune.cu -- launch shapes of the sparse product Y = H X and the
// table of the autotuner that picks them (bh_krylov.cuh describes the shapes).
//
// The product's best row tile (lanes per row) and vector block (columns per
// lane per pass) depend on the width of the batch, which changes at every
// restart as solves converge and are retired, and on the operator (stored
// CSR or matrix-free, entries per row, dimension).  The tuner times the
// candidate shapes on the caller's stream the first time a width class of an
// operator is seen (outside any graph capture), and every later product of
// that class, including those captured into graphs, uses the fastest.
#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>

#include "bh_internal.h"
#include "bh_krylov.cuh"

namespace bh {

int spmm_lmax(int ncols) {
    int L = 1;
    while (L < 32 && L * 2 <= ncols && ncols % (L * 2) == 0) L *= 2;
    return L;
}

// Columns per lane of the wide choice for cpl columns per lane in all.
static int wide_cw(int L, int cpl) {
    if (cpl <= 1) return 1;
    if (cpl == 2) return L == 32 ? 2 : 4;
    return 4;
}

// Lanes per row of the contiguous-column product at ncols with VW columns
// per lane (one pass when ncols <= 32 VW).
static int vec_lanes(int ncols, int vw) {
    int L = 2;
    while (L < 32 && L * vw < ncols) L *= 2;
    return L;
}

int spmm_vec_width(int ncols) { return ncols % 4 == 0 ? 4 : (ncols % 2 == 0 ? 2 : 0); }

SpmmShape spmm_resolve(const SpmmChoice& c, int ncols, bool matrix_free) {
    SpmmShape s;
    if (c.vec && !matrix_free) {
        s.VW = spmm_vec_width(ncols);
        s.L = std::max(2, vec_lanes(ncols, s.VW) >> c.dl);
        s.CW = 0;
        s.grid = c.wave ? -1 : 0;
        return s;
    }
    const int lmax = spmm_lmax(ncols);
    int L, cpl;
    if (matrix_free && c.dl == 0) {
        L = 32;  // warp per row, masked columns
        cpl = (ncols + 31) / 32;
    } else {
        const int top = matrix_free ? (lmax == 32 ? 16 : lmax) : lmax;
        L = top >> (matrix_free ? c.dl - 1 : c.dl);
        if (L < 1) L = 1;
        cpl = ncols / L;
    }
    s.L = L;
    s.CW = c.narrow ? 1 : wide_cw(L, cpl);
    s.grid = c.wave ? -1 : 0;
    return s;
}

std::vector<SpmmChoice> spmm_candidates(int ncols, bool matrix_free) {
    std::vector<SpmmChoice> out;
    std::vector<std::tuple<int, int, int64_t>> seen;
    const int lmax = spmm_lmax(ncols);
    const int top = matrix_free ? (lmax == 32 ? 16 : lmax) : lmax;
    for (int wave = 0; wave < 2; ++wave)
        for (int dl = 0; dl < 3; ++dl) {
            const int shift = matrix_free ? dl - 1 : dl;
            if (shift >= 0 && (top >> shift) < 1) continue;
            for (int narrow = 0; narrow < 2; ++narrow) {
                const SpmmChoice c{dl, narrow, wave};
                const SpmmShape s = spmm_resolve(c, ncols, matrix_free);
                const auto t = std::make_tuple(s.L, s.CW, s.grid);
                if (std::find(seen.begin(), seen.end(), t) != seen.end()) continue;
                seen.push_back(t);
                out.push_back(c);
            }
        }
    // stored CSR at even widths of at least 4: the contiguous-column product
    // on the lanes that cover the row in one pass, and half as many
    if (!matrix_free && ncols >= 4 && spmm_vec_width(ncols) > 0) {
        std::vector<std::tuple<int, int64_t>> vseen;
        for (int wave = 0; wave < 2; ++wave)
            for (int dl = 0; dl < 2; ++dl) {
                const SpmmChoice c{dl, 0, wave, 1};
                const SpmmShape s = spmm_resolve(c, ncols, false);
                const auto t = std::make_tuple(s.L, s.grid);
                if (std::find(vseen.begin(), vseen.end(), t) != vseen.end()) continue;
                vseen.push_back(t);
                out.push_back(c);
            }
    }
    return out;
}

bool spmm_shape_valid(const SpmmShape& s, int ncols, bool matrix_free) {
    if (ncols < 1 || s.grid < -1) return false;
    if (s.VW != 0) {
        if (matrix_free || !(s.VW == 2 || s.VW == 4) || ncols % s.VW != 0) return false;
        return s.L == 2 || s.L == 4 || s.L == 8 || s.L == 16 || s.L == 32;
    }
    if (!(s.L == 1 || s.L == 2 || s.L == 4 || s.L == 8 || s.L == 16 || s.L == 32)) return false;
    if (!(s.CW == 1 || s.CW == 4 || (s.CW == 2 && s.L == 32))) return false;
    if (matrix_free && s.L == 32) return true;  // warp per row, masked columns
    return ncols % s.L == 0;
}

bool spmm_fuses_vec(int ncols, int group) {
    const int vw = spmm_vec_width(ncols);
    return vw > 0 && vw % group == 0 && ncols >= 4 && vec_lanes(ncols, vw) * vw >= ncols;
}

bool spmm_fuses(bool matrix_free, bool has_dpart, int ncols, int group) {
    if (matrix_free || !has_dpart || !(group == 2 || group == 4) || ncols < 1) return false;
    if (spmm_fuses_vec(ncols, group)) return true;
    const SpmmShape d = spmm_resolve(SpmmChoice{}, ncols, false);
    return ncols / d.L <= d.CW && d.L >= group;
}

bool autotune_on() {
    static const bool on = [] {
        const char* e = std::getenv("BH_AUTOTUNE");
        return !(e && e[0] == '0' && e[1] == '\0');
    }();
    return on;
}

bool TuneKey::operator<(const TuneKey& o) const {
    return std::tie(mf, elem, lmax, cls, aux, D, nnz) < std::tie(o.mf, o.elem, o.lmax, o.cls, o.aux, o.D, o.nnz);
}

namespace {
std::mutex g_tune_mu;
std::map<TuneKey, TuneEntry> g_tune;
}  // namespace

bool tune_lookup(const TuneKey& k, SpmmChoice* c) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const auto it = g_tune.find(k);
    if (it == g_tune.end()) return false;
    if (c) *c = it->second.choice;
    return true;
}

void tune_store(const TuneKey& k, const TuneEntry& e) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[k] = e;
}

std::vector<std::pair<TuneKey, TuneEntry>> tune_table() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return std::vector<std::pair<TuneKey, TuneEntry>>(g_tune.begin(), g_tune.end());
}

void tune_reset() {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
}

template <class A, class B>
__global__ void k_cast(int64_t n, const A* __restrict__ in, B* __restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (B)in[i];
}

template <class A, class B>
static void cast_launch(int64_t n, const A* in, B* out, cudaStream_t st) {
    if (n <= 0) return;
    const int64_t g = std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8);
    k_cast<A, B><<<(unsigned)std::max<int64_t>(1, g), 256, 0, st>>>(n, in, out);
    BH_CUDA(cudaGetLastError());
}

void cast_f64_f32(int64_t n, const double* in, float* out, cudaStream_t st) { cast_launch(n, in, out, st); }
void cast_f32_f64(int64_t n, const float* in, double* out, cudaStream_t st) { cast_launch(n, in, out, st); }

}  // namespace bh
