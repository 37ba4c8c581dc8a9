// bh_lattice.cpp -- neighbour lists of the lattices the reference supports.
//
// Replaces Neighbours::chain_neighbours, square_neighbours and
// cube_neighbours (src/neighbours.cpp:21-120).  The 1D list reproduces the
// reference entry for entry (including the order of the periodic entries).
// The 2D and 3D lists are the ones the reference's loops describe; the
// reference itself fills a local vector that shadows the member and so
// returns empty lists (neighbours.cpp:45, 82).
#include <cmath>
#include <string>
#include <vector>

#include "bh_internal.h"

namespace bh {

using Lists = std::vector<std::vector<int32_t>>;

Lists chain_lists(int m, bool closed) {
    BH_REQUIRE(m >= 1, "the number of sites must be positive");
    Lists nb(m);
    for (int i = 0; i < m; ++i) {
        if (i > 0) nb[i].push_back(i - 1);
        if (i < m - 1) nb[i].push_back(i + 1);
    }
    if (closed) {
        nb[0].push_back(m - 1);
        nb[m - 1].push_back(0);
    }
    return nb;
}

Lists square_lists(int m, bool closed) {
    const int side = (int)std::sqrt((double)m);
    if (side * side != m) throw Error(BH_ERR_ARG, "The number of sites (m) must be a perfect square.");
    Lists nb(m);
    for (int i = 0; i < side; ++i)
        for (int j = 0; j < side; ++j) {
            const int idx = i * side + j;
            if (j > 0) nb[idx].push_back(idx - 1);
            else if (closed) nb[idx].push_back(idx + side - 1);
            if (j < side - 1) nb[idx].push_back(idx + 1);
            else if (closed) nb[idx].push_back(idx - side + 1);
            if (i > 0) nb[idx].push_back(idx - side);
            else if (closed) nb[idx].push_back(idx + (side - 1) * side);
            if (i < side - 1) nb[idx].push_back(idx + side);
            else if (closed) nb[idx].push_back(idx - (side - 1) * side);
        }
    return nb;
}

Lists cube_lists(int m, bool closed) {
    const int side = (int)std::cbrt((double)m);
    int s2 = side;
    // guard against cbrt rounding just below an integer
    if ((s2 + 1) * (s2 + 1) * (s2 + 1) == m) ++s2;
    if (s2 * s2 * s2 != m) throw Error(BH_ERR_ARG, "The number of sites (m) must be a perfect cube.");
    const int sd = s2, sq = sd * sd;
    Lists nb(m);
    for (int i = 0; i < sd; ++i)
        for (int j = 0; j < sd; ++j)
            for (int k = 0; k < sd; ++k) {
                const int idx = i * sq + j * sd + k;
                if (k > 0) nb[idx].push_back(idx - 1);
                else if (closed) nb[idx].push_back(idx + sd - 1);
                if (k < sd - 1) nb[idx].push_back(idx + 1);
                else if (closed) nb[idx].push_back(idx - sd + 1);
                if (j > 0) nb[idx].push_back(idx - sd);
                else if (closed) nb[idx].push_back(idx + (sd - 1) * sd);
                if (j < sd - 1) nb[idx].push_back(idx + sd);
                else if (closed) nb[idx].push_back(idx - (sd - 1) * sd);
                if (i > 0) nb[idx].push_back(idx - sq);
                else if (closed) nb[idx].push_back(idx + (sd - 1) * sq);
                if (i < sd - 1) nb[idx].push_back(idx + sq);
                else if (closed) nb[idx].push_back(idx - (sd - 1) * sq);
            }
    return nb;
}

void flatten(const Lists& nb, int32_t* off, int32_t* out, int cap, int* count) {
    int c = 0;
    off[0] = 0;
    for (size_t i = 0; i < nb.size(); ++i) {
        for (int32_t j : nb[i]) {
            if (out && c < cap) out[c] = j;
            ++c;
        }
        off[i + 1] = c;
    }
    if (count) *count = c;
    if (out && c > cap) throw Error(BH_ERR_ARG, "neighbour buffer too small: need " + std::to_string(c));
}

}  // namespace bh
