// bh_device.cuh -- device helpers for combinadic ranking of Fock states.
//
// Lexicographic index r of a state (the order of the reference's
// init_lexicographic, src/hamiltonian.cpp:60-85, which starts at (n,0,...,0)
// and decrements the rightmost movable site) is
//     r = sum_{i=0}^{m-2} RT[i][s_i],   s_i = n_{i+1} + ... + n_{m-1},
//     RT[i][s] = C(s + m - i - 2, m - i - 1)
// (RT[i][s] counts the states sharing the prefix n_0..n_{i-1} whose n_i is
// larger).  RT[i][.] is strictly increasing for s >= 0 with RT[i][0] = 0, so
// unranking walks the sites and picks the largest admissible suffix sum.
#pragma once
#include <stdint.h>

namespace bh {

// rt: (m-1) x (n+1) table, row-major
__device__ __forceinline__ void unrank_state(uint32_t r, int m, int n, const uint32_t* rt,
                                             uint8_t* occ) {
    int sprev = n;
    for (int i = 0; i + 1 < m; ++i) {
        const uint32_t* row = rt + i * (n + 1);
        int s = sprev;
        while (row[s] > r) --s;
        occ[i] = (uint8_t)(sprev - s);
        r -= row[s];
        sprev = s;
    }
    occ[m - 1] = (uint8_t)sprev;
}

__device__ __forceinline__ uint32_t rank_state(const uint8_t* occ, int m, int n,
                                               const uint32_t* rt) {
    uint32_t r = 0;
    int suffix = 0;
    for (int i = m - 2; i >= 0; --i) {
        suffix += occ[i + 1];
        r += rt[i * (n + 1) + suffix];
    }
    return r;
}

}  // namespace bh
