"""Sparse products of one sector's stored-CSR Hamiltonian, the ncu driver of
the product kernels.

    python bose-hubbard-phase-transition_gb300/profile_spmm.py [m] [ncols]

The 1D periodic chain with n = m bosons (m = 13: D = 5 200 300, 70.3 M stored
entries), a random D x ncols block in FP32 (mixed precision), J = 0.1, U = 1,
mu = 0: two products with the default launch shape (k_spmm), then two with
the contiguous-column shape (k_spmm_v, four adjacent columns per lane on the
fewest lanes that cover the row in one pass).  Prints D, the stored entries
and whether both shapes gave the same result bit for bit.
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main(argv):
    import __graft_entry__ as g

    m = int(argv[1]) if len(argv) > 1 else 13
    ncol = int(argv[2]) if len(argv) > 2 else 16
    pkg = g.load_package()
    pkg.load()
    nb = pkg.Neighbours(m)
    nb.chain_neighbours()
    h = pkg.Hamiltonian(pkg.Basis(m, m), nb.getNeighbours())
    x = np.random.RandomState(0).randn(h.D, ncol)
    vl = 2
    while vl < 32 and vl * 4 < ncol:
        vl *= 2
    ys = [h.apply_shape(x, 0.1, 1.0, 0.0, shape, precision=pkg.PREC_MIXED)
          for shape in (None, None, (vl, -4, 0), (vl, -4, 0))]
    print("D", h.D, "stored entries", h.nnz_offdiag, "contiguous-column product equals the default:",
          bool(np.array_equal(ys[0], ys[2])))


if __name__ == "__main__":
    main(sys.argv)
