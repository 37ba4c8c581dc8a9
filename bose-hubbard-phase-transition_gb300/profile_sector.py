"""One batched eigensolve of one sector, with the per-kernel timing table.

    python bose-hubbard-phase-transition_gb300/profile_sector.py [m] [n] [nJ] [prec] [ncv] [block] [warm]
                                                                 [lattice] [operator]

Defaults: the 1D periodic chain m=10, n=10 (D = 92 378), 64 J values
J_b = 0.3 (b + 1) / 64, U = 1, mu = 0, lowest 10 eigenvalues, mixed precision,
stored CSR.  lattice "square" takes the periodic square lattice of m sites
(m a perfect square) instead of the chain; operator "mf" the matrix-free
Hamiltonian (rows regenerated from packed occupations in every product).
One untimed warm-up solve with 8 J values comes first (warm = 0 leaves it
out, so that an ncu launch filter counts the measured solve's launches only).  The table lists, per
kernel, its launches, the summed CUDA-event duration, its share and the
algorithmic bytes / duration.  This is the small case the ncu captures of
the solver kernels are taken on.
"""
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main(argv):
    import __graft_entry__ as g

    m = int(argv[1]) if len(argv) > 1 else 10
    n = int(argv[2]) if len(argv) > 2 else 10
    nj = int(argv[3]) if len(argv) > 3 else 64
    pkg = g.load_package()
    pkg.load()
    prec = {"mixed": pkg.PREC_MIXED, "fp64": pkg.PREC_FP64}[argv[4] if len(argv) > 4 else "mixed"]
    ncv = int(argv[5]) if len(argv) > 5 else 0
    block = int(argv[6]) if len(argv) > 6 else 0
    warm = int(argv[7]) if len(argv) > 7 else 1
    lattice = argv[8] if len(argv) > 8 else "chain"
    mf = (argv[9] if len(argv) > 9 else "csr") == "mf"
    nb = pkg.Neighbours(m)
    {"chain": nb.chain_neighbours, "square": nb.square_neighbours}[lattice]()
    h = pkg.Hamiltonian(pkg.Basis(m, n), nb.getNeighbours(), matrix_free=mf)
    js = 0.3 * (np.arange(nj) + 1) / nj
    if warm:
        h.eigsh_batch(js[:8], 1.0, 0.0, nev=10, precision=prec, ncv=ncv, block=block)
    pkg.profile_reset()
    pkg.profile_enable(True)
    t0 = time.time()
    ev, rs, nc, info = h.eigsh_batch(js, 1.0, 0.0, nev=10, precision=prec, ncv=ncv, block=block)
    wall = time.time() - t0
    pkg.profile_enable(False)
    prof = pkg.profile_read()
    tot = sum(v["ms"] for v in prof.values())
    print(f"{lattice} m={m} n={n} {'matrix-free' if mf else 'CSR'} D={h.D} solves={nj} wall {wall:.3f} s, kernel sum {tot / 1e3:.3f} s, "
          f"restarts {info.restarts}, matvecs {info.matvecs}, launches {info.launches}, min nconv {nc.min()}")
    print(f"{'kernel':24s} {'launches':>8s} {'ms':>10s} {'share':>7s} {'GB/s':>9s}")
    for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"]):
        print(f"{k:24s} {v['launches']:8d} {v['ms']:10.2f} {100 * v['ms'] / tot:6.2f}% "
              f"{v['bytes'] / (v['ms'] * 1e6):9.1f}")


if __name__ == "__main__":
    main(sys.argv)
