"""GPU: the solver's alternative code paths give the same spectrum.

- block sizes 1, 2, 4 (per-solve vector kernels for P = 1, 2, 4) and 8 (the
  generic kernels), FP64 and mixed precision, against dense eigvalsh;
- odd batch widths (the SpMM cannot fuse the local coefficient there, and
  the row mapping changes), against the same points solved alone;
- the restart cycles replayed from captured CUDA graphs against direct
  launches (BH_NO_GRAPHS=1 in a child process): the same kernels in the same
  order, so the eigenvalues agree bit for bit.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, chain_lists

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("block", [1, 2, 4, 8])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_block_sizes_match_dense(pkg, block, prec):
    m, n = 7, 6  # D = 924
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    J = np.array([0.04, 0.13, 0.29])
    p = pkg.PREC_FP64 if prec == "fp64" else pkg.PREC_MIXED
    ev, _, nc, _ = h.eigsh_batch(J, 1.0, 0.2, nev=6, block=block, precision=p)
    assert nc.min() >= 6
    for k, j in enumerate(J):
        w = np.linalg.eigvalsh(h.csr(j, 1.0, 0.2).toarray())[:6]
        tol = 1e-10 if prec == "fp64" else 1e-8
        np.testing.assert_allclose(ev[k], w, rtol=tol, atol=1e-10)


def test_odd_batch_width_matches_single_solves(pkg):
    m, n = 8, 7  # D = 3432
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    J = np.linspace(0.03, 0.28, 7)  # 7 solves x block 2 = 14 columns
    ev, _, nc, _ = h.eigsh_batch(J, 1.0, 0.1, nev=5, precision=pkg.PREC_FP64)
    assert nc.min() >= 5
    for k in (0, 3, 6):
        e1, _, _, _ = h.eigsh(J[k], 1.0, 0.1, nev=5)
        np.testing.assert_allclose(ev[k], e1, rtol=1e-10, atol=1e-12)


_CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import __graft_entry__ as g
bh = g.load_package(); bh.load()
nb = bh.Neighbours(9); nb.chain_neighbours()
h = bh.Hamiltonian(bh.Basis(9, 7), nb.getNeighbours())
J = 0.3 * (np.arange(24) + 1) / 24
ev, _, nc, info = h.eigsh_batch(J, 1.0, 0.0, nev=8, precision=bh.PREC_MIXED)
print(json.dumps({"ev": [float.hex(float(v)) for v in ev.ravel()], "restarts": info.restarts}))
"""


def test_graph_replay_matches_direct_launches():
    out = {}
    for tag, extra in (("graphs", {}), ("direct", {"BH_NO_GRAPHS": "1"})):
        env = dict(os.environ, **extra)
        r = subprocess.run([sys.executable, "-c", _CHILD, ROOT], capture_output=True, text=True,
                           env=env, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        out[tag] = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["graphs"]["restarts"] == out["direct"]["restarts"]
    assert out["graphs"]["ev"] == out["direct"]["ev"]
