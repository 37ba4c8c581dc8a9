"""GPU: launch shapes of the sparse product and the autotuner that picks them.

- every candidate shape (and explicit grids) gives the default shape's y bit
  for bit, for the stored-CSR and matrix-free operators, FP64 and FP32, at
  widths that exercise one and several passes per lane;
- an explicit tuning run records an entry and leaves the products' values
  unchanged;
- batched solves with automatic tuning give the same eigenvalues, bit for
  bit, and the same restart count as with tuning off (BH_AUTOTUNE=0 in a
  child process): the tuner changes which thread computes each entry of
  H X, never the arithmetic.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, chain_lists

pytestmark = pytest.mark.gpu

WIDTHS = [1, 2, 6, 12, 28, 60, 64, 128]


def square_lists(pkg, m):
    nb = pkg.Neighbours(m)
    nb.square_neighbours(True)
    return nb.getNeighbours()


def operators(pkg):
    yield "csr", pkg.Hamiltonian(pkg.Basis(8, 6), chain_lists(8))                      # D = 1716
    yield "mf-chain", pkg.Hamiltonian(pkg.Basis(8, 6), chain_lists(8), matrix_free=True)
    yield "mf-square", pkg.Hamiltonian(pkg.Basis(16, 4), square_lists(pkg, 16), matrix_free=True)  # D = 3876


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_every_shape_gives_the_default_product_bit_for_bit(pkg, prec):
    p = pkg.PREC_FP64 if prec == "fp64" else pkg.PREC_MIXED
    for name, h in operators(pkg):
        for nvec in WIDTHS:
            x = np.random.RandomState(nvec).uniform(-1, 1, (h.D, nvec))
            y0 = h.apply_shape(x, 0.11, 1.0, 0.3, None, precision=p)
            if p == pkg.PREC_FP64:
                # the allocating lexicographic apply (default or tuned shape)
                ya = h.apply(x, 0.11, 1.0, 0.3, order=pkg.ORDER_LEX)
                assert np.array_equal(ya, y0), (name, nvec)
            shapes = pkg.spmm_candidates(nvec, h.matrix_free)
            L0, c0, _ = shapes[0]
            shapes += [(L0, c0, 1), (L0, c0, 7), (1, 1, 3)]
            if h.matrix_free:
                # the warp-per-row kernel at every column width, one and several passes
                shapes += [(32, 1, 0), (32, 2, 5), (32, 4, -1)]
            else:
                # the contiguous-column product: several passes per lane, odd grids
                if nvec % 2 == 0:
                    shapes += [(2, -2, 0), (32, -2, -1), (4, -2, 5)]
                if nvec % 4 == 0:
                    shapes += [(2, -4, 3), (8, -4, 0)]
            for s in shapes:
                y = h.apply_shape(x, 0.11, 1.0, 0.3, s, precision=p)
                assert np.array_equal(y, y0), (name, nvec, s)


def test_shape_arguments_are_checked(pkg):
    h = pkg.Hamiltonian(pkg.Basis(4, 3), chain_lists(4))
    x = np.ones((h.D, 6))
    for bad in [(4, 4, 0), (3, 1, 0), (2, 2, 0), (2, 4, -2), (64, 1, 0), (32, -4, 0), (3, -2, 0),
                (64, -2, 0), (4, -3, 0)]:
        with pytest.raises(ValueError, match="launch shape"):
            h.apply_shape(x, 0.1, 1.0, 0.0, bad)


def test_explicit_autotune_records_an_entry(pkg):
    pkg.spmm_tuning_reset()
    h = pkg.Hamiltonian(pkg.Basis(9, 7), chain_lists(9))  # D = 6435
    x = np.random.RandomState(3).uniform(-1, 1, (h.D, 46))
    y0 = h.apply_shape(x, 0.2, 1.0, 0.1, None)
    for prec in (pkg.PREC_MIXED, pkg.PREC_FP64):
        r = h.autotune(46, precision=prec)
        assert r["shape"] in pkg.spmm_candidates(46, False)
        assert 0.0 < r["ms"] <= r["ms_default"]
    tab = pkg.spmm_tuning_table()
    assert {e["elem_bytes"] for e in tab if e["dim"] == h.D} == {4, 8}
    for e in tab:
        assert e["candidates"] >= 1 and e["shape"] in pkg.spmm_candidates(e["ncols"], e["matrix_free"])
    # the FP64 apply now takes the tuned shape: same values
    assert np.array_equal(h.apply(x, 0.2, 1.0, 0.1, order=pkg.ORDER_LEX), y0)


_CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import __graft_entry__ as g
bh = g.load_package(); bh.load()
out = {}
nb = bh.Neighbours(9); nb.chain_neighbours()
h = bh.Hamiltonian(bh.Basis(9, 7), nb.getNeighbours())
J = 0.3 * (np.arange(23) + 1) / 23      # 23 solves x block 2: odd widths, unfused products
for tag, prec in (("mixed", bh.PREC_MIXED), ("fp64", bh.PREC_FP64)):
    ev, _, nc, info = h.eigsh_batch(J, 1.0, 0.0, nev=6, precision=prec)
    out[tag] = [float.hex(float(v)) for v in ev.ravel()] + [info.restarts]
nb = bh.Neighbours(16); nb.square_neighbours()
hf = bh.Hamiltonian(bh.Basis(16, 4), nb.getNeighbours(), matrix_free=True)
ev, _, nc, info = hf.eigsh_batch(np.linspace(0.02, 0.1, 7), 1.0, 0.4, nev=4, block=4,
                                 precision=bh.PREC_MIXED)
out["mf"] = [float.hex(float(v)) for v in ev.ravel()] + [info.restarts]
out["entries"] = len(bh.spmm_tuning_table())
print(json.dumps(out))
"""


def test_tuned_solves_match_untuned_bit_for_bit():
    out = {}
    for tag, extra in (("tuned", {}), ("off", {"BH_AUTOTUNE": "0"})):
        env = dict(os.environ, **extra)
        r = subprocess.run([sys.executable, "-c", _CHILD, ROOT], capture_output=True, text=True,
                           env=env, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        out[tag] = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["tuned"]["entries"] > 0
    assert out["off"]["entries"] == 0
    for k in ("mixed", "fp64", "mf"):
        assert out["tuned"][k] == out["off"][k], k
