"""GPU: the matrix-free Hamiltonian (rows regenerated from packed occupation
strings in every product) against the oracle's stored T and against the
stored-CSR operator of the same sector."""
import numpy as np
import pytest

from conftest import chain_lists, oracle_H

pytestmark = pytest.mark.gpu


def square_lists(pkg, m):
    nb = pkg.Neighbours(m)
    nb.square_neighbours(True)
    return nb.getNeighbours()


CASES = [("chain", 8, 6), ("chain", 2, 3), ("square", 9, 5), ("square", 16, 4), ("square", 4, 3)]


def _lists(pkg, kind, m):
    return chain_lists(m) if kind == "chain" else square_lists(pkg, m)


@pytest.mark.parametrize("kind,m,n", CASES)
def test_matrix_free_apply_matches_oracle(pkg, orc, kind, m, n):
    lists = _lists(pkg, kind, m)
    b = pkg.Basis(m, n)
    hf = pkg.Hamiltonian(b, lists, matrix_free=True)
    assert hf.matrix_free
    _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, lists)
    assert hf.nnz_offdiag == rp[-1]  # entries of the equivalent stored T
    x = np.random.RandomState(m * 100 + n).randn(b.D, 3)
    J, U, mu = 0.13, 1.1, 0.35
    y = hf.apply(x, J, U, mu)
    for k in range(3):
        yo = orc.spmv(rp, ci, tv, vd, n, J, U, mu, np.ascontiguousarray(x[:, k]))
        np.testing.assert_allclose(y[:, k], yo, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("kind,m,n", CASES[:4])
def test_matrix_free_apply_matches_stored_csr(pkg, kind, m, n):
    lists = _lists(pkg, kind, m)
    b = pkg.Basis(m, n)
    hc = pkg.Hamiltonian(b, lists)
    hf = pkg.Hamiltonian(b, lists, matrix_free=True)
    x = np.random.RandomState(7).randn(b.D, 4)
    for order in (pkg.ORDER_REFERENCE, pkg.ORDER_LEX):
        yc = hc.apply(x, 0.21, 0.9, 0.1, order=order)
        yf = hf.apply(x, 0.21, 0.9, 0.1, order=order)
        # same terms, summed in bond order instead of column order
        np.testing.assert_allclose(yf, yc, rtol=1e-14, atol=1e-13)
    # the stored form assembled on request is the same matrix
    Hc = hc.csr(0.3, 1.0, 0.2)
    Hf = hf.csr(0.3, 1.0, 0.2)
    assert np.array_equal(Hc.indptr, Hf.indptr) and np.array_equal(Hc.indices, Hf.indices)
    assert np.array_equal(Hc.data, Hf.data)


def test_matrix_free_eigen_fp64_and_mixed(pkg):
    # 4x4 torus, n = 5 (D = 15504).  The torus's symmetry makes the second
    # level four-fold degenerate, so the block holds 4 vectors (a block
    # Krylov space of width p holds at most p copies of a level in exact
    # arithmetic).  FP64 matrix-free vs FP64 stored CSR vs scipy on the stored
    # matrix, and the batched mixed-precision matrix-free solve within 1e-8.
    import scipy.sparse.linalg as sla

    m, n = 16, 5
    lists = square_lists(pkg, m)
    b = pkg.Basis(m, n)
    hc = pkg.Hamiltonian(b, lists)
    hf = pkg.Hamiltonian(b, lists, matrix_free=True)
    Js = np.linspace(0.02, 0.1, 6)
    ev_c, _, nc_c, _ = hc.eigsh_batch(Js, 1.0, 0.4, nev=4, block=4, precision=pkg.PREC_FP64)
    ev_f, _, nc_f, _ = hf.eigsh_batch(Js, 1.0, 0.4, nev=4, block=4, precision=pkg.PREC_FP64)
    assert nc_c.min() >= 4 and nc_f.min() >= 4
    np.testing.assert_allclose(ev_f, ev_c, rtol=1e-10, atol=1e-12)
    w = np.sort(sla.eigsh(hc.csr(Js[0], 1.0, 0.4), k=6, which="SA", tol=1e-13, ncv=60)[0])[:4]
    np.testing.assert_allclose(ev_f[0], w, rtol=1e-10, atol=1e-12)
    ev_m, _, nc_m, _ = hf.eigsh_batch(Js, 1.0, 0.4, nev=4, block=4, precision=pkg.PREC_MIXED, ncv=60)
    assert nc_m.min() >= 4
    np.testing.assert_allclose(ev_m, ev_c, rtol=1e-8, atol=1e-10)


def test_matrix_free_plain_solve_matches_dense(pkg):
    m, n = 9, 4  # 3x3 torus, D = 495; its second level is four-fold: block of 4
    lists = square_lists(pkg, m)
    hf = pkg.Hamiltonian(pkg.Basis(m, n), lists, matrix_free=True)
    ev, _, _, _ = hf.eigsh(0.17, 1.0, 0.3, nev=5, block=4)
    H = hf.csr(0.17, 1.0, 0.3).toarray()
    w = np.linalg.eigvalsh(H)[:5]
    np.testing.assert_allclose(ev, w, rtol=1e-10, atol=1e-12)


def test_matrix_free_rejects_wide_strings(pkg):
    # 17 sites x 4 bits (n = 8 needs 4 bits per site) = 68 bits > 64
    b = pkg.Basis(17, 8)
    with pytest.raises(ValueError, match="64 bits"):
        pkg.Hamiltonian(b, chain_lists(17), matrix_free=True)


def test_matrix_free_wide_batch_block4(pkg):
    # 16 solves x block 4 = 64 columns: the 32-lane matrix-free kernel and the
    # fused (block 4) CSR epilogue, both precisions, against each other
    m, n = 16, 6  # 4x4 torus, D = 54264
    lists = square_lists(pkg, m)
    b = pkg.Basis(m, n)
    hc = pkg.Hamiltonian(b, lists)
    hf = pkg.Hamiltonian(b, lists, matrix_free=True)
    Js = np.linspace(0.02, 0.1, 16)
    ev_c, _, nc_c, _ = hc.eigsh_batch(Js, 1.0, 0.4, nev=4, block=4, precision=pkg.PREC_FP64)
    ev_f, _, nc_f, _ = hf.eigsh_batch(Js, 1.0, 0.4, nev=4, block=4, precision=pkg.PREC_MIXED, ncv=60)
    ev_cm, _, nc_cm, _ = hc.eigsh_batch(Js, 1.0, 0.4, nev=4, block=4, precision=pkg.PREC_MIXED, ncv=60)
    assert min(nc_c.min(), nc_f.min(), nc_cm.min()) >= 4
    np.testing.assert_allclose(ev_f, ev_c, rtol=1e-8, atol=1e-10)
    np.testing.assert_allclose(ev_cm, ev_c, rtol=1e-8, atol=1e-10)
