"""GPU: device basis and device Hamiltonian against the oracle and the reference's
golden basis (bit-exact order, tags, CSR pattern; values within 1 ulp)."""
import hashlib

import numpy as np
import pytest

from conftest import chain_lists, oracle_H

pytestmark = pytest.mark.gpu


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_basis_bit_exact_vs_reference(pkg, golden):
    for key, rec in golden["basis"].items():
        b = pkg.Basis(rec["m"], rec["n"])
        assert b.D == rec["D"]
        col_of_lex, lex_of_col = b.orders()
        assert _sha(col_of_lex.astype("<i4")) == rec["col_of_lex_sha256"], key
        assert np.array_equal(col_of_lex[lex_of_col], np.arange(b.D)), key
        tags, basis = b.copy()
        assert _sha(tags.astype("<f8")) == rec["tags_sha256"], key
        if "tags_hex" in rec:
            assert [float.fromhex(h) for h in rec["tags_hex"]] == tags.tolist()
        assert basis.shape == (rec["m"], rec["D"])
        assert np.all(basis.sum(axis=0) == rec["n"])


def test_basis_large_sizes_consistent(pkg, orc):
    # 128-bit keys (m = 14, n = 14 needs 76 bits; 4x4 / n = 12 needs 69 bits)
    for m, n in [(14, 8), (16, 6), (25, 3)]:
        b = pkg.Basis(m, n)
        col_of_lex, lex_of_col = b.orders()
        occ = orc.lex_states(m, n)
        ref_col, _ = orc.reference_order(occ)
        assert np.array_equal(col_of_lex, ref_col), (m, n)


def test_basis_index_lookup(pkg, orc):
    m, n = 7, 5
    b = pkg.Basis(m, n)
    occ = orc.lex_states(m, n)
    col_of_lex, _ = b.orders()
    got = b.index(occ)
    assert np.array_equal(got, col_of_lex)
    bad = occ[:3].copy()
    bad[:, 0] += 1  # wrong particle number
    assert np.all(b.index(bad) == -1)


@pytest.mark.parametrize("m,n", [(2, 3), (3, 3), (6, 6), (8, 8), (5, 9)])
def test_csr_pattern_and_values_vs_oracle(pkg, orc, m, n):
    lists = chain_lists(m)
    h = pkg.Hamiltonian(pkg.Basis(m, n), lists)
    occ, col_of_lex, lex_of_col, rp, ci, tv, vd = oracle_H(orc, m, n, lists)
    assert h.nnz_offdiag == rp[-1]
    J, U, mu = 0.37, 1.3, 0.45
    H = h.csr(J, U, mu)
    Ho = orc.full_csr(rp, ci, tv, vd, n, J, U, mu)
    # pattern: explicit diagonal in every row + the hopping entries
    Hd = Ho.tolil()
    Hd.setdiag(Ho.diagonal())
    Hd = Hd.tocsr()
    Hd.sort_indices()
    assert np.array_equal(H.indptr, Hd.indptr)
    assert np.array_equal(H.indices, Hd.indices)
    np.testing.assert_array_max_ulp(H.data, Hd.data, maxulp=1)


def test_csr_lex_order_vs_oracle(pkg, orc):
    m, n = 7, 6
    lists = chain_lists(m, closed=False)
    h = pkg.Hamiltonian(pkg.Basis(m, n), lists)
    _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, lists, order="lex")
    rpg, cig, vg = h.csr_arrays(1.0, 0.0, 0.0, order=pkg.ORDER_LEX)
    # strip the (zero) diagonal entries
    rows = np.repeat(np.arange(h.D), np.diff(rpg))
    keep = cig != rows
    assert np.array_equal(cig[keep], ci)
    np.testing.assert_array_max_ulp(vg[keep], tv, maxulp=1)


def test_square_lattice_and_duplicate_bonds(pkg, orc):
    # 2x2 torus: each neighbour appears twice -> merged entries (2 sqrt(..))
    nb = pkg.Neighbours(4)
    nb.square_neighbours(True)
    lists = nb.getNeighbours()
    h = pkg.Hamiltonian(pkg.Basis(4, 3), lists)
    _, _, _, rp, ci, tv, vd = oracle_H(orc, 4, 3, lists)
    rpg, cig, vg = h.csr_arrays(1.0, 0.0, 0.0)
    rows = np.repeat(np.arange(h.D), np.diff(rpg))
    keep = cig != rows
    assert np.array_equal(cig[keep], ci)
    np.testing.assert_array_max_ulp(vg[keep], tv, maxulp=1)


def test_apply_matches_oracle(pkg, orc):
    m, n = 8, 8
    lists = chain_lists(m)
    h = pkg.Hamiltonian(pkg.Basis(m, n), lists)
    _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, lists)
    x = np.random.RandomState(1).randn(h.D, 3)
    for order in (pkg.ORDER_REFERENCE,):
        y = h.apply(x, 0.1, 1.0, 0.5, order=order)
        for k in range(3):
            yo = orc.spmv(rp, ci, tv, vd, n, 0.1, 1.0, 0.5, np.ascontiguousarray(x[:, k]))
            np.testing.assert_allclose(y[:, k], yo, rtol=1e-13, atol=1e-13)


def test_invalid_lattices_rejected(pkg):
    b = pkg.Basis(3, 2)
    with pytest.raises(ValueError, match="self-bond"):
        pkg.Hamiltonian(b, [[0], [2], [1]])
    with pytest.raises(ValueError, match="symmetric"):
        pkg.Hamiltonian(b, [[1], [2], [0]])


def test_fixed_bosons_hamiltonian_term_selection(pkg, orc):
    m, n = 5, 4
    lists = chain_lists(m)
    tags, basis = pkg.BH.fixed_set_basis(m, n)
    JH = pkg.BH.fixed_bosons_hamiltonian(lists, basis, tags, m, n, 1.0, 0.0, 0.0)
    UH = pkg.BH.fixed_bosons_hamiltonian(lists, basis, tags, m, n, 0.0, 1.0, 0.0)
    uH = pkg.BH.fixed_bosons_hamiltonian(lists, basis, tags, m, n, 0.0, 0.0, 1.0)
    _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, lists)
    T = orc.full_csr(rp, ci, tv, vd, n, 1.0, 0.0, 0.0)
    assert (JH - T).count_nonzero() == 0 and JH.diagonal().sum() == 0
    assert UH.nnz == len(vd) and np.array_equal(UH.diagonal(), vd)
    assert np.all(uH.diagonal() == -n)
    H = JH * 0.2 + UH * 1.0 + uH * 0.3  # analysis.cpp:311 composition
    Ho = orc.full_csr(rp, ci, tv, vd, n, 0.2, 1.0, 0.3)
    assert abs(H - Ho).max() < 1e-15


def test_multi_sector_csr_is_the_block_diagonal_of_the_sectors(pkg):
    # BH::max_bosons_hamiltonian (hamiltonian.cpp:260-288): sectors n_min..n_max
    # of one lattice as one block-diagonal matrix, assembled on the device
    import scipy.sparse as sp

    m = 6
    lists = chain_lists(m)
    hams = [pkg.Hamiltonian(pkg.Basis(m, n), lists) for n in range(0, 5)]
    for order in (pkg.ORDER_REFERENCE, pkg.ORDER_LEX):
        H = pkg.multi_sector_csr(hams, 0.13, 0.9, 0.4, order=order)
        want = sp.block_diag([h.csr(0.13, 0.9, 0.4, order=order) for h in hams], format="csr")
        assert H.shape == want.shape
        assert np.array_equal(H.indptr, want.indptr) and np.array_equal(H.indices, want.indices)
        assert np.array_equal(H.data, want.data)
    # the reference's term selection, block by block
    for J, U, mu in ((0.1, 0.0, 0.0), (0.0, 1.0, 0.0), (0.0, 0.0, 0.7)):
        Hm = pkg.BH.max_bosons_hamiltonian(lists, m, -1, 4, J, U, mu)
        blocks = [pkg.BH.fixed_bosons_hamiltonian(lists, None, None, m, n, J, U, mu) for n in range(0, 5)]
        want = sp.block_diag(blocks, format="csr")
        assert Hm.shape == want.shape and abs(Hm - want).max() == 0.0
        assert Hm.nnz == want.nnz
