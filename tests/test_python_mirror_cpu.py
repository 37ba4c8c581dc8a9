"""CPU: the host-only members of the Python mirror of the reference's BH
namespace (hamiltonian.hpp:33-112) against the reference's own values:
tags of the reference-ordered basis bit for bit (golden vectors made by the
reference's compiled code), the tag search, and the mean-field single-site
matrix."""
import math

import numpy as np
import pytest


@pytest.mark.parametrize("key", ["3,3", "4,4", "2,3"])
def test_calculate_tags_match_reference(pkg, orc, golden, key):
    rec = golden["basis"][key]
    m, n = int(rec["m"]), int(rec["n"])
    occ = orc.lex_states(m, n)
    _, lex_of_col = orc.reference_order(occ)
    basis = occ[lex_of_col].T.astype(np.float64)  # column c = state at reference column c
    tags = pkg.BH.calculate_tags(basis, pkg.BH.PRIMES)
    assert tags.tolist() == [float.fromhex(h) for h in rec["tags_hex"]]
    for k in range(len(tags)):
        assert pkg.BH.search_tag(tags, tags[k]) == k


def test_h_mf_entries(pkg):
    p, mu, J, q, psi = 3, 0.7, 0.05, 4, 0.31
    BH = pkg.BH
    h = BH.h_MF(psi, p, mu, J, q)
    k = 2 * p + 1
    assert h.shape == (k, k)
    assert np.array_equal(h, h.T)
    for i in range(k):
        assert h[i, i] == -mu * i + 0.5 * i * (i - 1) + q * J * psi * psi
        for j in range(k):
            if abs(i - j) > 1:
                assert h[i, j] == 0.0
    for a in range(k - 1):
        assert h[a + 1, a] == -q * J * psi * math.sqrt(a + 1)
    # psi = 0: diagonal, lowest level at the occupation nearest mu + 1/2
    h0 = BH.h_MF(0.0, p, 1.3, J, q)
    assert np.count_nonzero(h0 - np.diag(np.diag(h0))) == 0
    assert int(np.argmin(np.diag(h0))) == 2


@pytest.mark.parametrize("key", ["3,3", "4,4", "2,3", "1,3"])
def test_sort_basis_gives_the_reference_order(pkg, orc, golden, key):
    # the reference's fixed_set_basis is init_lexicographic -> calculate_tags
    # -> sort_basis; applied to the lexicographic basis, the mirror's
    # sort_basis must give the golden order and tags bit for bit
    rec = golden["basis"][key]
    m, n = int(rec["m"]), int(rec["n"])
    occ = orc.lex_states(m, n)
    basis_lex = occ.T.astype(np.float64)
    tags_lex = pkg.BH.calculate_tags(basis_lex, pkg.BH.PRIMES)
    tags, basis = pkg.BH.sort_basis(tags_lex, basis_lex)
    assert tags.tolist() == [float.fromhex(h) for h in rec["tags_hex"]]
    col_of_lex = rec["col_of_lex"]
    for r in range(occ.shape[0]):
        assert np.array_equal(basis[:, col_of_lex[r]], basis_lex[:, r])


def _fake_sectors(pkg, orc, monkeypatch, m, lists):
    """fixed_set_basis / fixed_bosons_hamiltonian from the oracle (host only)."""
    import scipy.sparse as sp

    def fixed_set_basis(mm, n):
        occ = orc.lex_states(mm, n)
        b = occ.T.astype(np.float64)
        return pkg.BH.sort_basis(pkg.BH.calculate_tags(b, pkg.BH.PRIMES), b)

    def fixed_bosons_hamiltonian(nb, basis, tags, mm, n, J, U, mu):
        from conftest import oracle_H

        _, _, _, rp, ci, tv, vd = oracle_H(orc, mm, n, nb)
        D = len(rp) - 1
        if J != 0.0:
            return sp.csr_matrix((J * tv, ci, rp), shape=(D, D))
        return sp.diags(U * vd - mu * n).tocsr()

    monkeypatch.setattr(pkg.BH, "fixed_set_basis", staticmethod(fixed_set_basis))
    monkeypatch.setattr(pkg.BH, "fixed_bosons_hamiltonian", staticmethod(fixed_bosons_hamiltonian))


def test_max_set_basis_holds_every_state_once(pkg, orc, monkeypatch):
    from conftest import chain_lists

    m, n = 4, 3
    _fake_sectors(pkg, orc, monkeypatch, m, chain_lists(m))
    tags, basis = pkg.BH.max_set_basis(m, n)
    assert basis.shape == (m, sum(pkg.BH.dimension(m, k) for k in range(1, n + 1)))
    seen = {tuple(basis[:, c].astype(int)) for c in range(basis.shape[1])}
    assert len(seen) == basis.shape[1]
    assert all(1 <= sum(s) <= n for s in seen)
    # the reference's sort: column argsort(concatenated tags)[r] = concatenated column r
    for c in range(basis.shape[1]):
        assert tags[c] == pkg.BH.calculate_tag(basis, pkg.BH.PRIMES, c)


def _fake_multi_sector(pkg, orc, monkeypatch):
    """Device Basis / Hamiltonian / multi_sector_csr replaced by the oracle's
    sectors (host only): the device assembly itself is a GPU test."""
    import scipy.sparse as sp
    from conftest import oracle_H

    class FakeBasis:
        def __init__(self, m, n):
            self.m, self.n, self.D = m, n, pkg.BH.dimension(m, n)

    class FakeHam:
        def __init__(self, basis, lists):
            self.basis, self.lists = basis, lists

    def multi(hams, J, U, mu, order=pkg.ORDER_REFERENCE):
        blocks = []
        for h in hams:
            m, n = h.basis.m, h.basis.n
            _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, h.lists)
            D = len(rp) - 1
            blocks.append(sp.csr_matrix((J * tv, ci, rp), shape=(D, D)) + sp.diags(U * vd - mu * n))
        return sp.block_diag(blocks, format="csr")

    monkeypatch.setattr(pkg, "Basis", FakeBasis)
    monkeypatch.setattr(pkg, "Hamiltonian", FakeHam)
    monkeypatch.setattr(pkg, "multi_sector_csr", multi)


def test_max_bosons_hamiltonian_blocks_and_clamping(pkg, orc, monkeypatch):
    from conftest import chain_lists

    m = 4
    lists = chain_lists(m)
    _fake_sectors(pkg, orc, monkeypatch, m, lists)
    _fake_multi_sector(pkg, orc, monkeypatch)
    H = pkg.BH.max_bosons_hamiltonian(lists, m, -2, 3, 0.1, 0.0, 0.0)
    dims = [pkg.BH.dimension(m, k) for k in range(0, 4)]
    assert H.shape == (sum(dims), sum(dims))
    o = 0
    for k, d in enumerate(dims):
        blk = pkg.BH.fixed_bosons_hamiltonian(lists, None, None, m, k, 0.1, 0.0, 0.0)
        assert abs(H[o:o + d, o:o + d] - blk).max() == 0.0
        assert H[o:o + d, o + d:].nnz == 0
        o += d
    # n_max < n_min: the single sector n_min
    H1 = pkg.BH.max_bosons_hamiltonian(lists, m, 2, 1, 0.0, 1.0, 0.0)
    assert H1.shape == (dims[2], dims[2])


def test_folm_eigen_clamps_and_orders(pkg, monkeypatch):
    # the eigensolve itself is the GPU path of IRLM_eigen (tested with -m gpu);
    # here a dense stand-in checks FOLM's count and ordering around it
    rng = np.random.default_rng(3)
    A = rng.standard_normal((12, 12))
    A = A + A.T
    w, z = np.linalg.eigh(A)
    calls = []

    def irlm(O, nev, **opt):
        calls.append(nev)
        order = np.argsort(-np.abs(w[:nev]), kind="stable")
        return w[:nev][order].astype(complex), z[:, :nev][:, order].astype(complex)

    monkeypatch.setattr(pkg.Op, "IRLM_eigen", staticmethod(irlm))
    vals, vecs = pkg.Op.FOLM_eigen(A, 5)
    assert calls[-1] == 5 and np.array_equal(vals, w[:5]) and np.array_equal(vecs, z[:, :5])
    vals, _ = pkg.Op.FOLM_eigen(A, 50)
    assert calls[-1] == 10 and np.array_equal(vals, w[:10])  # n - 2
    pkg.Op.FOLM_eigen(A, 0)
    assert calls[-1] == 1


def test_folm_diag_checks_its_start_vector_before_the_device(pkg):
    # v_0 is normalised in place by the library, so it must be the caller's own
    # contiguous float64 array of the matrix dimension: anything else is
    # refused on the host, before any library call
    import scipy.sparse as sp

    H = sp.diags(np.arange(1.0, 5.0)).tocsr()
    for bad in (np.ones(4, np.float32), np.ones(5), np.ones((4, 1)), np.ones(8)[::2], [1.0, 0.0, 0.0, 0.0]):
        with pytest.raises(TypeError):
            pkg.Op.FOLM_diag(H, 2, bad)
