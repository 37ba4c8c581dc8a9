"""CPU: the oracle is pinned against golden vectors recorded from the reference."""
import hashlib

import numpy as np
import pytest

from conftest import chain_lists, oracle_H


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_basis_order_and_tags_match_reference(orc, golden):
    for key, rec in golden["basis"].items():
        m, n = rec["m"], rec["n"]
        occ = orc.lex_states(m, n)
        assert len(occ) == rec["D"] == orc.dimension(m, n)
        col_of_lex, lex_of_col = orc.reference_order(occ)
        assert _sha(col_of_lex.astype("<i4")) == rec["col_of_lex_sha256"], key
        tags = orc.tags(occ)[lex_of_col]
        assert _sha(tags.astype("<f8")) == rec["tags_sha256"], key
        if "col_of_lex" in rec:
            assert col_of_lex.tolist() == rec["col_of_lex"]
            assert [float.fromhex(h) for h in rec["tags_hex"]] == tags.tolist()


def test_rank_inverts_enumeration(orc):
    for m, n in [(1, 4), (2, 5), (4, 4), (7, 3), (3, 9)]:
        occ = orc.lex_states(m, n)
        assert all(orc.rank(occ[r]) == r for r in range(len(occ)))


def test_nnz_formula(orc):
    # nnz_off = (#directed bonds) * C(m+n-2, n-1) on a ring
    for m, n in [(8, 8), (6, 4), (5, 7)]:
        _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, chain_lists(m))
        assert rp[-1] == 2 * m * orc.dimension(m, n - 1)


def test_irlm_port_matches_reference(orc, golden):
    for name in ["m8n8", "m6n6", "m5n5_J0.2", "m6n4_J0.3"]:
        rec = golden["irlm"][name]
        m, n = rec["m"], rec["n"]
        _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, chain_lists(m))
        ev, _, _, _ = orc.irlm(rp, ci, tv, vd, n, rec["J"], rec["U"], rec["mu"], nev=rec["nev"])
        ref = np.array(rec["evals_sorted"])
        assert len(ev) == len(ref)
        np.testing.assert_allclose(np.sort(ev), ref, rtol=1e-10, atol=1e-12)
        # reference output order: descending magnitude
        np.testing.assert_allclose(ev, rec["evals_reference_order"], rtol=1e-10, atol=1e-12)


def test_oracle_against_dense_reference(orc, golden):
    for key, vals in golden["exact_eigen"].items():
        m, n, J, U, mu = key.split(",")
        m, n, J, U, mu = int(m), int(n), float(J), float(U), float(mu)
        _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, chain_lists(m))
        H = orc.full_csr(rp, ci, tv, vd, n, J, U, mu).toarray()
        np.testing.assert_allclose(np.linalg.eigvalsh(H), vals, rtol=1e-12, atol=1e-12)


def test_analytic_limits(orc):
    m, n = 6, 5
    _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, chain_lists(m))
    # J = 0: diagonal U/2 sum n(n-1) - mu n
    H0 = orc.full_csr(rp, ci, tv, vd, n, 0.0, 1.0, 0.3).toarray()
    assert np.count_nonzero(H0 - np.diag(np.diag(H0))) == 0
    # U = 0: free bosons on a ring, single-particle -2J cos(2 pi k / m)
    J = 0.7
    H = orc.full_csr(rp, ci, tv, vd, n, J, 0.0, 0.0).toarray()
    e0 = np.linalg.eigvalsh(H)[0]
    assert abs(e0 - (-2 * J * n)) < 1e-10


def test_gap_ratio_and_coherence_match_reference(orc, golden):
    ev = np.array(golden["irlm"]["m8n8"]["evals_reference_order"])
    g, r = orc.gap_ratio(ev)
    np.testing.assert_allclose(r, golden["gap_ratios_m8n8"], rtol=0, atol=0)
    rho = np.array(golden["coherence"]["rho"])
    assert orc.coherence(rho) == pytest.approx(golden["coherence"]["value"], rel=1e-14)


def test_reference_irlm_grid_recorded(golden):
    # every recorded grid point converged in the reference
    for name, rec in golden["irlm"].items():
        assert rec["converged"], name
        assert rec["imag_max"] == 0.0
