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
