"""GPU: Op::FOLM_diag (operator.cpp:39-71) through bh_folm_diag_csr -- the
Lanczos tridiagonalisation of a symmetric CSR matrix from a given start vector,
FP64 with full re-orthogonalisation.  Checked by the properties that define it
(the reference's own loop leaves v_i out of its orthogonalisation and stores
beta one row late, so its T and V are not an oracle):
V^T V = I, V^T H V = T tridiagonal, the start vector normalised in place and
V's first column equal to it, the lowest Ritz value of T converging to the
ground-state energy, and a breakdown in an invariant subspace."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import chain_lists

pytestmark = pytest.mark.gpu


def _sector_csr(pkg, m, n, J, U, mu):
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    rp, ci, val = h.csr_arrays(J, U, mu)
    return h, sp.csr_matrix((val, ci, rp), shape=(h.D, h.D))


def test_folm_diag_defines_the_lanczos_relation(pkg):
    m = n = 8
    J, U, mu = 0.1, 1.0, 0.5
    h, H = _sector_csr(pkg, m, n, J, U, mu)
    D, k = H.shape[0], 40
    v0 = np.random.default_rng(3).uniform(-1.0, 1.0, D)
    start = v0 / np.linalg.norm(v0)
    T, V, steps = pkg.Op.FOLM_diag(H, k, v0)
    assert steps == k
    assert np.allclose(v0, start, rtol=0, atol=1e-15)  # normalised in place
    assert np.allclose(V[:, 0], start, rtol=0, atol=1e-15)
    assert np.abs(V.T @ V - np.eye(k)).max() < 1e-12
    scale = np.abs(H).sum(axis=1).max()
    assert np.abs(V.T @ (H @ V) - T).max() < 1e-11 * scale
    band = np.abs(np.subtract.outer(np.arange(k), np.arange(k))) > 1
    assert np.all(T[band] == 0.0) and np.allclose(T, T.T, rtol=0, atol=0)
    assert np.all(np.diag(T, 1) > 0.0)
    e0 = h.eigsh(J, U, mu, nev=1)[0][0]
    ritz = np.linalg.eigvalsh(T)
    assert abs(ritz[0] - e0) < 1e-7 * abs(e0)
    assert ritz[0] >= e0 - 1e-12 * abs(e0)  # Ritz values bound the spectrum from inside


def test_folm_diag_breaks_down_in_an_invariant_subspace(pkg):
    # diag(1..8) from e_1 + e_2: the Krylov space is two-dimensional
    D = 8
    H = sp.diags(np.arange(1.0, D + 1)).tocsr()
    v0 = np.zeros(D)
    v0[0] = v0[1] = 1.0
    T, V, steps = pkg.Op.FOLM_diag(H, 5, v0)
    assert steps == 2
    assert np.allclose(np.sort(np.linalg.eigvalsh(T[:2, :2])), [1.0, 2.0], rtol=0, atol=1e-12)
    assert np.all(T[2:, :] == 0.0) and np.all(T[:, 2:] == 0.0) and np.all(V[:, 2:] == 0.0)


def test_folm_diag_rejects_bad_arguments(pkg):
    H = sp.diags(np.arange(1.0, 5.0)).tocsr()
    with pytest.raises(Exception):
        pkg.Op.FOLM_diag(H, 5, np.ones(4))  # more steps than the dimension
    with pytest.raises(Exception):
        pkg.Op.FOLM_diag(H, 2, np.zeros(4))  # zero start vector
    with pytest.raises(Exception):
        pkg.Op.FOLM_diag(H, 2, np.array([1.0, np.nan, 0.0, 0.0]))  # non-finite start vector
