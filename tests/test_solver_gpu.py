"""GPU: eigensolver parity.

FP64 plain method: eigenvalues within 1e-10 relative of the reference's Spectra
IRLM results (golden), including degenerate copies.  Mixed precision: within
1e-8 relative of the FP64 results."""
import numpy as np
import pytest

from conftest import chain_lists, oracle_H, reference_lowest

pytestmark = pytest.mark.gpu

# Parity bar: |dE| <= RTOL |E| + ATOL.  The absolute floor matters only for
# eigenvalues near zero, whose relative error is ill-conditioned (a change of
# mu shifts them); it is far below the eps * ||H|| ~ 1e-14 noise of FP64.
RTOL_FP64, ATOL_FP64 = 1e-10, 1e-12
RTOL_MIXED, ATOL_MIXED = 1e-8, 1e-10


def _rel(a, b, atol=ATOL_FP64, rtol=RTOL_FP64):
    """max of |a - b| / (|b| + atol / rtol): < rtol  <=>  |a - b| < rtol |b| + atol."""
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b) / (np.abs(b) + atol / rtol))


@pytest.mark.parametrize("name", ["m8n8", "m6n6", "m5n5_J0.2", "m6n4_J0.3", "m10n8"])
def test_fp64_matches_reference_irlm(pkg, golden, name):
    rec = golden["irlm"][name]
    m, n = rec["m"], rec["n"]
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    ev, rs, _, info = h.eigsh(rec["J"], rec["U"], rec["mu"], nev=rec["nev"])
    assert _rel(ev, reference_lowest(rec)) < RTOL_FP64
    assert np.all(rs < 1e-9)
    assert info.nconv == rec["nev"]


def test_m8_known_answers(pkg):
    h = pkg.Hamiltonian(pkg.Basis(8, 8), chain_lists(8))
    ev, _, _, _ = h.eigsh(0.1, 1.0, 0.5, nev=10)
    assert abs(ev[0] - (-4.317353604401086)) < 1e-12
    # degenerate pairs are resolved with multiplicity
    assert abs(ev[2] - ev[3]) < 1e-11 and abs(ev[2] - (-3.7235662)) < 1e-7


def test_analytic_limits(pkg, orc):
    m, n = 8, 6
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    # U = 0: free bosons, E0 = -2 J n
    J = 0.4
    ev, _, _, _ = h.eigsh(J, 0.0, 0.0, nev=4)
    assert abs(ev[0] + 2 * J * n) < 1e-10
    # sums of single-particle levels -2J cos(2 pi k / m): first excitation
    eps = np.sort(-2 * J * np.cos(2 * np.pi * np.arange(m) / m))
    assert abs(ev[1] - ((n - 1) * eps[0] + eps[1])) < 1e-10
    # small J: the Mott manifold (all sites singly occupied, energy -mu n)
    # shifted at second order in J; compared with the dense oracle spectrum
    _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, chain_lists(m))
    H = orc.full_csr(rp, ci, tv, vd, n, 0.05, 1.0, 0.3).toarray()
    w = np.linalg.eigvalsh(H)[:4]
    ev, _, _, _ = h.eigsh(0.05, 1.0, 0.3, nev=4)
    np.testing.assert_allclose(ev, w, rtol=1e-10)
    assert ev[0] < -0.3 * n  # below the Mott manifold energy


def test_irlm_eigen_dropin_on_generic_matrix(pkg, golden, orc):
    rec = golden["irlm"]["m8n8"]
    _, _, _, rp, ci, tv, vd = oracle_H(orc, 8, 8, chain_lists(8))
    H = orc.full_csr(rp, ci, tv, vd, 8, rec["J"], rec["U"], rec["mu"])
    vals, vecs = pkg.Op.IRLM_eigen(H, 10)
    assert vals.dtype == complex and vecs.shape == (H.shape[0], 10)
    # reference ordering: descending magnitude
    np.testing.assert_allclose(vals.real, rec["evals_reference_order"], rtol=RTOL_FP64)
    R = H @ vecs.real - vecs.real * vals.real
    assert np.linalg.norm(R, axis=0).max() < 1e-8
    G = vecs.real.T @ vecs.real
    assert np.abs(G - np.eye(10)).max() < 1e-10


def test_eigenvectors_reference_order(pkg, orc):
    m, n = 6, 6
    lists = chain_lists(m)
    h = pkg.Hamiltonian(pkg.Basis(m, n), lists)
    ev, _, vec, _ = h.eigsh(0.2, 1.0, 0.1, nev=4, vectors=True)
    _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, lists)
    H = orc.full_csr(rp, ci, tv, vd, n, 0.2, 1.0, 0.1)
    R = H @ vec - vec * ev
    assert np.linalg.norm(R, axis=0).max() < 1e-9


def test_mixed_precision_vs_fp64(pkg, golden):
    rec = golden["irlm"]["m10n8"]
    h = pkg.Hamiltonian(pkg.Basis(10, 8), chain_lists(10))
    Js = np.array([0.05, 0.15, 0.25])
    ev64, _, _, _ = h.eigsh_batch(Js, 1.0, 0.0, nev=10)
    ev32, rs32, nc, info = h.eigsh_batch(Js, 1.0, 0.0, nev=10, precision=pkg.PREC_MIXED)
    assert _rel(ev32, ev64, ATOL_MIXED, RTOL_MIXED) < RTOL_MIXED
    assert _rel(ev64[1], reference_lowest(rec)) < RTOL_FP64


def test_tiny_dimensions(pkg, orc):
    # D = 1 (n = 0), D = n + 1 (m = 2), D <= nev + block
    for m, n, nev in [(3, 0, 1), (2, 3, 2), (3, 2, 4)]:
        lists = chain_lists(m)
        h = pkg.Hamiltonian(pkg.Basis(m, n), lists)
        if h.D < 3 and nev > h.D:
            continue
        _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, lists)
        H = orc.full_csr(rp, ci, tv, vd, n, 0.3, 1.0, 0.2).toarray()
        w = np.linalg.eigvalsh(H)[:nev]
        ev, _, _, _ = h.eigsh(0.3, 1.0, 0.2, nev=nev)
        np.testing.assert_allclose(ev, w, rtol=1e-10, atol=1e-12)


def test_nonconvergence_is_reported(pkg):
    h = pkg.Hamiltonian(pkg.Basis(8, 8), chain_lists(8))
    with pytest.raises(pkg.BHError, match="Eigenvalue computation failed"):
        h.eigsh(0.1, 1.0, 0.5, nev=10, max_restarts=1, ncv=22)


def test_exact_eigen_matches_reference_dense_spectra(pkg, orc, golden):
    # Op::exact_eigen (operator.cpp:92-101): every eigenvalue of the dense
    # Hamiltonian, ascending, against the reference's own Eigen
    # SelfAdjointEigenSolver run on the same matrices
    for key, want in golden["exact_eigen"].items():
        m, n, J, U, mu = key.split(",")
        m, n, J, U, mu = int(m), int(n), float(J), float(U), float(mu)
        _, _, _, rp, ci, tv, vd = oracle_H(orc, m, n, chain_lists(m))
        H = orc.full_csr(rp, ci, tv, vd, n, J, U, mu)
        w, z = pkg.Op.exact_eigen(H)
        want = np.array(want)
        assert w.shape == want.shape
        scale = max(1.0, np.abs(want).max())
        np.testing.assert_allclose(w, want, rtol=1e-12, atol=1e-12 * scale)
        # the eigenvectors: orthonormal columns with H z = z diag(w)
        Hd = H.toarray()
        np.testing.assert_allclose(z.T @ z, np.eye(len(w)), atol=1e-12)
        np.testing.assert_allclose(Hd @ z, z * w, atol=1e-11 * scale)
