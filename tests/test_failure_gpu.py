"""GPU: failure detection with host-side causes only (no device fault is
provoked).  Non-finite parameters are refused before any launch; a point whose
Krylov space is exhausted (H a multiple of the identity: every start block is
invariant) is reported as BH_ERR_BREAKDOWN for that point while the others of
the batch finish; a one-state sector solves exactly; a Krylov basis larger
than the device's memory fails its allocation with BH_ERR_NOMEM and leaves the
context usable."""
import numpy as np
import pytest

from conftest import chain_lists

pytestmark = pytest.mark.gpu


def test_non_finite_parameters_are_refused(pkg):
    h = pkg.Hamiltonian(pkg.Basis(6, 4), chain_lists(6))
    for J, U, mu in ((np.nan, 1.0, 0.0), (0.1, np.inf, 0.0), (0.1, 1.0, -np.inf)):
        with pytest.raises(ValueError, match="finite"):
            h.eigsh(J, U, mu, nev=2)
        with pytest.raises(ValueError, match="finite"):
            h.eigsh_batch(np.array([0.1, J]), U, mu, nev=2)
        with pytest.raises(ValueError, match="finite"):
            pkg.eigsh_sectors([h], np.array([J]), U, mu, nev=2)
        with pytest.raises(ValueError, match="finite"):
            h.apply(np.ones(h.D), J, U, mu)
        with pytest.raises(ValueError, match="finite"):
            h.csr(J, U, mu)
    # the library still works after the refusals
    ev, _, _, _ = h.eigsh(0.1, 1.0, 0.0, nev=2)
    assert np.all(np.isfinite(ev))


def test_invariant_start_block_is_a_breakdown(pkg):
    # J = U = 0: H = -mu n I, every block is invariant, the Krylov space holds
    # one block (2 directions) and nev = 4 cannot be reached
    m, n = 5, 3
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    with pytest.raises(pkg.BHError) as ei:
        h.eigsh(0.0, 0.0, 0.5, nev=4, block=2)
    assert ei.value.code == pkg.BH_ERR_BREAKDOWN
    # in a batch the failing point is reported on its own; the others finish
    J = np.array([0.1, 0.0, 0.2])
    U = np.array([1.0, 0.0, 1.0])
    ev, rs, nc, info, st = h.eigsh_batch(J, U, 0.5, nev=4, block=2, status=True)
    assert st.tolist() == [pkg.BH_OK, pkg.BH_ERR_BREAKDOWN, pkg.BH_OK]
    assert nc[0] == 4 and nc[2] == 4 and nc[1] < 4
    # the values it holds are the level -mu n; NaN beyond them
    held = ev[1][np.isfinite(ev[1])]
    assert len(held) >= 1 and np.allclose(held, -0.5 * n, rtol=1e-12)
    w = np.linalg.eigvalsh(h.csr(0.2, 1.0, 0.5).toarray())[:4]
    np.testing.assert_allclose(ev[2], w, rtol=1e-10, atol=1e-12)
    # without status the point shows up as nconv < nev, and the call succeeds
    ev2, _, nc2, _ = h.eigsh_batch(J, U, 0.5, nev=4, block=2)
    assert nc2.tolist() == nc.tolist()


def test_one_state_sectors(pkg):
    # m = 1 (no bonds): one state |n>, E = U n (n - 1) / 2 - mu n
    b = pkg.Basis(1, 3)
    assert b.D == 1
    h = pkg.Hamiltonian(b, [[]])
    ev, rs, _, _ = h.eigsh(0.3, 1.5, 0.25, nev=1)
    assert abs(ev[0] - (1.5 * 3 - 0.25 * 3)) < 1e-14
    # n = 0: the empty state, E = 0
    h0 = pkg.Hamiltonian(pkg.Basis(4, 0), chain_lists(4))
    ev0, _, nc0, _ = h0.eigsh_batch(np.array([0.1, 0.2]), 1.0, 0.7, nev=1)
    assert nc0.tolist() == [1, 1] and np.all(ev0 == 0.0)


def test_krylov_basis_beyond_device_memory_is_nomem(pkg):
    # 601 basis blocks x D = 293930 rows x (256 points x block 2) columns in
    # FP64 is about 723 GB for the first basis buffer: more than the device
    # holds.  The allocation fails cleanly before any kernel of the solve has
    # run, and later calls work.
    h = pkg.Hamiltonian(pkg.Basis(10, 12), chain_lists(10))
    J = np.full(256, 0.1)
    with pytest.raises(pkg.BHError) as ei:
        h.eigsh_batch(J, 1.0, 0.0, nev=10, block=2, ncv=1200, precision=pkg.PREC_FP64)
    assert ei.value.code == pkg.BH_ERR_NOMEM
    assert "cudaMalloc" in str(ei.value)
    ev, _, nc, _ = h.eigsh_batch(np.array([0.1]), 1.0, 0.0, nev=4)
    assert nc[0] == 4 and np.all(np.isfinite(ev))
