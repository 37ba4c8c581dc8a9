"""GPU: the multi-sector batched entry point returns, per sector, what the
single-sector batch returns (the sectors run concurrently on their own
streams)."""
import numpy as np
import pytest

from conftest import chain_lists

pytestmark = pytest.mark.gpu


def test_sectors_match_single_sector_batches(pkg):
    m = 8
    hams = [pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m)) for n in (5, 6, 7, 8)]
    J = np.linspace(0.02, 0.3, 12)
    ev, rs, nc, info = pkg.eigsh_sectors(hams, J, 1.0, 0.3, nev=6, precision=pkg.PREC_MIXED)
    assert ev.shape == (4, 12, 6) and nc.min() >= 6
    for k, h in enumerate(hams):
        e1, _, n1, _ = h.eigsh_batch(J, 1.0, 0.3, nev=6, precision=pkg.PREC_MIXED)
        # same kernels in the same order on each stream: identical results
        np.testing.assert_array_equal(ev[k], e1)
    ev64, _, _, _ = pkg.eigsh_sectors(hams, J, 1.0, 0.3, nev=6, precision=pkg.PREC_FP64)
    np.testing.assert_allclose(ev, ev64, rtol=1e-8, atol=1e-10)


def test_sectors_report_errors_per_sector(pkg):
    h = pkg.Hamiltonian(pkg.Basis(4, 2), chain_lists(4))  # D = 10
    with pytest.raises(Exception):
        pkg.eigsh_sectors([h], [0.1], 1.0, 0.0, nev=20)  # more values than the dimension
