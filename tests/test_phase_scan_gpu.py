"""GPU: the exact phase scan (Analysis::exact_parameters + calculate_and_save,
src/analysis.cpp:207-427) on the device against the same quantities computed
point by point from dense eigensolves of the stored Hamiltonian."""
import numpy as np
import pytest

from conftest import chain_lists

pytestmark = pytest.mark.gpu


def test_phase_scan_matches_dense_per_point(pkg, tmp_path):
    m, n, nev = 6, 6, 20
    path = tmp_path / "phase.txt"
    # J fixed at 0.25; the swept pairs (exact steps): param1 in {0.25, 0.5, 0.75}
    # scales V (the reference pairs the J range with the U term), param2 in {0.5, 0.75, 1}
    P1, P2, gap, cf, coh = pkg.Analysis.exact_parameters(m, n, 0.25, 1.0, 0.5, 0.25, 0.5, "J",
                                                         path=str(path), nb_eigen=nev,
                                                         precision=pkg.PREC_FP64)
    lines = path.read_text().splitlines()
    assert lines[0] == "J 0.25"
    assert len(lines) == 1 + len(P1) == 1 + 9
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    for k in range(len(P1)):
        J, U, mu = 0.25, P1[k], P2[k]  # fixed J: param1 scales V, param2 the -N term
        H = h.csr(J, U, mu).toarray()
        w, v = np.linalg.eigh(H)
        ev = w[:nev]
        r = pkg.Analysis.gap_ratios(ev, nev)
        assert abs(gap[k] - r.mean()) < 1e-9
        i = int(np.argmax(np.abs(ev)))
        # the largest-|lambda| level must be simple for its vector to be defined
        nbr = [abs(ev[i] - ev[t]) for t in (i - 1, i + 1) if 0 <= t < nev]
        if min(nbr + [abs(ev[i] - w[nev])] if i == nev - 1 else nbr) < 1e-6:
            continue
        rho = h.spdm(v[:, i])
        wr = np.linalg.eigvalsh(rho)
        assert abs(cf[k] - abs(wr[np.argmax(np.abs(wr))] / np.trace(rho))) < 1e-8
        assert abs(coh[k] - pkg.Analysis.coherence(rho)) < 1e-8
    assert np.all((gap > 0) & (gap < 1)) and np.all((cf > 0) & (cf <= 1))


def test_phase_scan_rejects_all_zero(pkg, capsys):
    assert pkg.Analysis.exact_parameters(4, 2, 0.0, 0.0, 0.0, 0.1, 0.1, "J", path=None) is None
    assert "At least one of the parameters" in capsys.readouterr().err
