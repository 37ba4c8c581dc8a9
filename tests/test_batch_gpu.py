"""GPU: the batched multi-sector solver (many J points of one sector per launch
sequence) against the reference's IRLM golden values, the FP64 plain path and
the observables."""
import numpy as np
import pytest

from conftest import chain_lists, oracle_H, reference_lowest

pytestmark = pytest.mark.gpu


def _rel(a, b, atol=1e-12, rtol=1e-10):
    """max of |a - b| / (|b| + atol / rtol): < rtol  <=>  |a - b| < rtol |b| + atol
    (the absolute floor only matters for eigenvalues near zero)."""
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b) / (np.abs(b) + atol / rtol))


def _grid_cases(golden):
    return {k: v for k, v in golden["irlm"].items() if k.startswith("grid_")}


def test_batched_grid_matches_reference(pkg, golden):
    cases = _grid_cases(golden)
    by_n = {}
    for name, rec in cases.items():
        by_n.setdefault(rec["n"], []).append(rec)
    for n, recs in by_n.items():
        h = pkg.Hamiltonian(pkg.Basis(10, n), chain_lists(10))
        Js = np.array([r["J"] for r in recs])
        for prec, tol, atol in ((pkg.PREC_FP64, 1e-10, 1e-12), (pkg.PREC_MIXED, 1e-8, 1e-10)):
            ev, rs, nc, info = h.eigsh_batch(Js, 1.0, 0.0, nev=10, precision=prec)
            assert nc.min() == 10
            for k, r in enumerate(recs):
                ref = np.array(reference_lowest(r))
                assert len(ref) == 10
                err = _rel(ev[k], ref, atol, tol)
                assert err < tol, (n, r["J"], prec, err)


def test_batched_equals_single_solves(pkg):
    m, n = 8, 7
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    Js = np.array([0.02, 0.08, 0.2, 0.3])
    mus = np.array([0.0, 0.1, 0.2, 0.3])
    evb, _, _, _ = h.eigsh_batch(Js, 1.0, mus, nev=6)
    for k in range(len(Js)):
        ev, _, _, _ = h.eigsh(Js[k], 1.0, mus[k], nev=6)
        assert _rel(evb[k], ev) < 1e-10


def test_mu_is_a_constant_shift(pkg):
    m, n = 8, 6
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    e0, _, _, _ = h.eigsh_batch(np.array([0.1, 0.1]), 1.0, np.array([0.0, 0.7]), nev=4)
    np.testing.assert_allclose(e0[1], e0[0] - 0.7 * n, rtol=1e-10)


def test_phase_map_density_and_compressibility(pkg):
    m = 6
    sectors = [4, 5, 6, 7, 8]
    Js = np.array([0.02, 0.1, 0.25])
    e0 = []
    for n in sectors:
        h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
        ev, _, _, _ = h.eigsh_batch(Js, 1.0, 0.0, nev=2)
        e0.append(ev[:, 0])
    e0 = np.array(e0)
    mu = np.linspace(0.0, 3.0, 64)
    dens, kap = pkg.Analysis.phase_map(m, sectors[0], e0, mu)
    # host check of the same definitions
    for j in range(len(Js)):
        for k, muv in enumerate(mu):
            best = np.argmin(e0[:, j] - muv * np.array(sectors))
            assert dens[j, k] == sectors[best] / m
        d = dens[j]
        ref = np.gradient(d, mu, edge_order=1)
        np.testing.assert_allclose(kap[j, 1:-1], (d[2:] - d[:-2]) / (mu[2:] - mu[:-2]))
    # density grows with mu; the J = 0.02 row shows a Mott plateau at n/m = 1
    assert np.all(np.diff(dens, axis=1) >= 0)
    assert np.any(dens[0] == 1.0)


def test_spdm_matches_oracle(pkg, orc):
    m, n = 7, 6
    lists = chain_lists(m)
    h = pkg.Hamiltonian(pkg.Basis(m, n), lists)
    ev, _, vec, _ = h.eigsh(0.2, 1.0, 0.0, nev=2, vectors=True, order=pkg.ORDER_LEX)
    occ = orc.lex_states(m, n)
    rho_o = orc.spdm(occ, np.ascontiguousarray(vec[:, 0]))
    rho = h.spdm(vec[:, 0], order=pkg.ORDER_LEX)
    np.testing.assert_allclose(rho, rho_o, rtol=1e-10, atol=1e-12)
    assert abs(np.trace(rho) - n) < 1e-9
    # reference-order input gives the same matrix
    evr, _, vecr, _ = h.eigsh(0.2, 1.0, 0.0, nev=2, vectors=True)
    rho_r = h.spdm(vecr[:, 0])
    np.testing.assert_allclose(np.abs(rho_r), np.abs(rho), rtol=1e-8, atol=1e-10)
    cf = orc.condensate_fraction(rho_o)
    assert 0.0 < cf <= 1.0
    assert abs(pkg.Analysis.coherence(rho) - orc.coherence(rho_o)) < 1e-10


def test_mixed_matches_fp64_pure_relative_on_the_bench_grid(pkg):
    # every eigenvalue of the benchmark grid (m = 10, n = 8..12, 64 J in
    # (0, 0.3], lowest 10) from the mixed-precision batch within 1e-8 of the
    # FP64 batch relative to its own magnitude, with no absolute floor (the
    # levels near zero are the hardest case)
    Js = 0.3 * (np.arange(64) + 1) / 64
    lists = chain_lists(10)
    hams = [pkg.Hamiltonian(pkg.Basis(10, n), lists) for n in (8, 9, 10, 11, 12)]
    ev_m, _, nc_m, _ = pkg.eigsh_sectors(hams, Js, 1.0, 0.0, nev=10, precision=pkg.PREC_MIXED)
    ev_d, _, nc_d, _ = pkg.eigsh_sectors(hams, Js, 1.0, 0.0, nev=10, precision=pkg.PREC_FP64)
    assert nc_m.min() == 10 and nc_d.min() == 10
    rel = np.abs(ev_m - ev_d) / np.abs(ev_d)
    assert rel.max() < 1e-8, (rel.max(), np.unravel_index(rel.argmax(), rel.shape))
