"""GPU: the large sector configurations pinned to the reference.

* plain FP64, 1D periodic m=n=12 (D=1 352 078), J=0.05, U=1, mu=0.6, the
  lowest 10: against the reference's own Op::IRLM_eigen (Spectra
  GenEigsSolver, operator.cpp:22-33) run on the model Hamiltonian, 1e-10
  relative;
* the reference's fixed_set_basis column order at m=n=12, m=n=14 (prime
  products up to 76 bits) and m=16, n=12, as SHA-256 of col_of_lex;
* mixed precision, 1D periodic m=n=14 (D=20 058 300, stored CSR), lowest 6,
  80-vector Krylov basis: against the FP64 path on two of the eight J points,
  1e-8 relative (no absolute floor);
* matrix-free 4x4 periodic torus, n=12 (D=17 383 860), block 4, lowest 4,
  60-vector Krylov basis: mixed against FP64 on two J points at 1e-8, and the
  ground-state density and compressibility over the sectors n=11..13 within
  the error that 1e-8 relative eigenvalues allow.

The golden values come from tests/golden/make_golden.py --large (the
reference's sources compiled by oracle/Makefile)."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import chain_lists

pytestmark = pytest.mark.gpu

GOLDEN_LARGE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                            "reference_golden_large.json")


@pytest.fixture(scope="module")
def golden_large():
    with open(GOLDEN_LARGE) as f:
        return json.load(f)


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def square_lists(pkg, m):
    nb = pkg.Neighbours(m)
    nb.square_neighbours(True)
    return nb.getNeighbours()


@pytest.mark.parametrize("m,n", [(12, 12), (14, 14), (16, 12)])
def test_large_basis_order_matches_reference(pkg, golden_large, m, n):
    rec = golden_large["basis"][f"{m},{n}"]
    b = pkg.Basis(m, n)
    assert b.D == rec["D"]
    col_of_lex, lex_of_col = b.orders()
    assert _sha(col_of_lex.astype("<i4")) == rec["col_of_lex_sha256"]
    assert lex_of_col[:16].tolist() == rec["first_cols_lex"]
    tags, _ = b.copy(tags=True, basis=False)
    assert _sha(tags.astype("<f8")) == rec["tags_sha256"]


def test_plain_m12_matches_reference_irlm(pkg, golden_large):
    rec = golden_large["irlm"]["m12n12"]
    ref = np.array(rec["evals_lowest_from_nev_plus_2"])
    h = pkg.Hamiltonian(pkg.Basis(12, 12), chain_lists(12))
    ev, rs, _, info = h.eigsh(rec["J"], rec["U"], rec["mu"], nev=10)
    assert info.nconv == 10
    rel = np.abs(ev - ref) / np.abs(ref)
    assert rel.max() < 1e-10, rel
    # the drop-in Op::IRLM_eigen on the assembled sparse matrix: the same
    # values, in the reference's result order (descending |lambda|)
    vals, vecs = pkg.Op.IRLM_eigen(h.csr(rec["J"], rec["U"], rec["mu"]), 10)
    want = ref[np.argsort(-np.abs(ref), kind="stable")]
    assert np.max(np.abs(vals.real - want) / np.abs(want)) < 1e-10
    assert np.all(vals.imag == 0) and vecs.shape == (h.D, 10)


def test_mixed_m14_matches_fp64(pkg):
    m = n = 14
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    Js = np.linspace(0.02, 0.2, 8)[[0, 7]]
    opts = dict(nev=6, ncv=80, block=2)
    ev_m, rs_m, nc_m, _ = h.eigsh_batch(Js, 1.0, 0.0, precision=pkg.PREC_MIXED, **opts)
    ev_d, rs_d, nc_d, _ = h.eigsh_batch(Js, 1.0, 0.0, precision=pkg.PREC_FP64, **opts)
    assert nc_m.min() == 6 and nc_d.min() == 6
    rel = np.abs(ev_m - ev_d) / np.abs(ev_d)
    assert rel.max() < 1e-8, rel


def _e0_sectors(pkg, lists, sectors, J, prec):
    out = []
    for n in sectors:
        h = pkg.Hamiltonian(pkg.Basis(16, n), lists, matrix_free=True)
        ev, _, nc, _ = h.eigsh_batch(J, 1.0, 0.0, nev=4, block=4, ncv=60, precision=prec)
        assert nc.min() == 4
        out.append(ev)
        del h
    return np.array(out)  # [sector, J, nev]


def test_matrix_free_4x4_n12_mixed_matches_fp64(pkg):
    lists = square_lists(pkg, 16)
    Js = np.array([0.02, 0.1])
    e_m = _e0_sectors(pkg, lists, [12], Js, pkg.PREC_MIXED)[0]
    e_d = _e0_sectors(pkg, lists, [12], Js, pkg.PREC_FP64)[0]
    rel = np.abs(e_m - e_d) / np.abs(e_d)
    assert rel.max() < 1e-8, rel


def test_matrix_free_4x4_density_compressibility(pkg):
    # ground-state energies E0(n) of the sectors n = 11, 12, 13 at mu = 0;
    # the density map rho(mu) = n*/m with n* = argmin_n [E0(n) - mu n] and its
    # finite-difference compressibility on the mu grid, plus the sector's
    # inverse compressibility (charge gap) E0(n+1) + E0(n-1) - 2 E0(n)
    lists = square_lists(pkg, 16)
    sectors = [11, 12, 13]
    J = np.array([0.06])
    e_m = _e0_sectors(pkg, lists, sectors, J, pkg.PREC_MIXED)[:, :, 0]
    e_d = _e0_sectors(pkg, lists, sectors, J, pkg.PREC_FP64)[:, :, 0]
    assert np.all(np.abs(e_m - e_d) <= 1e-8 * np.abs(e_d))
    gap_m = e_m[2] + e_m[0] - 2 * e_m[1]
    gap_d = e_d[2] + e_d[0] - 2 * e_d[1]
    bound = 1e-8 * (np.abs(e_d[2]) + np.abs(e_d[0]) + 2 * np.abs(e_d[1]))
    assert np.all(np.abs(gap_m - gap_d) <= bound), (gap_m, gap_d)
    assert np.all(gap_d > 0)  # a stable sector: E0 convex in n
    mu = np.linspace(0.0, 3.0, 64)
    dens_m, kap_m = pkg.Analysis.phase_map(16, sectors[0], e_m, mu)
    dens_d, kap_d = pkg.Analysis.phase_map(16, sectors[0], e_d, mu)
    # the maps are piecewise constant in mu: equal unless a grid point lies
    # within the eigenvalue error of a transition, which the check rules out
    edges = [e_d[k + 1, 0] - e_d[k, 0] for k in range(len(sectors) - 1)]
    if all(np.min(np.abs(mu - e)) > 1e-6 for e in edges):
        assert np.array_equal(dens_m, dens_d)
        np.testing.assert_allclose(kap_m, kap_d, rtol=0, atol=1e-8)
    # host restatement of the definition on the FP64 energies
    for k, muv in enumerate(mu):
        best = int(np.argmin(e_d[:, 0] - muv * np.array(sectors)))
        assert dens_d[0, k] == sectors[best] / 16
