"""CPU: the concurrent solves the reference arm times (`Oracle.irlm_wave`:
points solved `groups` at a time, each on `inner` threads) give the
single-point restatement of Op::IRLM_eigen's eigenvalues.  Below 5e4 states
the row loops stay serial, so any grouping is bit-identical; above it the row
loops are split over the inner threads with chunked sums in a fixed order."""
import numpy as np
import pytest

from conftest import chain_lists


def _sector(orc, m, n):
    lists = chain_lists(m)
    off = np.zeros(m + 1, np.int32)
    flat = []
    for i, l in enumerate(lists):
        flat += l
        off[i + 1] = len(flat)
    flat = np.array(flat, np.int32)
    occ = orc.lex_states(m, n)
    col_of_lex, lex_of_col = orc.reference_order(occ)
    rp, ci, tv = orc.build_T(occ, off, flat, lex_of_col, col_of_lex)
    return rp, ci, tv, orc.diag_V(occ, lex_of_col)


def test_wave_groups_equal_single_solves(orc):
    m = n = 8
    rp, ci, tv, vd = _sector(orc, m, n)
    Js = np.array([0.05, 0.1, 0.17, 0.23])
    single = np.stack([np.sort(orc.irlm(rp, ci, tv, vd, n, J, 1.0, 0.3, nev=6)[0]) for J in Js])
    for groups, inner in ((1, 1), (2, 1), (4, 1), (2, 2)):
        ev, nc = orc.irlm_wave(rp, ci, tv, vd, n, Js, 1.0, 0.3, nev=6, groups=groups, inner=inner)
        assert np.all(nc == 6)
        assert np.array_equal(np.sort(ev, axis=1), single), (groups, inner)


def test_wave_with_parallel_row_loops_matches_serial(orc):
    # D = C(19, 9) = 92 378 > 5e4: the inner threads split the row loops
    m, n = 11, 9
    rp, ci, tv, vd = _sector(orc, m, n)
    J = np.array([0.2])
    e1, n1 = orc.irlm_wave(rp, ci, tv, vd, n, J, 1.0, 0.0, nev=4, groups=1, inner=1)
    e4, n4 = orc.irlm_wave(rp, ci, tv, vd, n, J, 1.0, 0.0, nev=4, groups=1, inner=4)
    assert n1[0] == 4 and n4[0] == 4
    assert np.max(np.abs(np.sort(e4[0]) - np.sort(e1[0])) / np.abs(np.sort(e1[0]))) < 1e-12
