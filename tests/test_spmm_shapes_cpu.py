"""CPU: the launch shapes the autotuner of the sparse product chooses from.

Every candidate must be a shape the library has a kernel for (lanes a power of
two <= 32 dividing the width, 1 or 4 columns per lane, 2 only with 32 lanes;
or, for stored CSR at even widths, -4 / -2: that many adjacent columns per
lane on 2..32 lanes), the default shape must come first and equal the fixed
rule the product used before it had a tuner, and no shape may repeat.  No GPU
is touched: these are host-only entry points."""
import ctypes as C

import pytest


def default_shape(nvec, matrix_free=False):
    if matrix_free:
        # one warp per row, columns masked: 1, 2 or 4 columns per lane per pass
        cpl = (nvec + 31) // 32
        return (32, 1 if cpl == 1 else 2 if cpl == 2 else 4, 0)
    L = 1
    while L < 32 and 2 * L <= nvec and nvec % (2 * L) == 0:
        L *= 2
    cpl = nvec // L
    cw = 4 if cpl > 2 else cpl
    if L < 32 and cw == 2:
        cw = 4
    return (L, cw, 0)


@pytest.mark.parametrize("nvec", [1, 2, 3, 4, 6, 10, 12, 20, 32, 60, 63, 64, 96, 126, 128, 256, 512])
def test_candidates_valid_default_first_unique(pkg, nvec):
    cands = pkg.spmm_candidates(nvec)
    assert cands[0] == default_shape(nvec)
    assert len(set(cands)) == len(cands)
    assert 1 <= len(cands) <= 16
    for lanes, cw, grid in cands:
        if cw < 0:  # contiguous columns: -cw adjacent columns per lane, masked
            assert cw in (-2, -4) and nvec % -cw == 0 and nvec >= 4
            assert lanes in (2, 4, 8, 16, 32)
        else:
            assert lanes in (1, 2, 4, 8, 16, 32) and nvec % lanes == 0
            assert cw in (1, 4) or (cw == 2 and lanes == 32)
        assert grid in (0, -1)
    # the contiguous-column shapes exist exactly at even widths >= 4
    assert any(c[1] < 0 for c in cands) == (nvec >= 4 and nvec % 2 == 0)
    # both grid rules for the default lane count
    assert (cands[0][0], cands[0][1], -1) in cands


@pytest.mark.parametrize("nvec", [1, 2, 3, 12, 28, 60, 63, 64, 100, 128, 512])
def test_matrix_free_candidates(pkg, nvec):
    cands = pkg.spmm_candidates(nvec, True)
    assert cands[0] == default_shape(nvec, True)
    assert len(set(cands)) == len(cands) and len(cands) <= 12
    for lanes, cw, grid in cands:
        # 32 lanes is the warp-per-row kernel, at any width; fewer lanes must divide it
        assert lanes == 32 or nvec % lanes == 0
        assert cw in (1, 4) or (cw == 2 and lanes == 32)
    # the per-lane kernels stay candidates
    assert any(c[0] < 32 for c in cands) or nvec == 1


def test_candidates_cover_fewer_lanes(pkg):
    cands = pkg.spmm_candidates(128)
    lanes = {c[0] for c in cands if c[1] > 0}
    assert lanes == {32, 16, 8}
    assert {c[0] for c in cands if c[1] < 0} == {32, 16} and all(c[1] == -4 for c in cands if c[1] < 0)
    # odd multiples of two (batches with an odd number of block-2 solves):
    # 1 or 2 lanes per row with strided columns, or 32 / 16 lanes with two
    # adjacent columns each
    cands = pkg.spmm_candidates(126)
    assert {c[0] for c in cands if c[1] > 0} == {2, 1}
    assert {(c[0], c[1]) for c in cands if c[1] < 0} == {(32, -2), (16, -2)}


def test_candidates_argument_errors(pkg):
    lib = pkg.load()
    buf = (pkg.bh_spmm_shape * 2)()
    n = C.c_int()
    assert lib.bh_spmm_candidates(0, 0, buf, 2, C.byref(n)) == pkg.BH_ERR_ARG
    assert lib.bh_spmm_candidates(128, 0, buf, 2, C.byref(n)) == pkg.BH_ERR_ARG  # capacity
    assert b"capacity" in lib.bh_last_error()


def test_tuning_table_starts_empty_and_resets(pkg):
    pkg.spmm_tuning_reset()
    assert pkg.spmm_tuning_table() == []
