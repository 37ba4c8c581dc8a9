"""CPU: the C-ABI library loads, exports every declared symbol, and its host-only
entry points (lattices, dimension, gap ratios, argument checks) behave like the
reference's."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "bh_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(bh_[a-z0-9_]+)\s*\(", txt)))


def test_exports_every_declared_symbol(pkg):
    lib = pkg.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(pkg.EXPORTS)


def test_version_and_error_string(pkg):
    lib = pkg.load()
    assert lib.bh_version() >= 10000
    assert isinstance(lib.bh_last_error(), bytes)


def test_chain_matches_reference(pkg, golden):
    for key, rec in golden["neighbours"].items():
        kind, m, closed = key.split(",")
        if kind != "chain":
            continue
        nb = pkg.Neighbours(int(m))
        nb.chain_neighbours(bool(int(closed)))
        off, flat = pkg.flatten_neighbours(nb.getNeighbours())
        assert off.tolist() == rec["off"]
        assert flat[: off[-1]].tolist() == rec["nbr"]


def test_square_and_cube_are_the_intended_lattices(pkg, golden):
    # the reference returns empty lists (shadowed local); we return the lattice
    for key, rec in golden["neighbours"].items():
        kind, m, closed = key.split(",")
        if kind == "chain":
            continue
        assert rec["nbr"] == []
    nb = pkg.Neighbours(16)
    nb.square_neighbours(True)
    lists = nb.getNeighbours()
    assert all(len(l) == 4 for l in lists)
    for i, l in enumerate(lists):
        r, c = divmod(i, 4)
        assert sorted(l) == sorted([r * 4 + (c - 1) % 4, r * 4 + (c + 1) % 4,
                                    ((r - 1) % 4) * 4 + c, ((r + 1) % 4) * 4 + c])
    nb = pkg.Neighbours(27)
    nb.cube_neighbours(True)
    assert all(len(l) == 6 for l in nb.getNeighbours())
    nb = pkg.Neighbours(9)
    nb.square_neighbours(False)
    assert sum(len(l) for l in nb.getNeighbours()) == 2 * 12


def test_lattice_errors_mirror_reference(pkg):
    with pytest.raises(ValueError, match="perfect square"):
        pkg.Neighbours(10).square_neighbours()
    with pytest.raises(ValueError, match="perfect cube"):
        pkg.Neighbours(10).cube_neighbours()


def test_dimension(pkg, orc):
    for m, n in [(1, 0), (3, 3), (8, 8), (10, 12), (12, 12), (14, 14), (16, 12)]:
        assert pkg.BH.dimension(m, n) == orc.dimension(m, n)
    assert pkg.BH.dimension(12, 12) == 1352078
    assert pkg.BH.dimension(14, 14) == 20058300
    assert pkg.BH.dimension(16, 12) == 17383860


def test_gap_ratios_bitwise_like_reference(pkg, golden):
    ev = np.array(golden["irlm"]["m8n8"]["evals_reference_order"])
    r = pkg.Analysis.gap_ratios(ev, len(ev))
    assert r.tolist() == golden["gap_ratios_m8n8"]


def test_coherence_like_reference(pkg, golden):
    rho = np.array(golden["coherence"]["rho"])
    assert pkg.Analysis.coherence(rho) == pytest.approx(golden["coherence"]["value"], rel=1e-14)


def test_argument_errors_without_gpu(pkg):
    lib = pkg.load()
    d = C.c_int64()
    assert lib.bh_dimension(0, 3, C.byref(d)) == pkg.BH_ERR_ARG
    assert b"m must be" in lib.bh_last_error()
    h = C.c_void_p()
    assert lib.bh_basis_create(26, 3, C.byref(h)) == pkg.BH_ERR_ARG
    assert b"primes" in lib.bh_last_error()
