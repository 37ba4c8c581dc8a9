import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_golden.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as g

    p = g.load_package()
    p.load()
    return p


@pytest.fixture(scope="session")
def orc():
    import oracle

    return oracle.Oracle()


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def chain_lists(m, closed=True):
    lists = [[] for _ in range(m)]
    for i in range(m):
        if i > 0:
            lists[i].append(i - 1)
        if i < m - 1:
            lists[i].append(i + 1)
    if closed:
        lists[0].append(m - 1)
        lists[m - 1].append(0)
    return lists


def oracle_H(orc, m, n, lists, order="reference"):
    """Oracle T (CSR), V and the order maps for one sector."""
    import numpy as np

    occ = orc.lex_states(m, n)
    col_of_lex, lex_of_col = orc.reference_order(occ)
    off = np.zeros(m + 1, np.int32)
    flat = []
    for i, l in enumerate(lists):
        flat += l
        off[i + 1] = len(flat)
    flat = np.array(flat if flat else [0], np.int32)
    if order == "reference":
        rp, ci, tv = orc.build_T(occ, off, flat, lex_of_col, col_of_lex)
        vd = orc.diag_V(occ, lex_of_col)
    else:
        rp, ci, tv = orc.build_T(occ, off, flat)
        vd = orc.diag_V(occ)
    return occ, col_of_lex, lex_of_col, rp, ci, tv, vd


def reference_lowest(rec):
    """The reference's lowest nev eigenvalues with multiplicity: its run with
    nev + 2 wanted values (see tests/golden/make_golden.py), else its nev run."""
    v = rec.get("evals_lowest_from_nev_plus_2") or rec["evals_sorted"]
    return v
