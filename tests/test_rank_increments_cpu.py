"""CPU: the rank arithmetic of the warp-per-row matrix-free product.

The product ranks the state reached by a hop i -> j (one boson from site i to
site j) without a search: with the rank table RT[t][s] = C(s + m - t - 2,
m - t - 1) (t <= m - 2), the lexicographic index of a state is
sum_t RT[t][s_t] with the suffix sums s_t = sum_{u > t} n_u, and a hop only
moves the suffix sums between i and j by one.  Per row the kernel forms the
per-site increments
    a_t = RT[t][s_t + 1] - RT[t][s_t]   (s_t < n),
    b_t = RT[t][s_t] - RT[t][s_t - 1]   (s_t > 0),
their exclusive prefix sums P_a, P_b over sites in uint32 (modulo 2^32), and
takes
    r' = r + int32(P_a[j] - P_a[i])   (i < j),
    r' = r - int32(P_b[i] - P_b[j])   (i > j).
These tests restate that arithmetic in numpy and check it against the
oracle's enumeration of every sector state (the lexicographic order of the
reference's init_lexicographic, hamiltonian.cpp:60-85) for every hop, and on
sampled states of the large 4x4, n = 12 sector."""
from math import comb

import numpy as np
import pytest


def rank_table(m, n):
    return np.array([[comb(s + m - t - 2, m - t - 1) for s in range(n + 1)] for t in range(m - 1)],
                    dtype=np.int64)


def prefix_increments(occ, RT, n):
    """P_a, P_b (uint32, exclusive prefix sums over sites) of every row of occ."""
    D, m = occ.shape
    o = occ.astype(np.int64)
    suf = np.cumsum(o[:, ::-1], axis=1)[:, ::-1] - o  # s_t = sum_{u > t} n_u
    a = np.zeros((D, m), np.uint32)
    b = np.zeros((D, m), np.uint32)
    for t in range(m - 1):
        st = suf[:, t]
        up = st < n
        dn = st > 0
        a[up, t] = (RT[t, st[up] + 1] - RT[t, st[up]]).astype(np.uint32)
        b[dn, t] = (RT[t, st[dn]] - RT[t, st[dn] - 1]).astype(np.uint32)
    pa = (np.cumsum(a, axis=1, dtype=np.uint32) - a).astype(np.uint32)
    pb = (np.cumsum(b, axis=1, dtype=np.uint32) - b).astype(np.uint32)
    return suf, pa, pb


def hop_rank(r, pa, pb, i, j):
    if i < j:
        return r + (pa[:, j] - pa[:, i]).astype(np.uint32).view(np.int32).astype(np.int64)
    return r - (pb[:, i] - pb[:, j]).astype(np.uint32).view(np.int32).astype(np.int64)


@pytest.mark.parametrize("m,n", [(2, 3), (3, 3), (4, 5), (6, 4), (8, 6), (9, 9), (16, 3)])
def test_hop_ranks_match_the_enumeration(orc, m, n):
    occ = orc.lex_states(m, n)
    D = occ.shape[0]
    RT = rank_table(m, n)
    suf, pa, pb = prefix_increments(occ, RT, n)
    r = np.arange(D, dtype=np.int64)
    # the rank of each state itself
    assert np.array_equal(sum(RT[t, suf[:, t]] for t in range(m - 1)), r)
    index = {tuple(row): k for k, row in enumerate(occ.tolist())}
    for i in range(m):
        for j in range(m):
            if i == j:
                continue
            rows = np.nonzero(occ[:, i] >= 1)[0]
            got = hop_rank(r[rows], pa[rows], pb[rows], i, j)
            moved = occ[rows].astype(np.int64)
            moved[:, i] -= 1
            moved[:, j] += 1
            want = np.array([index[tuple(x)] for x in moved.tolist()])
            assert np.array_equal(got, want), (m, n, i, j)


def test_hop_ranks_on_the_large_torus_sector():
    # 4x4 torus, n = 12 (D = 17 383 860): sampled states, exact Python ranks
    m, n = 16, 12
    RT = rank_table(m, n)
    rng = np.random.default_rng(7)
    occ = np.zeros((400, m), np.int64)
    for k in range(400):
        for _ in range(n):
            occ[k, rng.integers(m)] += 1

    def exact_rank(row):
        s, r = 0, 0
        for t in range(m - 1, -1, -1):
            if t <= m - 2:
                r += comb(s + m - t - 2, m - t - 1)
            s += int(row[t])
        return r

    r = np.array([exact_rank(x) for x in occ], np.int64)
    assert r.max() < comb(n + m - 1, n)
    suf, pa, pb = prefix_increments(occ, RT, n)
    for i in range(m):
        for j in range(m):
            if i == j:
                continue
            rows = np.nonzero(occ[:, i] >= 1)[0]
            got = hop_rank(r[rows], pa[rows], pb[rows], i, j)
            moved = occ[rows].copy()
            moved[:, i] -= 1
            moved[:, j] += 1
            want = np.array([exact_rank(x) for x in moved])
            assert np.array_equal(got, want), (i, j)
