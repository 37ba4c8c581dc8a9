"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own exact-path code, compiled from its sources by
oracle/Makefile into oracle/_ref/libbhref.so:
  - BH::fixed_set_basis / init_lexicographic (hamiltonian.cpp:60-149):
    reference column order and tags (tags recorded bit-exactly as hex);
  - Neighbours (neighbours.cpp:21-120): the lists the reference returns;
  - Op::IRLM_eigen (operator.cpp:22-33, Spectra GenEigsSolver) and
    Op::exact_eigen on the Bose-Hubbard Hamiltonian with the physics of the
    reference's model definition (H = -J sum b+b + U/2 sum n(n-1) - mu sum n),
    assembled in the reference's column order by the CPU oracle (the
    reference's own builder is not a valid Hamiltonian: it loops over
    neighbour slots and reads out of bounds);
  - Analysis::gap_ratios and Analysis::coherence;
  - Analysis::SCMF (analysis.cpp:111-178), the mean-field order parameter.
Usage:  python tests/golden/make_golden.py [--quick | --scmf-only | --large]
(--large writes reference_golden_large.json: basis orders at m=n=12, m=n=14
and m=16, n=12, and the reference's IRLM at m=n=12; see large_cases).
The reference tree is read from BH_REFERENCE_TREE (default /root/reference).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as orc  # noqa: E402

REF_TREE = os.environ.get("BH_REFERENCE_TREE", "/root/reference")


def hexs(a):
    return [float(x).hex() for x in a]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ref_order_from_reference(ref, m, n):
    """col_of_lex from the reference's own basis matrix."""
    tags, basis = ref.fixed_set_basis(m, n)  # basis[c] = occupation at column c
    lex = ref.init_lexicographic(m, n)
    index = {tuple(row.astype(int)): i for i, row in enumerate(lex)}
    lex_of_col = np.array([index[tuple(row.astype(int))] for row in basis], np.int32)
    col_of_lex = np.empty_like(lex_of_col)
    col_of_lex[lex_of_col] = np.arange(len(lex_of_col), dtype=np.int32)
    return tags, col_of_lex, lex_of_col


def chain(m):
    off = np.zeros(m + 1, np.int32)
    nb = []
    lists = [[] for _ in range(m)]
    for i in range(m):
        if i > 0:
            lists[i].append(i - 1)
        if i < m - 1:
            lists[i].append(i + 1)
    lists[0].append(m - 1)
    lists[m - 1].append(0)
    for i, l in enumerate(lists):
        nb += l
        off[i + 1] = len(nb)
    return off, np.array(nb, np.int32)


def hamiltonian_ref_order(o, m, n, J, U, mu, nbr=None):
    occ = o.lex_states(m, n)
    col_of_lex, lex_of_col = o.reference_order(occ)
    off, nb = nbr if nbr is not None else chain(m)
    rp, ci, tv = o.build_T(occ, off, nb, lex_of_col, col_of_lex)
    vd = o.diag_V(occ, lex_of_col)
    return o.full_csr(rp, ci, tv, vd, n, J, U, mu)


def main(quick: bool):
    orc.build()
    if orc.build_ref(REF_TREE) is None:
        raise SystemExit("reference tree not available")
    o = orc.Oracle()
    ref = orc.Reference()
    out = {"generator": "tests/golden/make_golden.py", "reference": "Maximilien-Hantonne/Bose-Hubbard-Phase-Transition"}

    # ---- basis ----
    small = [(1, 0), (1, 3), (2, 0), (2, 3), (3, 3), (4, 4), (5, 3), (3, 5), (6, 6), (4, 7), (8, 8)]
    hashed = [(10, 10), (12, 6), (7, 9), (10, 8), (10, 12)]
    basis = {}
    for m, n in small + hashed:
        tags, col_of_lex, lex_of_col = ref_order_from_reference(ref, m, n)
        rec = {"m": m, "n": n, "D": int(len(tags)),
               "col_of_lex_sha256": sha(col_of_lex.astype("<i4")),
               "tags_sha256": sha(tags.astype("<f8"))}
        if (m, n) in small:
            rec["col_of_lex"] = col_of_lex.tolist()
            rec["tags_hex"] = hexs(tags)
        basis[f"{m},{n}"] = rec
    out["basis"] = basis

    # ---- neighbours as the reference returns them ----
    nbrs = {}
    for kind, name, ms in [(1, "chain", [2, 3, 4, 5, 8]), (2, "square", [4, 9, 16]), (3, "cube", [8, 27])]:
        for m in ms:
            for closed in (True, False):
                off, nb = ref.neighbours(kind, m, closed)
                nbrs[f"{name},{m},{int(closed)}"] = {"off": off.tolist(), "nbr": nb.tolist()}
    out["neighbours"] = nbrs

    # ---- eigenvalues: reference IRLM on the model Hamiltonian ----
    cases = [
        ("m8n8", 8, 8, 0.1, 1.0, 0.5, 10),
        ("m6n6", 6, 6, 0.1, 1.0, 0.5, 6),
        ("m5n5_J0.2", 5, 5, 0.2, 1.0, 0.0, 6),
        ("m6n4_J0.3", 6, 4, 0.3, 1.0, 0.25, 8),
        ("m10n8", 10, 8, 0.15, 1.0, 0.0, 10),
    ]
    if not quick:
        cases += [("m10n10", 10, 10, 0.15, 1.0, 0.0, 10)]
    # batched grid points: m = 10, sectors 8..12, J_b = 0.3 (b + 1) / 64
    grid_b = [3, 15, 31, 47, 63] if not quick else [31]
    grid_n = [8, 9, 10, 11, 12] if not quick else [8, 9]
    for n in grid_n:
        for b in grid_b:
            cases.append((f"grid_n{n}_b{b}", 10, n, 0.3 * (b + 1) / 64, 1.0, 0.0, 10))

    def run(case):
        name, m, n, J, U, mu, nev = case
        H = hamiltonian_ref_order(o, m, n, J, U, mu)
        t0 = time.time()
        try:
            re, im = ref.irlm(H, nev)
            ok = True
        except RuntimeError:
            re, im, ok = np.zeros(0), np.zeros(0), False
        dt = time.time() - t0
        rec = {"m": m, "n": n, "J": J, "U": U, "mu": mu, "nev": nev, "converged": ok,
               "evals_reference_order": re.tolist(), "imag_max": float(np.abs(im).max()) if len(im) else 0.0,
               "evals_sorted": sorted(re.tolist()), "seconds": dt, "nnz": int(H.nnz)}
        # The reference's single-vector IRLM can return the level above a
        # degenerate pair that straddles the edge of the wanted window
        # instead of the pair's second copy.  Running it with two more wanted
        # values puts the edge inside the window: its lowest nev values are
        # the true lowest nev with multiplicity.
        try:
            re2, _ = ref.irlm(H, nev + 2)
            rec["evals_lowest_from_nev_plus_2"] = sorted(re2.tolist())[:nev]
        except RuntimeError:
            rec["evals_lowest_from_nev_plus_2"] = []
        return name, rec

    eig = {}
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        for name, rec in ex.map(run, cases):
            eig[name] = rec
            print(f"{name}: conv={rec['converged']} t={rec['seconds']:.1f}s E0={rec['evals_sorted'][:1]}", flush=True)
    out["irlm"] = eig

    # ---- dense spectra (Op::exact_eigen) for small sectors ----
    dense = {}
    for m, n, J, U, mu in [(4, 4, 0.1, 1.0, 0.5), (5, 3, 0.3, 1.0, 0.2), (3, 3, 0.0, 1.0, 0.5), (4, 3, 0.25, 0.0, 0.0)]:
        H = hamiltonian_ref_order(o, m, n, J, U, mu)
        dense[f"{m},{n},{J},{U},{mu}"] = ref.exact_eigen(H).tolist()
    out["exact_eigen"] = dense

    # ---- analysis helpers ----
    ev = np.array(eig["m8n8"]["evals_reference_order"])
    out["gap_ratios_m8n8"] = ref.gap_ratios(ev).tolist()
    rng = np.random.RandomState(7)
    rho = rng.rand(5, 5)
    rho = rho + rho.T
    out["coherence"] = {"rho": rho.tolist(), "value": ref.coherence(rho)}

    out["scmf"] = scmf_cases(ref)

    path = os.path.join(HERE, "reference_golden.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, os.path.getsize(path), "bytes")


def scmf_cases(ref):
    """Analysis::SCMF (src/analysis.cpp:111-178) on a (mu, J) grid with fixed
    seeds psi0 (the reference draws psi0 from std::random_device)."""
    cases = []
    rng = np.random.RandomState(11)
    for q, prec in [(1, 6), (2, 8), (4, 7)]:
        for mu in [0.1, 0.45, 0.9, 1.5, 2.3, 3.1, 3.8]:
            for J in [0.01, 0.04, 0.09, 0.16, 0.24]:
                psi0 = float(rng.uniform(0.05, 1.0))
                cases.append({"mu": mu, "J": J, "q": q, "psi0": psi0, "precision": prec,
                              "psi": ref.scmf(mu, J, q, psi0, prec)})
    return cases


def update_scmf_only():
    """Adds or replaces only the scmf section of the committed fixture."""
    orc.build_ref()
    ref = orc.Reference()
    path = os.path.join(HERE, "reference_golden.json")
    with open(path) as f:
        out = json.load(f)
    out["scmf"] = scmf_cases(ref)
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, os.path.getsize(path), "bytes")


def large_cases():
    """Golden values at the sizes of the large workloads, written to
    reference_golden_large.json:
      - the reference's own fixed_set_basis order at m=n=12, m=n=14 (76-bit
        prime products) and m=16, n=12 (the 4x4 torus sector), checked here
        state by state against the oracle's order and recorded as SHA-256 of
        col_of_lex (int32 little-endian) and of the tags;
      - the reference's Op::IRLM_eigen (Spectra, single thread) on the model
        Hamiltonian at m=n=12, J=0.05, U=1, mu=0.6, nev=10, and with nev+2
        (whose lowest 10 values are the lowest 10 with multiplicity).
    The IRLM at D=1 352 078 takes about 15 minutes per run."""
    orc.build()
    if orc.build_ref(REF_TREE) is None:
        raise SystemExit("reference tree not available")
    o = orc.Oracle()
    ref = orc.Reference()
    out = {"generator": "tests/golden/make_golden.py --large",
           "reference": "Maximilien-Hantonne/Bose-Hubbard-Phase-Transition"}
    basis = {}
    for m, n in [(12, 12), (14, 14), (16, 12)]:
        t0 = time.time()
        tags, rbasis = ref.fixed_set_basis(m, n)
        occ = o.lex_states(m, n)
        lex_ref = ref.init_lexicographic(m, n)
        assert np.array_equal(lex_ref, occ.astype(np.float64)), (m, n, "lexicographic order")
        del lex_ref
        col_of_lex, lex_of_col = o.reference_order(occ)
        assert np.array_equal(rbasis, occ[lex_of_col].astype(np.float64)), (m, n, "column order")
        del rbasis
        otags = o.tags(occ)
        basis[f"{m},{n}"] = {
            "m": m, "n": n, "D": int(len(tags)),
            "col_of_lex_sha256": sha(col_of_lex.astype("<i4")),
            "tags_sha256": sha(tags.astype("<f8")),
            "oracle_tags_equal": bool(np.array_equal(otags[lex_of_col], tags)),
            "first_cols_lex": lex_of_col[:16].tolist(),
        }
        print(f"basis {m},{n}: D={len(tags)} {time.time() - t0:.1f}s", flush=True)
        del occ, tags
    out["basis"] = basis

    m, n, J, U, mu, nev = 12, 12, 0.05, 1.0, 0.6, 10
    H = hamiltonian_ref_order(o, m, n, J, U, mu)

    def run(k):
        t0 = time.time()
        re, im = ref.irlm(H, k)
        return k, re, im, time.time() - t0

    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        res = {k: (re, im, dt) for k, re, im, dt in ex.map(run, [nev, nev + 2])}
    re, im, dt = res[nev]
    re2, _, dt2 = res[nev + 2]
    out["irlm"] = {"m12n12": {
        "m": m, "n": n, "J": J, "U": U, "mu": mu, "nev": nev, "converged": True,
        "evals_reference_order": re.tolist(), "imag_max": float(np.abs(im).max()),
        "evals_sorted": sorted(re.tolist()), "seconds": dt, "nnz": int(H.nnz),
        "evals_lowest_from_nev_plus_2": sorted(re2.tolist())[:nev], "seconds_nev_plus_2": dt2,
    }}
    print(f"m12n12: {dt:.0f}s / {dt2:.0f}s E0={min(re)}", flush=True)
    path = os.path.join(HERE, "reference_golden_large.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    if "--scmf-only" in sys.argv:
        update_scmf_only()
    elif "--large" in sys.argv:
        large_cases()
    else:
        main("--quick" in sys.argv)
