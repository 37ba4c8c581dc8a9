"""ctypes front-end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
arm may import this module, and only to check results against the oracle or
as the timed CPU restatement of the reference's path; the product library
never does.

`Oracle` wraps oracle/liboracle.so (plain-C restatement of the reference's
basis, Hamiltonian, IRLM eigensolver and observables, see bh_oracle.c for the
file:line it follows).  `Reference` wraps oracle/_ref/libbhref.so, the
reference's own sources compiled in place (only present where the reference
tree was available at build time).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libbhref.so")

_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(
        os.path.join(HERE, "bh_oracle.c")
    ):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB


REFERENCE_TREE = os.environ.get("BH_REFERENCE_TREE", "/root/reference")


def build_ref(ref_root: str = REFERENCE_TREE) -> str | None:
    """Compile the reference harness where the reference tree exists
    (BH_REFERENCE_TREE, default /root/reference)."""
    if not os.path.isdir(os.path.join(ref_root, "src")):
        return None
    if not os.path.exists(REF_LIB):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}"], check=True)
    return REF_LIB


class Oracle:
    def __init__(self):
        lib = C.CDLL(build())
        self.lib = lib
        lib.bho_dimension.restype = C.c_int64
        lib.bho_dimension.argtypes = [C.c_int, C.c_int]
        lib.bho_lex_states.argtypes = [C.c_int, C.c_int, C.c_int64, _u8p]
        lib.bho_rank.restype = C.c_int64
        lib.bho_rank.argtypes = [C.c_int, _u8p]
        lib.bho_tags.argtypes = [C.c_int, C.c_int64, _u8p, _f64p]
        lib.bho_reference_order.argtypes = [C.c_int, C.c_int64, _u8p, _i32p, _i32p]
        lib.bho_build_T.argtypes = [
            C.c_int, C.c_int, C.c_int64, _u8p, _i32p, _i32p, C.c_void_p, C.c_void_p,
            _i64p, C.c_void_p, C.c_void_p,
        ]
        lib.bho_diag_V.argtypes = [C.c_int, C.c_int64, _u8p, C.c_void_p, _f64p]
        lib.bho_spmv.argtypes = [
            C.c_int64, _i64p, _i32p, _f64p, _f64p, C.c_int, C.c_double, C.c_double,
            C.c_double, _f64p, _f64p,
        ]
        lib.bho_sym_eig.argtypes = [C.c_int, _f64p, _f64p]
        lib.bho_start_vector.argtypes = [C.c_uint64, C.c_int64, _f64p]
        lib.bho_irlm.argtypes = [
            C.c_int64, _i64p, _i32p, _f64p, _f64p, C.c_int, C.c_double, C.c_double,
            C.c_double, C.c_int, C.c_int, C.c_double, _f64p, C.c_void_p,
            C.POINTER(C.c_int), C.POINTER(C.c_long),
        ]
        lib.bho_irlm_batch.argtypes = [
            C.c_int64, _i64p, _i32p, _f64p, _f64p, C.c_int, C.c_int, _f64p, _f64p, _f64p,
            C.c_int, C.c_int, C.c_double, C.c_int, _f64p, _i32p,
        ]
        lib.bho_max_threads.restype = C.c_int
        lib.bho_set_inner_threads.argtypes = [C.c_int]
        lib.bho_irlm_wave.argtypes = [
            C.c_int64, _i64p, _i32p, _f64p, _f64p, C.c_int, C.c_int, _f64p, _f64p, _f64p,
            C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, _f64p, _i32p,
        ]
        lib.bho_gap_ratio.restype = C.c_double
        lib.bho_gap_ratio.argtypes = [C.c_int, _f64p, C.c_void_p]
        lib.bho_spdm.argtypes = [C.c_int, C.c_int, C.c_int64, _u8p, _f64p, _f64p]
        lib.bho_coherence.restype = C.c_double
        lib.bho_coherence.argtypes = [C.c_int, _f64p]
        lib.bho_condensate_fraction.restype = C.c_double
        lib.bho_condensate_fraction.argtypes = [C.c_int, _f64p]
        lib.bho_scmf.restype = C.c_double
        lib.bho_scmf.argtypes = [C.c_double, C.c_double, C.c_int, C.c_double, C.c_int, C.c_int,
                                 C.c_void_p]
        lib.bho_scmf_batch.argtypes = [C.c_int, _f64p, _f64p, C.c_int, _f64p, C.c_int, C.c_int,
                                       C.c_int, _f64p, C.c_void_p]

    # ---- basis ----
    def dimension(self, m: int, n: int) -> int:
        return int(self.lib.bho_dimension(m, n))

    def lex_states(self, m: int, n: int) -> np.ndarray:
        D = self.dimension(m, n)
        occ = np.zeros((D, m), dtype=np.uint8)
        rc = self.lib.bho_lex_states(m, n, D, occ)
        assert rc == 0, rc
        return occ

    def rank(self, occ_row: np.ndarray) -> int:
        o = np.ascontiguousarray(occ_row, dtype=np.uint8)
        return int(self.lib.bho_rank(len(o), o))

    def tags(self, occ: np.ndarray) -> np.ndarray:
        D, m = occ.shape
        t = np.zeros(D)
        self.lib.bho_tags(m, D, np.ascontiguousarray(occ), t)
        return t

    def reference_order(self, occ: np.ndarray):
        """(col_of_lex, lex_of_col) of the reference's fixed_set_basis order."""
        D, m = occ.shape
        a = np.zeros(D, np.int32)
        b = np.zeros(D, np.int32)
        assert self.lib.bho_reference_order(m, D, np.ascontiguousarray(occ), a, b) == 0
        return a, b

    # ---- Hamiltonian ----
    def build_T(self, occ, nbr_off, nbr, lex_of_row=None, col_of_lex=None):
        D, m = occ.shape
        n = int(occ[0].sum()) if D else 0
        occ = np.ascontiguousarray(occ)
        off = np.ascontiguousarray(nbr_off, np.int32)
        nb = np.ascontiguousarray(nbr, np.int32)
        lr = None if lex_of_row is None else np.ascontiguousarray(lex_of_row, np.int32)
        cl = None if col_of_lex is None else np.ascontiguousarray(col_of_lex, np.int32)
        vp = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
        rp = np.zeros(D + 1, np.int64)
        rc = self.lib.bho_build_T(m, n, D, occ, off, nb, vp(lr), vp(cl), rp, None, None)
        if rc != 0:
            raise ValueError(f"bho_build_T failed ({rc})")
        nnz = int(rp[-1])
        ci = np.zeros(max(nnz, 1), np.int32)
        tv = np.zeros(max(nnz, 1), np.float64)
        rc = self.lib.bho_build_T(m, n, D, occ, off, nb, vp(lr), vp(cl), rp, vp(ci), vp(tv))
        assert rc == 0
        return rp, ci[:nnz], tv[:nnz]

    def diag_V(self, occ, lex_of_row=None):
        D, m = occ.shape
        v = np.zeros(D)
        lr = None if lex_of_row is None else np.ascontiguousarray(lex_of_row, np.int32)
        self.lib.bho_diag_V(m, D, np.ascontiguousarray(occ),
                            None if lr is None else lr.ctypes.data_as(C.c_void_p), v)
        return v

    def spmv(self, rp, ci, tv, vd, n, J, U, mu, x):
        y = np.zeros_like(x)
        self.lib.bho_spmv(len(vd), rp, ci, tv, vd, n, J, U, mu, np.ascontiguousarray(x), y)
        return y

    def full_csr(self, rp, ci, tv, vd, n, J, U, mu):
        """H = J T + U V - mu n as CSR with the diagonal stored in every row."""
        D = len(vd)
        rows = np.repeat(np.arange(D), np.diff(rp))
        import scipy.sparse as sp

        Tm = sp.csr_matrix((J * tv, (rows, ci)), shape=(D, D))
        H = Tm + sp.diags(U * vd - mu * n)
        H = sp.csr_matrix(H)
        H.sort_indices()
        return H

    # ---- eigensolver ----
    def start_vector(self, D: int, seed: int = 0) -> np.ndarray:
        v = np.zeros(D)
        self.lib.bho_start_vector(seed, D, v)
        return v

    def sym_eig(self, a: np.ndarray):
        n = a.shape[0]
        A = np.asfortranarray(a, dtype=np.float64).copy(order="F")
        flat = np.ascontiguousarray(A.reshape(-1, order="F"))
        w = np.zeros(n)
        rc = self.lib.bho_sym_eig(n, flat, w)
        assert rc == 0, rc
        return w, flat.reshape((n, n), order="F")

    def irlm(self, rp, ci, tv, vd, n, J, U, mu, nev=10, maxit=1000, tol=1e-10,
             want_vectors=False):
        """Op::IRLM_eigen restatement: (evals in reference order, evecs, niter, nop)."""
        D = len(vd)
        ev = np.zeros(nev)
        vec = np.zeros((nev, D)) if want_vectors else None
        it = C.c_int(0)
        nop = C.c_long(0)
        nc = self.lib.bho_irlm(D, rp, ci, tv, vd, n, J, U, mu, nev, maxit, tol, ev,
                               None if vec is None else vec.ctypes.data_as(C.c_void_p),
                               C.byref(it), C.byref(nop))
        if nc < 0:
            raise ValueError("invalid nev for this dimension")
        return ev[:nc], (None if vec is None else vec[:nc]), it.value, nop.value

    def irlm_batch(self, rp, ci, tv, vd, n, J, U, mu, nev=10, maxit=1000, tol=1e-10,
                   nthreads=0):
        J = np.ascontiguousarray(J, np.float64)
        S = len(J)
        U = np.ascontiguousarray(np.broadcast_to(U, (S,)), np.float64)
        mu = np.ascontiguousarray(np.broadcast_to(mu, (S,)), np.float64)
        ev = np.zeros((S, nev))
        nc = np.zeros(S, np.int32)
        self.lib.bho_irlm_batch(len(vd), rp, ci, tv, vd, n, S, J, U, mu, nev, maxit, tol,
                                nthreads, ev, nc)
        return ev, nc

    def irlm_wave(self, rp, ci, tv, vd, n, J, U, mu, nev=10, maxit=1000, tol=1e-10,
                  groups=1, inner=1):
        """Independent solves, `groups` at a time, each on `inner` threads."""
        J = np.ascontiguousarray(J, np.float64)
        S = len(J)
        U = np.ascontiguousarray(np.broadcast_to(U, (S,)), np.float64)
        mu = np.ascontiguousarray(np.broadcast_to(mu, (S,)), np.float64)
        ev = np.zeros((S, nev))
        nc = np.zeros(S, np.int32)
        self.lib.bho_irlm_wave(len(vd), rp, ci, tv, vd, n, S, J, U, mu, nev, maxit, tol,
                               groups, inner, ev, nc)
        return ev, nc

    def max_threads(self) -> int:
        return int(self.lib.bho_max_threads())

    def set_inner_threads(self, t: int):
        """Threads of the row loops inside each IRLM solve (0 = serial)."""
        self.lib.bho_set_inner_threads(int(t))

    # ---- observables ----
    def gap_ratio(self, evals):
        e = np.ascontiguousarray(evals, np.float64)
        r = np.zeros(max(len(e) - 2, 1))
        g = self.lib.bho_gap_ratio(len(e), e, r.ctypes.data_as(C.c_void_p))
        return g, r[: max(len(e) - 2, 0)]

    def spdm(self, occ, phi):
        D, m = occ.shape
        n = int(occ[0].sum())
        rho = np.zeros(m * m)
        self.lib.bho_spdm(m, n, D, np.ascontiguousarray(occ), np.ascontiguousarray(phi), rho)
        return rho.reshape(m, m)

    def coherence(self, rho):
        return float(self.lib.bho_coherence(rho.shape[0], np.ascontiguousarray(rho.ravel())))

    def condensate_fraction(self, rho):
        return float(self.lib.bho_condensate_fraction(rho.shape[0],
                                                      np.ascontiguousarray(rho.ravel())))

    # ---- mean field ----
    def scmf(self, mu, J, q, psi0, precision, pmax=64):
        it = C.c_int(0)
        v = self.lib.bho_scmf(mu, J, q, psi0, precision, pmax, C.byref(it))
        return float(v), it.value

    def scmf_batch(self, mu, J, q, psi0, precision, pmax=64, nthreads=0):
        mu = np.ascontiguousarray(mu, np.float64)
        J = np.ascontiguousarray(np.broadcast_to(J, mu.shape), np.float64)
        psi0 = np.ascontiguousarray(np.broadcast_to(psi0, mu.shape), np.float64)
        psi = np.zeros(len(mu))
        outer = np.zeros(len(mu), np.int32)
        self.lib.bho_scmf_batch(len(mu), mu, J, q, psi0, precision, pmax, nthreads, psi,
                                outer.ctypes.data_as(C.c_void_p))
        return psi, outer


class Reference:
    """The reference's own exact-path code, compiled from its sources."""

    def __init__(self, path: str = REF_LIB):
        lib = C.CDLL(path)
        self.lib = lib
        lib.ref_dimension.argtypes = [C.c_int, C.c_int]
        lib.ref_fixed_set_basis.argtypes = [C.c_int, C.c_int, _f64p, _f64p]
        lib.ref_init_lexicographic.argtypes = [C.c_int, C.c_int, _f64p]
        lib.ref_neighbours.argtypes = [C.c_int, C.c_int, C.c_int, _i32p, _i32p, C.c_int]
        lib.ref_irlm.argtypes = [C.c_int64, _i64p, _i32p, _f64p, C.c_int, _f64p, _f64p,
                                 C.c_void_p]
        lib.ref_exact_eigen.argtypes = [C.c_int64, _i64p, _i32p, _f64p, _f64p]
        lib.ref_gap_ratios.argtypes = [C.c_int, _f64p, _f64p]
        lib.ref_coherence.restype = C.c_double
        lib.ref_coherence.argtypes = [C.c_int, _f64p]
        lib.ref_scmf.restype = C.c_double
        lib.ref_scmf.argtypes = [C.c_double, C.c_double, C.c_int, C.c_double, C.c_int]

    def fixed_set_basis(self, m, n):
        D = self.lib.ref_dimension(m, n)
        tags = np.zeros(D)
        basis = np.zeros(m * D)
        self.lib.ref_fixed_set_basis(m, n, tags, basis)
        return tags, basis.reshape(D, m)  # row c = column c of the reference matrix

    def init_lexicographic(self, m, n):
        D = self.lib.ref_dimension(m, n)
        basis = np.zeros(m * D)
        self.lib.ref_init_lexicographic(m, n, basis)
        return basis.reshape(D, m)

    def neighbours(self, kind, m, closed=True):
        off = np.zeros(m + 1, np.int32)
        nb = np.zeros(8 * m + 8, np.int32)
        c = self.lib.ref_neighbours(kind, m, int(closed), off, nb, len(nb))
        if c < 0:
            raise ValueError("reference Neighbours threw")
        return off, nb[:c]

    def irlm(self, H, nev):
        H = H.tocsr()
        H.sort_indices()
        D = H.shape[0]
        re = np.zeros(nev)
        im = np.zeros(nev)
        nc = self.lib.ref_irlm(D, H.indptr.astype(np.int64), H.indices.astype(np.int32),
                               H.data.astype(np.float64), nev, re, im, None)
        if nc < 0:
            raise RuntimeError("Eigenvalue computation failed.")
        return re[:nc], im[:nc]

    def exact_eigen(self, H):
        H = H.tocsr()
        D = H.shape[0]
        ev = np.zeros(D)
        self.lib.ref_exact_eigen(D, H.indptr.astype(np.int64), H.indices.astype(np.int32),
                                 H.data.astype(np.float64), ev)
        return ev

    def gap_ratios(self, evals):
        e = np.ascontiguousarray(evals, np.float64)
        r = np.zeros(len(e) - 2)
        self.lib.ref_gap_ratios(len(e), e, r)
        return r

    def coherence(self, rho):
        return float(self.lib.ref_coherence(rho.shape[0], np.ascontiguousarray(rho.ravel())))

    def scmf(self, mu, J, q, psi0, precision):
        return float(self.lib.ref_scmf(mu, J, q, psi0, precision))
