"""Host-side mirror of the reference's exact-path API over the C ABI.

Maximilien-Hantonne/Bose-Hubbard-Phase-Transition exposes its exact path as
C++ functions (``BH::fixed_set_basis``, ``BH::fixed_bosons_hamiltonian``,
``Neighbours``, ``Op::IRLM_eigen``, ``Analysis::gap_ratios``).  This module
keeps those names, argument meanings and error behaviour and routes every
computation of the exact path (basis, Hamiltonian, eigensolves, observables)
through ``libbhgb300.so`` (include/bh_gb300.h): none of it runs on the CPU.
The only host arithmetic is in small helpers of the reference's BH namespace
that act on arrays the caller already holds (tags of a basis, the tag search,
the mean-field single-site matrix).  The library must load; if it is missing
it is built, and if that fails the import fails loudly.

Layout conventions: a basis is returned as the reference returns it
(tags[D], basis[m, D]); sparse matrices are scipy CSR in the reference's
column order; eigenvectors are columns.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

_HERE = os.path.dirname(os.path.abspath(__file__))

BH_OK, BH_ERR_ARG, BH_ERR_NOCONV, BH_ERR_BREAKDOWN, BH_ERR_TIMEOUT, BH_ERR_CUDA, BH_ERR_NOMEM = range(7)
ORDER_REFERENCE, ORDER_LEX = 0, 1
PREC_FP64, PREC_MIXED = 0, 1


class BHError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class bh_solver_opts(C.Structure):
    _fields_ = [
        ("nev", C.c_int), ("ncv", C.c_int), ("block", C.c_int), ("precision", C.c_int),
        ("max_restarts", C.c_int), ("tol", C.c_double), ("seed", C.c_uint64),
        ("want_vectors", C.c_int), ("order", C.c_int),
    ]


class bh_solve_info(C.Structure):
    _fields_ = [
        ("nconv", C.c_int), ("restarts", C.c_int), ("matvecs", C.c_int64),
        ("max_resid", C.c_double), ("seconds", C.c_double), ("launches", C.c_int64),
    ]


class bh_spmm_shape(C.Structure):
    _fields_ = [("lanes", C.c_int), ("cols_per_lane", C.c_int), ("grid", C.c_int64)]


class bh_spmm_tuning(C.Structure):
    _fields_ = [
        ("matrix_free", C.c_int), ("elem_bytes", C.c_int), ("dim", C.c_int64), ("nnz", C.c_int64),
        ("ncols", C.c_int), ("shape", bh_spmm_shape), ("ms", C.c_float), ("ms_default", C.c_float),
        ("candidates", C.c_int),
    ]


EXPORTS = [
    "bh_last_error", "bh_version", "bh_neighbours_chain", "bh_neighbours_square",
    "bh_neighbours_cube", "bh_dimension", "bh_basis_create", "bh_basis_destroy",
    "bh_basis_info", "bh_basis_copy", "bh_basis_index", "bh_hamiltonian_create",
    "bh_hamiltonian_create_matrix_free", "bh_hamiltonian_is_matrix_free",
    "bh_hamiltonian_destroy", "bh_hamiltonian_nnz", "bh_hamiltonian_csr", "bh_hamiltonian_multi_csr",
    "bh_hamiltonian_apply", "bh_hamiltonian_apply_noalloc", "bh_solver_opts_default", "bh_eigsh", "bh_eigsh_csr",
    "bh_eigsh_batch", "bh_eigsh_batch_status", "bh_eigsh_batch_vectors", "bh_eigsh_batch_sectors", "bh_folm_diag_csr", "bh_dense_eigh", "bh_gap_ratios", "bh_spdm", "bh_phase_map", "bh_scmf", "bh_mean_field_grid", "bh_profile_enable",
    "bh_profile_reset", "bh_profile_count", "bh_profile_get",
    "bh_spmm_candidates", "bh_hamiltonian_apply_shape", "bh_spmm_autotune", "bh_spmm_tuning_count",
    "bh_spmm_tuning_get", "bh_spmm_tuning_reset",
]

_lib = None


def lib_path() -> str:
    return _build.LIB


def load() -> C.CDLL:
    """Load (building first if needed) libbhgb300.so and declare its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    L = C.CDLL(path)
    vp, i32p, i64p, f64p = C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_double)
    L.bh_last_error.restype = C.c_char_p
    L.bh_version.restype = C.c_int
    for f in ("bh_neighbours_chain", "bh_neighbours_square", "bh_neighbours_cube"):
        getattr(L, f).argtypes = [C.c_int, C.c_int, vp, vp, C.c_int, C.POINTER(C.c_int)]
    L.bh_dimension.argtypes = [C.c_int, C.c_int, i64p]
    L.bh_basis_create.argtypes = [C.c_int, C.c_int, C.POINTER(vp)]
    L.bh_basis_destroy.argtypes = [vp]
    L.bh_basis_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), i64p]
    L.bh_basis_copy.argtypes = [vp, vp, vp, vp, vp]
    L.bh_basis_index.argtypes = [vp, C.c_int64, vp, vp]
    L.bh_hamiltonian_create.argtypes = [vp, vp, vp, C.POINTER(vp)]
    L.bh_hamiltonian_create_matrix_free.argtypes = [vp, vp, vp, C.POINTER(vp)]
    L.bh_hamiltonian_is_matrix_free.argtypes = [vp, C.POINTER(C.c_int)]
    L.bh_hamiltonian_destroy.argtypes = [vp]
    L.bh_hamiltonian_nnz.argtypes = [vp, i64p]
    L.bh_hamiltonian_csr.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_double, vp, vp, vp]
    L.bh_hamiltonian_multi_csr.argtypes = [C.c_int, vp, C.c_int, C.c_double, C.c_double, C.c_double, vp, vp, vp]
    L.bh_hamiltonian_apply.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, vp, vp]
    L.bh_hamiltonian_apply_noalloc.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_double,
                                                C.c_int, vp, vp, vp]
    L.bh_solver_opts_default.argtypes = [C.POINTER(bh_solver_opts)]
    L.bh_solver_opts_default.restype = None
    L.bh_eigsh.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.POINTER(bh_solver_opts),
                           vp, vp, vp, C.POINTER(bh_solve_info)]
    L.bh_eigsh_csr.argtypes = [C.c_int64, vp, vp, vp, C.POINTER(bh_solver_opts), vp, vp, vp,
                               C.POINTER(bh_solve_info)]
    L.bh_eigsh_batch.argtypes = [vp, C.c_int, vp, vp, vp, C.POINTER(bh_solver_opts), vp, vp, vp,
                                 C.POINTER(bh_solve_info)]
    L.bh_eigsh_batch_status.argtypes = [vp, C.c_int, vp, vp, vp, C.POINTER(bh_solver_opts), vp, vp, vp,
                                        vp, C.POINTER(bh_solve_info)]
    L.bh_eigsh_batch_vectors.argtypes = [vp, C.c_int, vp, vp, vp, C.POINTER(bh_solver_opts), vp, vp, vp,
                                         vp, C.POINTER(bh_solve_info)]
    L.bh_eigsh_batch_sectors.argtypes = [C.c_int, vp, C.c_int, vp, vp, vp, C.POINTER(bh_solver_opts), vp, vp, vp,
                                         C.POINTER(bh_solve_info)]
    L.bh_folm_diag_csr.argtypes = [C.c_int64, vp, vp, vp, C.c_int, vp, vp, vp, vp]
    L.bh_dense_eigh.argtypes = [C.c_int64, vp, vp, vp]
    L.bh_gap_ratios.argtypes = [C.c_int, vp, vp, f64p]
    L.bh_spdm.argtypes = [vp, C.c_int, vp, vp]
    L.bh_phase_map.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, vp, C.c_int, vp, vp, vp]
    L.bh_scmf.argtypes = [C.c_int, vp, vp, C.c_int, vp, C.c_int, vp, vp]
    L.bh_mean_field_grid.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(C.c_int),
                                     C.POINTER(C.c_int), vp, vp, vp]
    L.bh_profile_enable.argtypes = [C.c_int]
    L.bh_profile_count.argtypes = [C.POINTER(C.c_int)]
    L.bh_profile_get.argtypes = [C.c_int, C.c_char_p, C.c_int, i64p, f64p, f64p]
    L.bh_spmm_candidates.argtypes = [C.c_int, C.c_int, C.POINTER(bh_spmm_shape), C.c_int, C.POINTER(C.c_int)]
    L.bh_hamiltonian_apply_shape.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                                             C.POINTER(bh_spmm_shape), vp, vp]
    L.bh_spmm_autotune.argtypes = [vp, C.c_int, C.c_int, C.POINTER(bh_spmm_shape),
                                   C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.bh_spmm_tuning_count.argtypes = [C.POINTER(C.c_int)]
    L.bh_spmm_tuning_get.argtypes = [C.c_int, C.POINTER(bh_spmm_tuning)]
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _check(rc: int):
    if rc != BH_OK:
        msg = load().bh_last_error().decode()
        if rc == BH_ERR_NOCONV:
            raise BHError(rc, msg or "Eigenvalue computation failed.")
        if rc == BH_ERR_ARG:
            err = BHError(rc, msg)
            raise ValueError(msg) from err
        raise BHError(rc, msg)


def default_opts(**kw) -> bh_solver_opts:
    o = bh_solver_opts()
    load().bh_solver_opts_default(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


# ---------------------------------------------------------------------------
# Neighbours (neighbours.hpp:20-58)
# ---------------------------------------------------------------------------
class Neighbours:
    """Neighbour lists of a chain / square / cube lattice of m sites."""

    def __init__(self, m: int):
        self.m = int(m)
        self._lists: list[list[int]] = [[] for _ in range(self.m)]

    def _fill(self, fn, closed: bool):
        L = load()
        off = np.zeros(self.m + 1, np.int32)
        cnt = C.c_int(0)
        _check(getattr(L, fn)(self.m, int(bool(closed)), _ptr(off), None, 0, C.byref(cnt)))
        nb = np.zeros(max(cnt.value, 1), np.int32)
        _check(getattr(L, fn)(self.m, int(bool(closed)), _ptr(off), _ptr(nb), len(nb), C.byref(cnt)))
        self._lists = [nb[off[i]:off[i + 1]].tolist() for i in range(self.m)]

    def chain_neighbours(self, closed: bool = True):
        self._fill("bh_neighbours_chain", closed)

    def square_neighbours(self, closed: bool = True):
        self._fill("bh_neighbours_square", closed)

    def cube_neighbours(self, closed: bool = True):
        self._fill("bh_neighbours_cube", closed)

    def getNeighbours(self) -> list[list[int]]:
        return [list(x) for x in self._lists]


def flatten_neighbours(lists) -> tuple[np.ndarray, np.ndarray]:
    off = np.zeros(len(lists) + 1, np.int32)
    for i, l in enumerate(lists):
        off[i + 1] = off[i] + len(l)
    flat = np.array([j for l in lists for j in l], np.int32) if off[-1] else np.zeros(1, np.int32)
    return off, flat


# ---------------------------------------------------------------------------
# device-resident basis + Hamiltonian (the engine objects)
# ---------------------------------------------------------------------------
class Basis:
    """Fixed-n Fock basis built on the device (BH::fixed_set_basis)."""

    def __init__(self, m: int, n: int):
        L = load()
        self._h = C.c_void_p()
        _check(L.bh_basis_create(int(m), int(n), C.byref(self._h)))
        mm, nn, D = C.c_int(), C.c_int(), C.c_int64()
        _check(L.bh_basis_info(self._h, C.byref(mm), C.byref(nn), C.byref(D)))
        self.m, self.n, self.D = mm.value, nn.value, D.value
        self._col_of_lex = None

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.bh_basis_destroy(self._h)
            self._h = None

    def copy(self, tags=True, basis=True):
        t = np.zeros(self.D) if tags else None
        b = np.zeros(self.D * self.m) if basis else None
        _check(load().bh_basis_copy(self._h, _ptr(t), _ptr(b), None, None))
        return t, (None if b is None else b.reshape(self.D, self.m).T.copy())

    def orders(self):
        a = np.zeros(self.D, np.int32)
        b = np.zeros(self.D, np.int32)
        _check(load().bh_basis_copy(self._h, None, None, _ptr(a), _ptr(b)))
        return a, b

    def index(self, occ: np.ndarray) -> np.ndarray:
        occ = np.ascontiguousarray(np.atleast_2d(occ), np.uint8)
        out = np.zeros(occ.shape[0], np.int32)
        _check(load().bh_basis_index(self._h, occ.shape[0], _ptr(occ), _ptr(out)))
        return out


@dataclass
class SolveInfo:
    nconv: int
    restarts: int
    matvecs: int
    max_resid: float
    seconds: float
    launches: int


class Hamiltonian:
    """H = J T + U V - mu N of one sector, assembled on the device once.

    matrix_free=True keeps no matrix entries: each product regenerates the
    rows from packed occupation strings (bh_hamiltonian_create_matrix_free).
    """

    def __init__(self, basis: Basis, neighbours, matrix_free: bool = False):
        self.basis = basis
        off, flat = flatten_neighbours(neighbours)
        if len(off) != basis.m + 1:
            raise ValueError("neighbour lists must have one entry per site")
        self._h = C.c_void_p()
        create = load().bh_hamiltonian_create_matrix_free if matrix_free else load().bh_hamiltonian_create
        _check(create(basis._h, _ptr(off), _ptr(flat), C.byref(self._h)))
        self.matrix_free = bool(matrix_free)
        nnz = C.c_int64()
        _check(load().bh_hamiltonian_nnz(self._h, C.byref(nnz)))
        self.nnz_offdiag = nnz.value
        self.m, self.n, self.D = basis.m, basis.n, basis.D

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.bh_hamiltonian_destroy(self._h)
            self._h = None

    def csr_arrays(self, J: float, U: float, mu: float, order: int = ORDER_REFERENCE):
        D, nz = self.D, self.nnz_offdiag + self.D
        rp = np.zeros(D + 1, np.int64)
        ci = np.zeros(nz, np.int32)
        val = np.zeros(nz, np.float64)
        _check(load().bh_hamiltonian_csr(self._h, order, J, U, mu, _ptr(rp), _ptr(ci), _ptr(val)))
        return rp, ci, val

    def csr(self, J: float, U: float, mu: float, order: int = ORDER_REFERENCE):
        import scipy.sparse as sp

        rp, ci, val = self.csr_arrays(J, U, mu, order)
        return sp.csr_matrix((val, ci, rp), shape=(self.D, self.D))

    def apply(self, x: np.ndarray, J: float, U: float, mu: float, order: int = ORDER_REFERENCE):
        x = np.asarray(x, np.float64)
        X = np.ascontiguousarray(x.reshape(self.D, -1))
        Y = np.zeros_like(X)
        _check(load().bh_hamiltonian_apply(self._h, order, J, U, mu, X.shape[1], _ptr(X), _ptr(Y)))
        return Y.reshape(x.shape)

    def apply_shape(self, x: np.ndarray, J: float, U: float, mu: float, shape=None,
                    precision: int = PREC_FP64):
        """y = H x in the lexicographic order with a given launch shape of the
        product ((lanes, cols_per_lane, grid) or None for the default); FP64,
        or FP32 vectors and values with PREC_MIXED."""
        x = np.asarray(x, np.float64)
        X = np.ascontiguousarray(x.reshape(self.D, -1))
        Y = np.zeros_like(X)
        sh = None if shape is None else C.byref(bh_spmm_shape(*shape))
        _check(load().bh_hamiltonian_apply_shape(self._h, precision, J, U, mu, X.shape[1], sh,
                                                 _ptr(X), _ptr(Y)))
        return Y.reshape(x.shape)

    def autotune(self, nvec: int, precision: int = PREC_MIXED) -> dict:
        """Times the product's launch shapes for nvec columns now and records
        the fastest for this operator's width class."""
        sh, ms, md = bh_spmm_shape(), C.c_float(), C.c_float()
        _check(load().bh_spmm_autotune(self._h, nvec, precision, C.byref(sh), C.byref(ms), C.byref(md)))
        return {"shape": (sh.lanes, sh.cols_per_lane, sh.grid), "ms": ms.value, "ms_default": md.value}

    def eigsh(self, J: float, U: float, mu: float, nev: int = 10, vectors: bool = False,
              order: int = ORDER_REFERENCE, **opt):
        o = default_opts(nev=nev, order=order, **opt)
        ev = np.zeros(nev)
        rs = np.zeros(nev)
        vec = np.zeros((nev, self.D)) if vectors else None
        info = bh_solve_info()
        _check(load().bh_eigsh(self._h, J, U, mu, C.byref(o), _ptr(ev), _ptr(rs), _ptr(vec),
                               C.byref(info)))
        return ev, rs, (None if vec is None else vec.T.copy()), _info(info)

    def eigsh_batch(self, J, U, mu, nev: int = 10, vectors: bool = False, status: bool = False, **opt):
        """Batched lowest eigenpairs of (J[s], U[s], mu[s]).  Returns
        ev, resid [S, nev], nconv [S], info, and with vectors=True also the
        eigenvectors [S, nev, D] (rows in opt['order'], reference by default);
        with status=True (not with vectors) a per-point status array [S]
        (BH_OK, BH_ERR_NOCONV or BH_ERR_BREAKDOWN) instead."""
        J = np.ascontiguousarray(J, np.float64)
        S = len(J)
        U = np.ascontiguousarray(np.broadcast_to(U, (S,)), np.float64)
        mu = np.ascontiguousarray(np.broadcast_to(mu, (S,)), np.float64)
        o = default_opts(nev=nev, **opt)
        ev = np.zeros((S, nev))
        rs = np.zeros((S, nev))
        nc = np.zeros(S, np.int32)
        info = bh_solve_info()
        if status:
            if vectors:
                raise ValueError("status=True is not available with vectors=True")
            st = np.zeros(S, np.int32)
            _check(load().bh_eigsh_batch_status(self._h, S, _ptr(J), _ptr(U), _ptr(mu), C.byref(o),
                                                _ptr(ev), _ptr(rs), _ptr(nc), _ptr(st), C.byref(info)))
            return ev, rs, nc, _info(info), st
        if vectors:
            vec = np.zeros((S, nev, self.D))
            _check(load().bh_eigsh_batch_vectors(self._h, S, _ptr(J), _ptr(U), _ptr(mu), C.byref(o),
                                                 _ptr(ev), _ptr(rs), _ptr(nc), _ptr(vec), C.byref(info)))
            return ev, rs, nc, _info(info), vec
        _check(load().bh_eigsh_batch(self._h, S, _ptr(J), _ptr(U), _ptr(mu), C.byref(o),
                                     _ptr(ev), _ptr(rs), _ptr(nc), C.byref(info)))
        return ev, rs, nc, _info(info)

    def spdm(self, phi: np.ndarray, order: int = ORDER_REFERENCE) -> np.ndarray:
        phi = np.ascontiguousarray(phi, np.float64)
        rho = np.zeros(self.m * self.m)
        _check(load().bh_spdm(self._h, order, _ptr(phi), _ptr(rho)))
        return rho.reshape(self.m, self.m)


def eigsh_sectors(hams, J, U, mu, nev: int = 10, **opt):
    """Batched solve of the same (J, U, mu) points in several Hamiltonians
    (particle-number sectors) at once, the sectors running concurrently on
    the device (bh_eigsh_batch_sectors).  Returns ev, resid [nh, S, nev],
    nconv [nh, S] and the aggregate SolveInfo."""
    J = np.ascontiguousarray(J, np.float64)
    S = len(J)
    U = np.ascontiguousarray(np.broadcast_to(U, (S,)), np.float64)
    mu = np.ascontiguousarray(np.broadcast_to(mu, (S,)), np.float64)
    nh = len(hams)
    o = default_opts(nev=nev, **opt)
    hs = (C.c_void_p * nh)(*[h._h.value for h in hams])
    ev = np.zeros((nh, S, nev))
    rs = np.zeros((nh, S, nev))
    nc = np.zeros((nh, S), np.int32)
    info = bh_solve_info()
    _check(load().bh_eigsh_batch_sectors(nh, C.cast(hs, C.c_void_p), S, _ptr(J), _ptr(U), _ptr(mu),
                                         C.byref(o), _ptr(ev), _ptr(rs), _ptr(nc), C.byref(info)))
    return ev, rs, nc, _info(info)


def multi_sector_csr(hams, J: float, U: float, mu: float, order: int = ORDER_REFERENCE):
    """Block-diagonal H = J T + U V - mu N of several sector Hamiltonians,
    assembled on the device (bh_hamiltonian_multi_csr), as scipy CSR."""
    import scipy.sparse as sp

    nh = len(hams)
    D = sum(h.D for h in hams)
    nz = sum(h.nnz_offdiag + h.D for h in hams)
    rp = np.zeros(D + 1, np.int64)
    ci = np.zeros(max(nz, 1), np.int32)
    val = np.zeros(max(nz, 1), np.float64)
    hs = (C.c_void_p * nh)(*[h._h.value for h in hams])
    _check(load().bh_hamiltonian_multi_csr(nh, C.cast(hs, C.c_void_p), order, J, U, mu, _ptr(rp), _ptr(ci),
                                           _ptr(val)))
    return sp.csr_matrix((val[:nz], ci[:nz], rp), shape=(D, D))


def _info(i: bh_solve_info) -> SolveInfo:
    return SolveInfo(i.nconv, i.restarts, i.matvecs, i.max_resid, i.seconds, i.launches)


# ---------------------------------------------------------------------------
# the grid over several ranks (one process per GPU): the (J, sector) points
# are independent eigensolves, so ranks split the J points and solve their
# share with no exchange; only the eigenvalues are gathered at the end
# ---------------------------------------------------------------------------
def shard_indices(n_points: int, world: int, rank: int) -> np.ndarray:
    """Grid points of `rank`: rank, rank + world, rank + 2 world, ...  The
    shares are disjoint, cover 0..n_points-1, differ in size by at most one,
    and each spans the whole J range (similar solve cost on every rank)."""
    if world < 1 or not 0 <= rank < world or n_points < 0:
        raise ValueError("need world >= 1, 0 <= rank < world and n_points >= 0")
    return np.arange(rank, n_points, world, dtype=np.int64)


def gather_grid(local: np.ndarray, n_points: int, group=None) -> np.ndarray:
    """Full grid from every rank's share: `local` holds this rank's rows
    (points shard_indices(n_points, world, rank), in that order, along axis 0
    of shape [k, ...]); returns the [n_points, ...] array on every rank.
    Host arrays through torch.distributed.all_gather_object (gloo or NCCL):
    the results, not the data path, cross ranks."""
    import torch.distributed as dist

    local = np.asarray(local)
    if not (dist.is_available() and dist.is_initialized()):
        if local.shape[0] != n_points:
            raise ValueError("without a process group the share is the whole grid")
        return local.copy()
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    mine = shard_indices(n_points, world, rank)
    if local.shape[0] != len(mine):
        raise ValueError(f"rank {rank} holds {local.shape[0]} points, its share is {len(mine)}")
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    out = np.empty((n_points,) + local.shape[1:], dtype=local.dtype)
    for r, part in enumerate(parts):
        out[shard_indices(n_points, world, r)] = part
    return out


def eigsh_sectors_sharded(hams, J, U, mu, nev: int = 10, group=None, **opt):
    """eigsh_sectors over the ranks of a torch.distributed process group:
    this rank solves its share of the J points (shard_indices) in every
    sector, then the eigenvalues and convergence counts are gathered so that
    every rank returns the whole grid: ev [nh, S, nev], nconv [nh, S], and
    this rank's SolveInfo."""
    import torch.distributed as dist

    J = np.ascontiguousarray(J, np.float64)
    S = len(J)
    U = np.broadcast_to(np.asarray(U, np.float64), (S,))
    mu = np.broadcast_to(np.asarray(mu, np.float64), (S,))
    on = dist.is_available() and dist.is_initialized()
    world = dist.get_world_size(group) if on else 1
    rank = dist.get_rank(group) if on else 0
    mine = shard_indices(S, world, rank)
    nh = len(hams)
    if len(mine):
        ev, _, nc, info = eigsh_sectors(hams, J[mine], U[mine], mu[mine], nev=nev, **opt)
    else:
        ev, nc, info = np.zeros((nh, 0, nev)), np.zeros((nh, 0), np.int32), None
    ev_all = gather_grid(np.moveaxis(ev, 1, 0), S, group)    # [S, nh, nev]
    nc_all = gather_grid(np.moveaxis(nc, 1, 0), S, group)    # [S, nh]
    return np.moveaxis(ev_all, 0, 1), np.moveaxis(nc_all, 0, 1), info


# ---------------------------------------------------------------------------
# tracing: per-kernel device time (CUDA events) and algorithmic bytes
# ---------------------------------------------------------------------------
def profile_enable(on: bool = True):
    _check(load().bh_profile_enable(int(bool(on))))


def profile_reset():
    _check(load().bh_profile_reset())


def profile_read() -> dict:
    """{kernel: {"launches", "ms", "bytes"}} accumulated since the last reset."""
    L = load()
    n = C.c_int()
    _check(L.bh_profile_count(C.byref(n)))
    out = {}
    for i in range(n.value):
        name = C.create_string_buffer(64)
        k, ms, by = C.c_int64(), C.c_double(), C.c_double()
        _check(L.bh_profile_get(i, name, 64, C.byref(k), C.byref(ms), C.byref(by)))
        out[name.value.decode()] = {"launches": k.value, "ms": ms.value, "bytes": by.value}
    return out


# ---------------------------------------------------------------------------
# launch shapes of the sparse product and the autotuner's table
# ---------------------------------------------------------------------------
def spmm_candidates(nvec: int, matrix_free: bool = False) -> list[tuple[int, int, int]]:
    """(lanes, cols_per_lane, grid) shapes the tuner times for nvec columns of
    a stored-CSR or matrix-free operator, the default first (grid 0: default,
    -1: one resident wave)."""
    buf = (bh_spmm_shape * 32)()
    n = C.c_int()
    _check(load().bh_spmm_candidates(nvec, int(bool(matrix_free)), buf, 32, C.byref(n)))
    return [(buf[i].lanes, buf[i].cols_per_lane, buf[i].grid) for i in range(n.value)]


def spmm_tuning_table() -> list[dict]:
    """Entries of the process-wide tuning table."""
    L = load()
    n = C.c_int()
    _check(L.bh_spmm_tuning_count(C.byref(n)))
    out = []
    for i in range(n.value):
        e = bh_spmm_tuning()
        _check(L.bh_spmm_tuning_get(i, C.byref(e)))
        out.append({"matrix_free": bool(e.matrix_free), "elem_bytes": e.elem_bytes, "dim": e.dim,
                    "nnz": e.nnz, "ncols": e.ncols,
                    "shape": (e.shape.lanes, e.shape.cols_per_lane, e.shape.grid),
                    "ms": e.ms, "ms_default": e.ms_default, "candidates": e.candidates})
    return out


def spmm_tuning_reset():
    _check(load().bh_spmm_tuning_reset())


# ---------------------------------------------------------------------------
# BH namespace mirror (hamiltonian.hpp:33-112)
# ---------------------------------------------------------------------------
class BH:
    # the primes table of the reference's tags (hamiltonian.cpp:144): site i
    # weighs ln(PRIMES[i]), so tags order states like the integer prod p_i^n_i
    PRIMES = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61, 67, 71, 73, 79,
              83, 89, 97)

    @staticmethod
    def calculate_tag(basis: np.ndarray, primes, k: int) -> float:
        """Tag of column k (hamiltonian.cpp:91-97): sum_i basis[i, k] ln(primes[i]),
        summed over the sites in order."""
        tag = 0.0
        for i in range(basis.shape[0]):
            tag += float(basis[i, k]) * math.log(float(primes[i]))
        return tag

    @staticmethod
    def calculate_tags(basis: np.ndarray, primes) -> np.ndarray:
        """Tags of every column (hamiltonian.cpp:100-106)."""
        return np.array([BH.calculate_tag(basis, primes, k) for k in range(basis.shape[1])])

    @staticmethod
    def search_tag(tags: np.ndarray, x: float) -> int:
        """Index of the tag closest to x (replaces hamiltonian.cpp:126-140, whose
        binary search assumes sorted tags, which fixed_set_basis does not
        produce; distinct states have tags far apart, so the closest tag is the
        state's own for any order)."""
        return int(np.argmin(np.abs(np.asarray(tags, np.float64) - x)))

    @staticmethod
    def sort_basis(tags: np.ndarray, basis: np.ndarray):
        """The reference's sort_basis (hamiltonian.cpp:109-123): an argsort of the
        tags followed by a cycle of swaps that applies the INVERSE of that
        permutation, i.e. new column argsort[r] = old column r.  Returns new
        (tags, basis); the tags of distinct states are distinct."""
        tags = np.asarray(tags, np.float64)
        perm = np.argsort(tags, kind="stable")
        t = np.empty_like(tags)
        t[perm] = tags
        b = np.empty_like(basis)
        b[:, perm] = basis
        return t, b

    @staticmethod
    def max_set_basis(m: int, n: int):
        """States with 1..n bosons (hamiltonian.cpp:151-165): the fixed-n bases
        concatenated in increasing n, then sort_basis over all of them."""
        tags = [np.zeros(0)]
        basis = [np.zeros((m, 0))]
        for bosons in range(1, n + 1):
            t, b = BH.fixed_set_basis(m, bosons)
            tags.append(t)
            basis.append(b)
        return BH.sort_basis(np.concatenate(tags), np.concatenate(basis, axis=1))

    @staticmethod
    def max_bosons_hamiltonian(neighbours, m: int, n_min: int, n_max: int, J: float, U: float,
                               mu: float):
        """Block-diagonal sum of the fixed-n Hamiltonians n_min..n_max
        (hamiltonian.cpp:260-288; n_min clamped to 0, n_max to n_min), each one
        term selected by fixed_bosons_hamiltonian as the reference selects it."""
        import scipy.sparse as sp

        n_min = max(0, n_min)
        n_max = max(n_max, n_min)
        eps = np.finfo(float).eps
        if abs(J) > eps:
            terms = (J, 0.0, 0.0)
        elif abs(U) > eps:
            terms = (0.0, U, 0.0)
        elif abs(mu) > eps:
            terms = (0.0, 0.0, mu)
        else:
            import sys

            for _ in range(n_min, n_max + 1):
                print("Error: At least one of the parameters J, U, mu must be different from zero.",
                      file=sys.stderr)
            D = sum(BH.dimension(m, b) for b in range(n_min, n_max + 1))
            return sp.csr_matrix((D, D))
        hams = [Hamiltonian(Basis(m, b), neighbours) for b in range(n_min, n_max + 1)]
        H = multi_sector_csr(hams, *terms)
        if terms[0] != 0.0:
            H.eliminate_zeros()  # hopping only: no diagonal entries, as fill_hopping
            return H
        d = H.diagonal()  # one explicit entry per row, as fill_interaction / fill_chemical
        D = len(d)
        return sp.csr_matrix((d, np.arange(D, dtype=np.int32), np.arange(D + 1)), shape=(D, D))

    @staticmethod
    def h_MF(psi: float, p: int, mu: float, J: float, q: int) -> np.ndarray:
        """Mean-field single-site Hamiltonian on occupations 0..2p
        (hamiltonian.cpp:290-309), the same entries."""
        k = 2 * p + 1
        h = np.zeros((k, k))
        for i in range(k):
            h[i, i] = -mu * i + 0.5 * i * (i - 1) + q * J * psi * psi
        for j in range(1, k):
            h[j, j - 1] = h[j - 1, j] = -q * J * psi * math.sqrt(float(j))
        return h

    @staticmethod
    def dimension(m: int, n: int) -> int:
        d = C.c_int64()
        _check(load().bh_dimension(int(m), int(n), C.byref(d)))
        return d.value

    @staticmethod
    def fixed_set_basis(m: int, n: int):
        """(tags[D], basis[m, D]) in the reference's column order."""
        b = Basis(m, n)
        return b.copy()

    @staticmethod
    def fixed_bosons_hamiltonian(neighbours, basis, tags, m: int, n: int, J: float, U: float,
                                 mu: float):
        """One term of H, selected as the reference selects it (hamiltonian.cpp:238-256):
        J T if J != 0, else U V, else -mu N; all zero prints an error and returns 0."""
        import sys

        import scipy.sparse as sp

        eps = np.finfo(float).eps
        D = BH.dimension(m, n)
        if abs(J) > eps:
            terms = (J, 0.0, 0.0)
        elif abs(U) > eps:
            terms = (0.0, U, 0.0)
        elif abs(mu) > eps:
            terms = (0.0, 0.0, mu)
        else:
            print("Error: At least one of the parameters J, U, mu must be different from zero.",
                  file=sys.stderr)
            return sp.csr_matrix((D, D))
        h = Hamiltonian(Basis(m, n), neighbours)
        H = h.csr(*terms)
        if terms[0] != 0.0:
            H.eliminate_zeros()  # hopping only: no diagonal entries, as fill_hopping
            return H
        # interaction / chemical term: one explicit entry per row, as fill_interaction
        d = H.diagonal()
        return sp.csr_matrix((d, np.arange(D, dtype=np.int32), np.arange(D + 1)), shape=(D, D))


# ---------------------------------------------------------------------------
# Op namespace mirror (operator.hpp:17-55)
# ---------------------------------------------------------------------------
class Op:
    @staticmethod
    def IRLM_eigen(O, nb_eigen: int, **opt):
        """Lowest nb_eigen eigenpairs of the symmetric matrix O, returned as the
        reference returns them: complex values ordered by descending |lambda|
        and the matching eigenvectors as complex columns.  Raises
        RuntimeError("Eigenvalue computation failed.") if not converged."""
        import scipy.sparse as sp

        A = sp.csr_matrix(O)
        A.sort_indices()
        D = A.shape[0]
        rp = np.ascontiguousarray(A.indptr, np.int64)
        ci = np.ascontiguousarray(A.indices, np.int32)
        val = np.ascontiguousarray(A.data, np.float64)
        o = default_opts(nev=nb_eigen, want_vectors=1, **opt)
        ev = np.zeros(nb_eigen)
        rs = np.zeros(nb_eigen)
        vec = np.zeros((nb_eigen, D))
        info = bh_solve_info()
        rc = load().bh_eigsh_csr(D, _ptr(rp), _ptr(ci), _ptr(val), C.byref(o), _ptr(ev), _ptr(rs),
                                 _ptr(vec), C.byref(info))
        if rc == BH_ERR_NOCONV:
            raise RuntimeError("Eigenvalue computation failed.")
        _check(rc)
        order = np.argsort(-np.abs(ev), kind="stable")
        return ev[order].astype(complex), vec[order].T.astype(complex)

    @staticmethod
    def FOLM_diag(O, nb_iter: int, v_0):
        """Op::FOLM_diag (operator.cpp:39-71): nb_iter Lanczos steps of the
        symmetric O from v_0 with full re-orthogonalisation, on the device in
        FP64 (bh_folm_diag_csr).  v_0 (float64 array) is normalised in place, as
        the reference does.  Returns T [nb_iter, nb_iter] (tridiagonal, zeros
        beyond the steps taken), V [D, nb_iter] (the Krylov vectors as
        columns, zeros beyond) and the number of steps (fewer than nb_iter
        after a breakdown, beta < 1e-6)."""
        import scipy.sparse as sp

        A = sp.csr_matrix(O)
        A.sort_indices()
        D = A.shape[0]
        if not (isinstance(v_0, np.ndarray) and v_0.dtype == np.float64 and v_0.flags.c_contiguous
                and v_0.shape == (D,)):
            raise TypeError("v_0 must be a contiguous float64 array of the matrix dimension")
        rp = np.ascontiguousarray(A.indptr, np.int64)
        ci = np.ascontiguousarray(A.indices, np.int32)
        val = np.ascontiguousarray(A.data, np.float64)
        T = np.zeros((nb_iter, nb_iter))
        V = np.zeros((nb_iter, D))  # column j of the reference's V is row j here
        steps = C.c_int()
        _check(load().bh_folm_diag_csr(D, _ptr(rp), _ptr(ci), _ptr(val), int(nb_iter), _ptr(v_0), _ptr(T),
                                       _ptr(V), C.byref(steps)))
        return T, np.ascontiguousarray(V.T), steps.value

    @staticmethod
    def FOLM_eigen(O, nb_iter: int, **opt):
        """Op::FOLM_eigen (operator.cpp:39-86) as intended: the lowest
        min(nb_iter, n - 2, 32) eigenpairs of the symmetric O by a fully
        re-orthogonalised Krylov method, real values ascending and the
        eigenvectors as real columns (the reference's own FOLM is unfinished
        and unused; this is the same solver as IRLM_eigen)."""
        n = O.shape[0]
        nev = max(1, min(int(nb_iter), n - 2, 32))
        vals, vecs = Op.IRLM_eigen(O, nev, **opt)
        order = np.argsort(vals.real, kind="stable")
        return vals.real[order], np.ascontiguousarray(vecs.real[:, order])


# ---------------------------------------------------------------------------
# Analysis namespace mirror (analysis.hpp)
# ---------------------------------------------------------------------------
def exact_eigen(O):
    """Op::exact_eigen: all eigenvalues (ascending) and eigenvectors (columns)."""
    A = np.asfortranarray(O.toarray() if hasattr(O, "toarray") else np.asarray(O), dtype=np.float64)
    n = A.shape[0]
    w = np.zeros(n)
    z = np.zeros((n, n), order="F")
    _check(load().bh_dense_eigh(n, _ptr(A), _ptr(w), z.ctypes.data_as(C.c_void_p)))
    return w, z


Op.exact_eigen = staticmethod(exact_eigen)


class Analysis:
    @staticmethod
    def gap_ratios(eigenvalues, nb_eigen: int) -> np.ndarray:
        ev = np.ascontiguousarray(np.real(np.asarray(eigenvalues))[:nb_eigen], np.float64)
        r = np.zeros(max(nb_eigen - 2, 1))
        mean = C.c_double()
        _check(load().bh_gap_ratios(nb_eigen, _ptr(ev), _ptr(r), C.byref(mean)))
        return r[: max(nb_eigen - 2, 0)]

    @staticmethod
    def coherence(spdm: np.ndarray) -> float:
        s = np.asarray(spdm)
        all_ = float(np.real(np.sum(s * s.T)))
        diag = float(np.real(np.sum(np.diag(s) ** 2)))
        return (all_ - diag) / all_

    @staticmethod
    def phase_map(m: int, n_lo: int, e0: np.ndarray, mu: np.ndarray):
        """density, compressibility [nJ, nmu] from e0[nsec, nJ] (mu = 0 energies)."""
        e0 = np.ascontiguousarray(e0, np.float64)
        mu = np.ascontiguousarray(mu, np.float64)
        nsec, nJ = e0.shape
        dens = np.zeros((nJ, len(mu)))
        kap = np.zeros((nJ, len(mu)))
        _check(load().bh_phase_map(m, n_lo, nsec, nJ, _ptr(e0), len(mu), _ptr(mu), _ptr(dens),
                                   _ptr(kap)))
        return dens, kap

    # ---- exact phase scan (analysis.cpp:207-427) ----
    @staticmethod
    def exact_parameters(m: int, n: int, J: float, U: float, mu: float, s: float, r: float,
                         fixed_param: str, path: str | None = "phase.txt", nb_eigen: int = 20,
                         precision: int = PREC_FP64, max_batch: int = 128):
        """Analysis::exact_parameters + calculate_and_save (analysis.cpp:207-427)
        on the device: the 1D periodic chain of m sites with n bosons; one of
        J, U, mu fixed ("J", "U", anything else = mu) and the other two swept
        over [x, x + r] in steps s (the parameter pairing of analysis.cpp:245-257);
        per grid point the lowest nb_eigen eigenvalues (batched solves), the
        mean gap ratio, and the condensate fraction and coherence of the
        single-particle density matrix of the eigenvector whose eigenvalue has
        the largest magnitude (the reference's first IRLM_eigen column).  The
        nb_eigen += 5 loop repeats while the gap-ratio variance stays at or below
        1e-8 of its mean (analysis.cpp:362-379).  Writes phase.txt like
        analysis.cpp:269-274, 384-387 when path is given.  Returns
        (param1, param2, gap_ratio, condensate_fraction, coherence) arrays."""
        import sys as _sys

        eps = np.finfo(float).eps
        if abs(J) < eps and abs(U) < eps and abs(mu) < eps:
            print("Error: At least one of the parameters J, U, mu must be different from zero.",
                  file=_sys.stderr)
            return None
        nb = Neighbours(m)
        nb.chain_neighbours()
        h = Hamiltonian(Basis(m, n), nb.getNeighbours())
        if fixed_param == "J":
            fixed_value, r1, r2 = J, (J, J + r), (mu, mu + r)
            point = lambda p1, p2: (J, p1, p2)  # noqa: E731  (H_fixed = J T, H1 = V, H2 = -N)
        elif fixed_param == "U":
            fixed_value, r1, r2 = U, (J, J + r), (U, U + r)
            point = lambda p1, p2: (p1, U, p2)  # noqa: E731  (H_fixed = U V, H1 = T, H2 = -N)
        else:
            fixed_value, r1, r2 = mu, (J, J + r), (mu, mu + r)
            point = lambda p1, p2: (p1, p2, mu)  # noqa: E731  (H_fixed = -mu N, H1 = T, H2 = V)
        n1 = int((r1[1] - r1[0]) / s) + 1
        n2 = int((r2[1] - r2[0]) / s) + 1
        P1 = np.zeros(n1 * n2)
        P2 = np.zeros(n1 * n2)
        for i in range(n1):  # row-major over (param1, param2); the reference indexes
            for j in range(n2):  # i * num_param1 + j, which equals this when n1 == n2
                P1[i * n2 + j] = r1[0] + i * s
                P2[i * n2 + j] = r2[0] + j * s
        pts = np.array([point(a, b) for a, b in zip(P1, P2)])
        while True:
            gap = np.zeros(len(P1))
            cf = np.zeros(len(P1))
            coh = np.zeros(len(P1))
            for k0 in range(0, len(P1), max_batch):
                sl = slice(k0, min(len(P1), k0 + max_batch))
                ev, _, nc, _, vec = h.eigsh_batch(pts[sl, 0], pts[sl, 1], pts[sl, 2], nev=nb_eigen,
                                                  vectors=True, precision=precision)
                for k in range(ev.shape[0]):
                    ratios = Analysis.gap_ratios(ev[k], nb_eigen)
                    gap[k0 + k] = ratios.sum() / len(ratios) if len(ratios) else 0.0
                    phi = vec[k, int(np.argmax(np.abs(ev[k])))]
                    rho = h.spdm(phi)
                    w = np.linalg.eigvalsh(rho)
                    cf[k0 + k] = abs(w[int(np.argmax(np.abs(w)))] / np.trace(rho))
                    coh[k0 + k] = Analysis.coherence(rho)
            mean = gap.mean()
            var = np.mean((gap - mean) ** 2)
            if var > 1e-8 * mean or nb_eigen + 5 > h.D:
                break
            nb_eigen += 5
        if path:
            with open(path, "w") as f:
                f.write(f"{fixed_param} {fixed_value:g}\n")
                for k in range(len(P1)):
                    f.write(f"{P1[k]:g} {P2[k]:g} {gap[k]:g} {cf[k]:g} {coh[k]:g}\n")
        return P1, P2, gap, cf, coh

    # ---- mean field (analysis.cpp:58-178) ----
    @staticmethod
    def SCMF(mu, J, q: int, psi0, precision: int):
        """Self-consistent mean-field order parameter for each (mu, J, psi0)
        point (arrays broadcast together); returns (psi, iterations)."""
        mu, J, psi0 = np.broadcast_arrays(np.asarray(mu, np.float64), np.asarray(J, np.float64),
                                          np.asarray(psi0, np.float64))
        shape = mu.shape
        mu, J, psi0 = (np.ascontiguousarray(a.ravel()) for a in (mu, J, psi0))
        psi = np.zeros(mu.size)
        it = np.zeros(mu.size, np.int32)
        _check(load().bh_scmf(mu.size, _ptr(mu), _ptr(J), q, _ptr(psi0), precision, _ptr(psi),
                              _ptr(it)))
        return psi.reshape(shape), it.reshape(shape)

    @staticmethod
    def mean_field_parameters(n: int, precision: int, q: int = 1, seed: int = 0,
                              path: str | None = None):
        """The reference's mean-field sweep (mu in [0, 4), J in [0, 0.25), n
        steps each): returns (mu, J, psi[len(mu), len(J)]) and, with path,
        writes the reference's "mu J psi" lines (mean_field.txt)."""
        mu = np.zeros(n + 1)
        J = np.zeros(n + 1)
        psi = np.zeros((n + 1) * (n + 1))
        a, b = C.c_int(), C.c_int()
        _check(load().bh_mean_field_grid(n, precision, q, seed, C.byref(a), C.byref(b), _ptr(mu),
                                         _ptr(J), _ptr(psi)))
        mu, J = mu[: a.value], J[: b.value]
        psi = psi[: a.value * b.value].reshape(a.value, b.value)
        if path:
            with open(path, "w") as f:
                for i, x in enumerate(mu):
                    for k, y in enumerate(J):
                        f.write(f"{x:g} {y:g} {psi[i, k]:g}\n")
        return mu, J, psi
