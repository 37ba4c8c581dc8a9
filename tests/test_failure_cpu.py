"""CPU: failure detection that needs no GPU.  The reference raises on bad
arguments (Spectra GenEigsBase.h:335-339, std::invalid_argument) and on
non-convergence (operator.cpp:27-29); the C ABI rejects non-finite inputs with
BH_ERR_ARG before any device work, so these calls return without touching a
GPU."""
import ctypes as C

import numpy as np


def _csr_call(pkg, val, tol=0.0):
    lib = pkg.load()
    D = 4
    rp = np.array([0, 2, 4, 6, 8], np.int64)
    ci = np.array([0, 1, 0, 1, 2, 3, 2, 3], np.int32)
    v = np.ascontiguousarray(val, np.float64)
    o = pkg.default_opts(nev=1, tol=tol)
    ev = np.zeros(1)
    info = pkg.bh_solve_info()
    return lib.bh_eigsh_csr(D, pkg._ptr(rp), pkg._ptr(ci), pkg._ptr(v), C.byref(o), pkg._ptr(ev),
                            None, None, C.byref(info))


def test_eigsh_csr_rejects_non_finite_values(pkg):
    lib = pkg.load()
    for bad in (np.nan, np.inf, -np.inf):
        val = np.array([2.0, 1.0, 1.0, 2.0, 3.0, bad, bad, 3.0])
        assert _csr_call(pkg, val) == pkg.BH_ERR_ARG
        assert b"finite" in lib.bh_last_error()


def test_solver_options_reject_non_finite_tolerance(pkg):
    lib = pkg.load()
    val = np.array([2.0, 1.0, 1.0, 2.0, 3.0, 0.5, 0.5, 3.0])
    for tol in (np.nan, np.inf, -1.0):
        assert _csr_call(pkg, val, tol=tol) == pkg.BH_ERR_ARG
        assert b"tol" in lib.bh_last_error()


def test_phase_map_rejects_non_finite_energies(pkg):
    lib = pkg.load()
    e0 = np.array([[-1.0, np.nan]])
    mu = np.linspace(0, 1, 4)
    d = np.zeros((2, 4))
    k = np.zeros((2, 4))
    rc = lib.bh_phase_map(4, 2, 1, 2, pkg._ptr(e0), 4, pkg._ptr(mu), pkg._ptr(d), pkg._ptr(k))
    assert rc == pkg.BH_ERR_ARG and b"e0" in lib.bh_last_error()
    e0 = np.array([[-1.0, -2.0]])
    mu[2] = np.inf
    rc = lib.bh_phase_map(4, 2, 1, 2, pkg._ptr(e0), 4, pkg._ptr(mu), pkg._ptr(d), pkg._ptr(k))
    assert rc == pkg.BH_ERR_ARG and b"mu" in lib.bh_last_error()


def test_batch_status_needs_its_output(pkg):
    lib = pkg.load()
    J = np.array([0.1])
    o = pkg.default_opts(nev=1)
    ev = np.zeros(1)
    rc = lib.bh_eigsh_batch_status(None, 1, pkg._ptr(J), pkg._ptr(J), pkg._ptr(J), C.byref(o),
                                   pkg._ptr(ev), None, None, None, None)
    assert rc == pkg.BH_ERR_ARG
