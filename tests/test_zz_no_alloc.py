"""GPU: the allocation-free apply entry point.

bh_hamiltonian_apply_noalloc serves callers that cannot allocate device memory
while they run (their device memory comes from a pool they set up once, or
many host threads share the GPU and must not serialise on cudaMalloc/cudaFree).
The caller passes device input/output buffers and a stream; the library uses a
fixed device array for its working memory.  This test allocates the caller's
buffers with torch (the caller's side), calls the entry point through the C ABI
twice in a row (the fixed array keeps the first call's contents) and compares
with the allocating entry point bh_hamiltonian_apply on the same inputs.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import chain_lists

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-13, 1e-13  # FP64 SpMV, same kernel and order of summation


def _call(pkg, h, order, J, U, mu, x):
    import torch

    lib = pkg.load()
    xd = torch.tensor(np.ascontiguousarray(x), dtype=torch.float64, device="cuda")
    yd = torch.full_like(xd, float("nan"))
    stream = torch.cuda.current_stream()
    rc = lib.bh_hamiltonian_apply_noalloc(h._h, order, J, U, mu, x.shape[1],
                                          C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()),
                                          C.c_void_p(stream.cuda_stream))
    return rc, yd.cpu().numpy()


def test_noalloc_apply_matches_allocating_apply(pkg):
    pytest.importorskip("torch")
    m, n = 8, 6
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    cases = [(pkg.ORDER_REFERENCE, 0.1, 1.0, 0.5, 3, 11), (pkg.ORDER_REFERENCE, 0.27, 0.6, 0.2, 2, 12),
             (pkg.ORDER_LEX, 0.05, 1.3, 0.0, 1, 13)]
    for order, J, U, mu, nvec, seed in cases:  # consecutive calls share the fixed array
        x = np.random.RandomState(seed).randn(h.D, nvec)
        y_ref = h.apply(x, J, U, mu, order=order)
        rc, y = _call(pkg, h, order, J, U, mu, x)
        assert rc == pkg.BH_OK, pkg.load().bh_last_error()
        np.testing.assert_allclose(y, y_ref, rtol=RTOL, atol=ATOL)


def test_noalloc_apply_rejects_sizes_beyond_the_fixed_scratch(pkg):
    pytest.importorskip("torch")
    m, n = 8, 6
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    nvec = (4 << 20) // (2 * h.D) + 1  # 2 D nvec just above 4 Mi doubles
    x = np.zeros((h.D, nvec))
    rc, _ = _call(pkg, h, pkg.ORDER_REFERENCE, 0.1, 1.0, 0.0, x)
    assert rc == pkg.BH_ERR_ARG
    assert b"exceeds the fixed scratch" in pkg.load().bh_last_error()


def test_noalloc_apply_rejects_overlapping_buffers_in_lex_order(pkg):
    # the lexicographic product reads rows of x while it writes y: one buffer
    # for both is refused before any launch
    import torch

    m, n = 6, 4
    h = pkg.Hamiltonian(pkg.Basis(m, n), chain_lists(m))
    xd = torch.zeros((h.D, 2), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    lib = pkg.load()
    rc = lib.bh_hamiltonian_apply_noalloc(h._h, pkg.ORDER_LEX, 0.1, 1.0, 0.0, 2,
                                          C.c_void_p(xd.data_ptr()), C.c_void_p(xd.data_ptr()),
                                          C.c_void_p(stream.cuda_stream))
    assert rc == pkg.BH_ERR_ARG
    assert b"overlap" in lib.bh_last_error()
