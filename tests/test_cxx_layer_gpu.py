"""GPU: the C++ layer under the Eigen-typed drop-in (include/bh_cxx.hpp), run
the way the reference runs Op::IRLM_eigen (operator.cpp:22-33): from several
OpenMP threads at once, as its grid loop does (analysis.cpp:302-314).  The
Eigen-typed wrapper itself (include/bh_reference_api.hpp) needs the Eigen
headers, which only the reference tree provides; its compile-and-link test is
tests/test_reference_api_build.py.  Checked here: the golden m = n = 8 values
in the reference's result order (descending |lambda|), concurrent results
equal to sequential ones bit for bit, the exception texts of a solve that does
not converge and of an invalid nev."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import reference_lowest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver(pkg, tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    lib = pkg.lib_path()
    exe = str(tmp_path_factory.mktemp("cxx") / "irlm_concurrent")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-fopenmp", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cxx", "irlm_concurrent.cpp"), "-o", exe, lib,
                        f"-Wl,-rpath,{os.path.dirname(lib)}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def test_concurrent_irlm_eigen_like_the_reference_grid_loop(driver, golden):
    nthreads = 8
    r = subprocess.run([driver, str(nthreads)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = r.stdout.splitlines()
    points = [l.split() for l in lines if l.startswith("point ")]
    assert len(points) == 2 * nthreads
    # point 0: J = 0.1, U = 1, mu = 0.5, the golden m8n8 case
    got = np.array([float(x) for x in points[0][4:]])
    want = np.array(reference_lowest(golden["irlm"]["m8n8"]))
    want = want[np.argsort(-np.abs(want), kind="stable")]
    assert np.max(np.abs(got - want) / np.abs(want)) < 1e-10
    # every point in descending |lambda| order
    for p in points:
        v = np.abs(np.array([float(x) for x in p[4:]]))
        assert np.all(np.diff(v) <= 0)
    # each call's result does not depend on what ran beside it
    same = [l.split() for l in lines if l.startswith("same ")]
    assert all(s[2] == "1" for s in same), same
    noconv = [l.split(" ", 2)[2] for l in lines if l.startswith("noconv ")]
    assert noconv == ["Eigenvalue computation failed."] * nthreads
    badarg = [l for l in lines if l.startswith("badarg ")]
    assert badarg == ["badarg nev must satisfy 1 <= nev <= n - 2, n is the size of matrix"]
    # Op::FOLM_diag through the C++ layer: orthonormal Krylov vectors and a
    # tridiagonal matrix whose lowest Ritz value approaches the ground state
    # from above (30 steps from this start: 2.9e-6 relative; the 40-step
    # convergence check is in tests/test_folm_gpu.py)
    folm = [l.split() for l in lines if l.startswith("folm ")]
    assert len(folm) == 1
    steps, orth = int(folm[0][1]), float(folm[0][2])
    vals = np.array([float(x) for x in folm[0][3:]])
    assert steps == 30 and orth < 1e-12
    T = np.diag(vals[:30]) + np.diag(vals[30:], 1) + np.diag(vals[30:], -1)
    e0, ritz0 = np.min(got), np.linalg.eigvalsh(T)[0]
    assert e0 - 1e-12 * abs(e0) <= ritz0 < e0 + 1e-4 * abs(e0)
