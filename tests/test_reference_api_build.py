"""CPU: the C++ drop-in (include/bh_reference_api.hpp) replaces the reference's
src/hamiltonian.cpp, src/neighbours.cpp and src/operator.cpp: the reference's
own main.cpp / analysis.cpp / resource.cpp compile against it and link with
libbhgb300.so.  Needs the reference tree (its headers and vendored Eigen /
Spectra); skipped where it is absent.  Running the program needs a GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("BH_REFERENCE_TREE", "/root/reference")

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")) or shutil.which("g++") is None,
                                reason="reference tree not available")

BACKEND_TU = """
#include "hamiltonian.hpp"
#include "neighbours.hpp"
#include "operator.hpp"
#define BH_GB300_IMPLEMENTATION
#include "bh_reference_api.hpp"
"""


def test_reference_program_links_against_the_dropin(tmp_path, pkg):
    lib = pkg.lib_path()
    (tmp_path / "gb300_backend.cpp").write_text(BACKEND_TU)
    inc = ["-I", os.path.join(REF, "include"), "-I", os.path.join(REF, "external/spectra/include"),
           "-I", os.path.join(ROOT, "include")]
    objs = []
    for src in [str(tmp_path / "gb300_backend.cpp"), os.path.join(REF, "src/main.cpp"),
                os.path.join(REF, "src/analysis.cpp"), os.path.join(REF, "src/resource.cpp")]:
        obj = str(tmp_path / (os.path.basename(src) + ".o"))
        r = subprocess.run(["g++", "-std=gnu++20", "-O1", "-w", "-fopenmp", *inc, "-c", src, "-o", obj],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        objs.append(obj)
    exe = str(tmp_path / "QuantumProject_gb300")
    r = subprocess.run(["g++", "-fopenmp", "-o", exe, *objs, lib, f"-Wl,-rpath,{os.path.dirname(lib)}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    # every symbol the reference's exact path needs is defined by the drop-in
    nm = subprocess.run(["nm", "-C", str(tmp_path / "gb300_backend.cpp.o")], capture_output=True, text=True).stdout
    for sym in ["BH::fixed_set_basis", "BH::fixed_bosons_hamiltonian", "BH::max_bosons_hamiltonian",
                "BH::max_set_basis", "BH::calculate_tag", "BH::search_tag", "BH::h_MF",
                "Neighbours::chain_neighbours", "Neighbours::square_neighbours",
                "Neighbours::getNeighbours", "Op::IRLM_eigen", "Op::FOLM_diag", "Op::FOLM_eigen", "Op::exact_eigen"]:
        assert sym in nm, sym
