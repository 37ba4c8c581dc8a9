"""GPU: the thick-restart rotation of the FP32 Krylov basis on the tensor
cores (tcgen05.mma kind::tf32 with three-piece TF32 splits, bh_rotate_tc.cu,
BH_TC_ROTATE=1) against the SIMT rotation (the default, BH_TC_ROTATE=0), each in
a child process because the switch is read once per process.  Both solves must give the FP64 path's
eigenvalues within 1e-8 (pure relative), for block sizes 1, 2 and 4 (the
tensor-core kernel's three layouts of a basis row).  Block 1 runs on the open
chain: the periodic chain's degenerate pairs need a block of 2 (one Krylov
vector finds one copy of a pair, and FP32 rounding can add a spurious second
copy that FP64 does not)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import chain_lists

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = [  # (m, n, lattice, block, nJ, nev)
    (10, 9, "chain", 2, 32, 10),
    (9, 7, "open", 1, 8, 6),
    (16, 5, "square", 4, 8, 4),
]

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, {root!r})
import __graft_entry__ as g
pkg = g.load_package(); pkg.load()
out = []
for m, n, lat, block, nj, nev in {cases!r}:
    nb = pkg.Neighbours(m)
    if lat == "square":
        nb.square_neighbours()
    else:
        nb.chain_neighbours(lat == "chain")
    h = pkg.Hamiltonian(pkg.Basis(m, n), nb.getNeighbours())
    Js = 0.3 * (np.arange(nj) + 1) / nj
    ev, _, nc, info = h.eigsh_batch(Js, 1.0, 0.0, nev=nev, block=block, precision=pkg.PREC_MIXED)
    out.append({{"ev": ev.tolist(), "nc": nc.tolist(), "restarts": info.restarts}})
print(json.dumps(out))
"""


def _solve_all(env_tc: str):
    env = dict(os.environ, BH_TC_ROTATE=env_tc)
    code = CHILD.format(root=ROOT, cases=CASES)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_tensor_core_rotation_matches_simt_and_fp64(pkg):
    tc = _solve_all("1")
    simt = _solve_all("0")
    for (m, n, lat, block, nj, nev), a, b in zip(CASES, tc, simt):
        nb = pkg.Neighbours(m)
        if lat == "square":
            nb.square_neighbours()
        else:
            nb.chain_neighbours(lat == "chain")
        h = pkg.Hamiltonian(pkg.Basis(m, n), nb.getNeighbours())
        Js = 0.3 * (np.arange(nj) + 1) / nj
        ev64, _, nc64, _ = h.eigsh_batch(Js, 1.0, 0.0, nev=nev, block=block, precision=pkg.PREC_FP64)
        ea, eb = np.array(a["ev"]), np.array(b["ev"])
        assert min(a["nc"]) == nev and min(b["nc"]) == nev
        for name, e in (("tensor cores", ea), ("SIMT", eb)):
            rel = np.abs(e - ev64) / np.abs(ev64)
            assert rel.max() < 1e-8, (name, m, n, lat, block, rel.max())
