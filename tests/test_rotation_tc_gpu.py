"""GPU: the thick-restart rotation of the FP32 Krylov basis on the tensor
cores -- tcgen05.mma kind::tf32 with three-piece TF32 splits (bh_rotate_tc.cu,
BH_TC_ROTATE=1), and the TMA-streamed, warp-specialised form with two-piece
splits (bh_rotate_tma.cu, for the restarts at which every solve continues:
the default, the split operand in tensor memory, or BH_TMA_ROTATE=1, in
shared memory) -- against the SIMT rotation (BH_TMA_ROTATE=0), each in a child
process because the switches are read once per process.  Every solve must give the FP64 path's
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


MODES = {"tensor cores": {"BH_TC_ROTATE": "1", "BH_TMA_ROTATE": "0"},
         "TMA, operand in shared memory": {"BH_TC_ROTATE": "0", "BH_TMA_ROTATE": "1"},
         "TMA, operand in tensor memory (default)": {"BH_TC_ROTATE": "0", "BH_TMA_ROTATE": "2"},
         "SIMT": {"BH_TC_ROTATE": "0", "BH_TMA_ROTATE": "0"}}


def _solve_all(mode: str):
    env = dict(os.environ, **MODES[mode])
    code = CHILD.format(root=ROOT, cases=CASES)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_tensor_core_rotation_matches_simt_and_fp64(pkg):
    res = {mode: _solve_all(mode) for mode in MODES}
    for k, (m, n, lat, block, nj, nev) in enumerate(CASES):
        nb = pkg.Neighbours(m)
        if lat == "square":
            nb.square_neighbours()
        else:
            nb.chain_neighbours(lat == "chain")
        h = pkg.Hamiltonian(pkg.Basis(m, n), nb.getNeighbours())
        Js = 0.3 * (np.arange(nj) + 1) / nj
        ev64, _, nc64, _ = h.eigsh_batch(Js, 1.0, 0.0, nev=nev, block=block, precision=pkg.PREC_FP64)
        for mode in MODES:
            r = res[mode][k]
            assert min(r["nc"]) == nev, (mode, m, n, lat, block)
            rel = np.abs(np.array(r["ev"]) - ev64) / np.abs(ev64)
            assert rel.max() < 1e-8, (mode, m, n, lat, block, rel.max())
