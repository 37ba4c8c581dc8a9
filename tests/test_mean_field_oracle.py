"""CPU: the oracle's restatement of the self-consistent mean field
(Analysis::SCMF, src/analysis.cpp:111-178) against golden values recorded
from the reference itself (tests/golden/make_golden.py)."""
import numpy as np


def test_oracle_scmf_matches_reference_golden(orc, golden):
    for c in golden["scmf"]:
        psi, it = orc.scmf(c["mu"], c["J"], c["q"], c["psi0"], c["precision"])
        eps = 10.0 ** -c["precision"]
        assert it >= 1
        assert abs(psi - c["psi"]) <= 10 * eps, c


def test_oracle_scmf_batch_equals_single_points(orc, golden):
    cs = golden["scmf"][:20]
    mu = np.array([c["mu"] for c in cs])
    J = np.array([c["J"] for c in cs])
    psi0 = np.array([c["psi0"] for c in cs])
    psi, outer = orc.scmf_batch(mu, J, 1, psi0, 6)
    for k, c in enumerate(cs):
        assert psi[k] == orc.scmf(c["mu"], c["J"], 1, c["psi0"], 6)[0]
