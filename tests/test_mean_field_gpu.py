"""GPU: the mean-field sweep (one device thread per (mu, J) point) against
the reference's own SCMF values and the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _splitmix_uniform(seed, k):
    m = (1 << 64) - 1
    z = (seed + 0x9E3779B97F4A7C15 * (k + 1)) & m
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
    z ^= z >> 31
    return (z >> 11) * (1.0 / 9007199254740992.0)


def test_scmf_matches_reference_golden(pkg, golden):
    for q in (1, 2, 4):
        cs = [c for c in golden["scmf"] if c["q"] == q]
        prec = cs[0]["precision"]
        mu = np.array([c["mu"] for c in cs])
        J = np.array([c["J"] for c in cs])
        psi0 = np.array([c["psi0"] for c in cs])
        psi, it = pkg.Analysis.SCMF(mu, J, q, psi0, prec)
        want = np.array([c["psi"] for c in cs])
        assert np.all(it >= 1)
        # both sides stop once psi moves by <= eps; they agree far below that
        np.testing.assert_allclose(psi, want, rtol=0, atol=10 * 10.0 ** -prec)


def test_scmf_matches_oracle_on_random_points(pkg, orc):
    rng = np.random.RandomState(3)
    n = 400
    mu = rng.uniform(0.0, 4.0, n)
    J = rng.uniform(0.002, 0.25, n)
    psi0 = rng.uniform(0.01, 1.0, n)
    psi, it = pkg.Analysis.SCMF(mu, J, 1, psi0, 8)
    po, _ = orc.scmf_batch(mu, J, 1, psi0, 8)
    assert np.all(it >= 1)
    np.testing.assert_allclose(psi, po, rtol=0, atol=1e-7)


def test_mean_field_grid_like_reference_sweep(pkg, orc, tmp_path):
    n, prec, seed = 40, 6, 5
    path = tmp_path / "mean_field.txt"
    mu, J, psi = pkg.Analysis.mean_field_parameters(n, prec, q=1, seed=seed, path=str(path))
    # the reference's loops: x = 0; x += dx while x < max
    mus, x = [], 0.0
    while x < 4.0:
        mus.append(x)
        x += 4.0 / n
    js, x = [], 0.0
    while x < 0.25:
        js.append(x)
        x += 0.25 / n
    assert mu.tolist() == mus and J.tolist() == js
    lines = path.read_text().splitlines()
    assert len(lines) == len(mus) * len(js)
    assert lines[1].split()[0] == "0" and float(lines[1].split()[1]) == js[1]
    # same points through the oracle with the same seeds
    M, JJ = np.meshgrid(mu, J, indexing="ij")
    seeds = np.array([_splitmix_uniform(seed, k) for k in range(M.size)])
    po, _ = orc.scmf_batch(M.ravel(), JJ.ravel(), 1, seeds, prec)
    np.testing.assert_allclose(psi.ravel(), po, rtol=0, atol=1e-5)
    # J = 0 column: no hopping, psi = 0; deep in the first Mott lobe psi -> 0
    assert np.all(psi[:, 0] == 0.0)
    lobe = (M > 0.3) & (M < 0.7) & (JJ < 0.02) & (JJ > 0)
    assert np.all(np.abs(psi[lobe]) < 1e-3)
    assert psi.max() > 0.5
