"""The MLP oracle's analytic gradient against central finite differences (CPU)."""
import numpy as np

from oracle import mlp as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = rng.normal(0, 0.1, M.num_params())
    X = rng.normal(0, 1, (37, M.F))
    t = rng.normal(0, 1, 37)
    loss, g = M.loss_grad(p, X, t, half_weights=False)
    idx = rng.choice(p.size, 40, replace=False)
    h = 1e-6
    for k in idx:
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (M.loss_grad(pp, X, t, half_weights=False)[0] - M.loss_grad(pm, X, t, half_weights=False)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])
    assert loss > 0


def test_oracle_features_layout():
    from ugacc_gb300.generator import make_hamiltonian
    h = make_hamiltonian(3, 5, 0)
    ints = h.ints_physicist()
    V = dict(M.blocks(ints, 3), eps=h.eps)
    F = M.features(3, 5, V)
    assert F.shape == (3 * 3 * 5 * 5, M.F)
    i, j, a, b = 1, 2, 4, 0
    r = ((i * 3 + j) * 5 + a) * 5 + b
    D = h.eps[i] + h.eps[j] - h.eps[3 + a] - h.eps[3 + b]
    A, B = 3 + a, 3 + b
    assert np.isclose(F[r, 0], M.SCALE * ints[i, j, A, B] / D)
    assert np.isclose(F[r, 1], M.SCALE * ints[i, j, B, A] / D)
    assert F[r, 6] == 0 and F[r, 7] == 0
    assert np.isclose(F[r, 8], M.SCALE * ints[A, B, A, B])
    assert np.isclose(F[r, 9], M.SCALE * ints[i, j, i, j])
    assert np.isclose(F[r, 10], M.SCALE * (ints[i, A, i, A] + ints[j, B, j, B]))
    assert np.isclose(F[r, 11], M.SCALE * (ints[i, i, A, A] + ints[j, j, B, B]))
    assert np.isclose(F[r, 14], 0.25 * (h.eps[i] - h.eps[j]) * (h.eps[A] - h.eps[B]))
    # invariance under the pair swap (i,j,a,b) -> (j,i,b,a)
    rs = ((j * 3 + i) * 5 + b) * 5 + a
    np.testing.assert_allclose(F[rs], F[r])
