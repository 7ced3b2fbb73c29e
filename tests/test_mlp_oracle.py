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
    V = h.ints_physicist()[:3, :3, 3:, 3:]
    F = M.features(3, 5, V, h.eps)
    assert F.shape == (3 * 3 * 5 * 5, 8)
    r = ((1 * 3 + 2) * 5 + 4) * 5 + 0  # (i, j, a, b) = (1, 2, 4, 0)
    D = h.eps[1] + h.eps[2] - h.eps[3 + 4] - h.eps[3 + 0]
    assert np.isclose(F[r, 0], M.SCALE * V[1, 2, 4, 0] / D)
    assert np.isclose(F[r, 1], M.SCALE * V[1, 2, 0, 4] / D)
    assert F[r, 6] == 0 and F[r, 7] == 0
