"""Learned T2 guess: the network's kernels against the CPU oracle, and its gain.

Forward, loss and every parameter gradient of the hand-written kernels are compared with
oracle/mlp.py on the same FP16-rounded weights; the pair features and targets with the
oracle's restatement; and on a family of uneven-size Hamiltonians the trained network
must save CCSD iterations over the MP2 guess while the plain iteration still converges
to the same energy.
"""
import numpy as np
import pytest

import ugacc_gb300 as U
from oracle import mlp as M
from ugacc_gb300.generator import make_family, make_hamiltonian

pytestmark = pytest.mark.gpu


def _data(rows, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(0, 1, (rows, M.F)).astype(np.float32), rng.normal(0, 1, rows).astype(np.float32)


def test_forward_matches_oracle():
    net = U.MLP(seed=5)
    X, _ = _data(2500, 1)
    y = net.predict(X)
    yref, _ = M.forward(net.params.astype(np.float64), X.astype(np.float64))
    np.testing.assert_allclose(y, yref, rtol=0, atol=1e-4 * np.abs(yref).max())


def test_loss_and_gradients_match_oracle():
    net = U.MLP(seed=7)
    X, t = _data(3000, 2)
    loss, g = net.loss_grad(X, t)
    lref, gref = M.loss_grad(net.params.astype(np.float64), X.astype(np.float64), t.astype(np.float64))
    assert abs(loss - lref) <= 1e-5 * lref
    o = 0
    for name, shape in M.SIZES:  # every parameter block on its own scale
        n = int(np.prod(shape))
        np.testing.assert_allclose(g[o:o + n], gref[o:o + n], rtol=0, atol=1e-4 * np.abs(gref[o:o + n]).max() + 1e-9,
                                   err_msg=name)
        o += n


def test_features_and_targets_match_oracle():
    h = make_hamiltonian(4, 20, 3)
    H = U.Hamiltonian.from_synthetic(h)
    no, nv = h.no, h.nv
    ints = h.ints_physicist()
    blocks = dict(M.blocks(ints, no), eps=h.eps)
    np.testing.assert_allclose(U.mlp_features(H), M.features(no, nv, blocks), rtol=2e-7, atol=1e-7)
    cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10})
    cc.compute_energy()
    X, t = U.mlp_features(H, with_targets=True)
    np.testing.assert_allclose(t, M.targets(no, nv, blocks["oovv"], h.eps, cc.t2), rtol=1e-6, atol=1e-5)


@pytest.mark.parametrize("no,nv", [(4, 40), (3, 27)])
def test_tensor_core_guess_matches_oracle(no, nv):
    """The fused guess kernel (features, both layers and t2 = t2_mp2 + y/1000 in one pass,
    second layer on the tensor cores with FP16 activations) against the oracle's forward
    pass with the same FP16 rounding, and against the FP32 inference path; nv = 27 leaves
    a partial last tile of 128 elements."""
    h = make_hamiltonian(no, nv, 3)
    H = U.Hamiltonian.from_synthetic(h)
    net = U.MLP(seed=9)
    net.guess(H)
    g = H.ctx.get("t2_guess", (no, no, nv, nv))
    blocks = dict(M.blocks(h.ints_physicist(), no), eps=h.eps)
    X = M.features(no, nv, blocks)
    y, _ = M.forward(net.params.astype(np.float64), X, half_activations=True)
    D = M._denominators(no, nv, h.eps)
    mp2 = blocks["oovv"] / D
    dy = (g - mp2).ravel() * M.TARGET - y
    # tanh-based SiLU (tanh.approx, ~2^-11) and FP32 features: a few 1e-3 of the output scale
    assert np.abs(dy).max() <= 4e-3 * np.abs(y).max(), (np.abs(dy).max(), np.abs(y).max())
    y32 = net.predict(U.mlp_features(H))
    assert np.abs((g - mp2).ravel() * M.TARGET - y32).max() <= 4e-3 * np.abs(y32).max()
    # the next solve starts from it and the plain iteration decides the answer
    e_guess = U.CCWfn(H, {"R_CONVERGENCE": 1e-10}).compute_energy()
    e_mp2 = U.CCWfn(H, {"R_CONVERGENCE": 1e-10}).compute_energy()
    assert abs(e_guess - e_mp2) < 1e-9


def test_training_lowers_the_loss():
    net = U.MLP(seed=1)
    rng = np.random.default_rng(4)
    X = rng.normal(0, 1, (20000, M.F)).astype(np.float32)
    t = (np.tanh(X[:, 0]) * X[:, 3] + 0.3 * X[:, 1]).astype(np.float32)
    before, _ = net.loss_grad(X, t)
    net.train(X, t, epochs=8, batch=1024, lr=2e-3, seed=0)
    after, _ = net.loss_grad(X, t)
    assert after < 0.2 * before


def _solve(h, guess=None):
    H = U.Hamiltonian.from_synthetic(h)
    if guess is not None:
        guess.guess(H)
    cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-8})
    e = cc.compute_energy()
    return H, cc, e, H.ctx.stats()["ccsd_iterations"]


def test_learned_guess_saves_iterations():
    fam = make_family(24, seed=11, no_range=(4, 8), nv_range=(20, 48))
    train, test = fam[:16], fam[16:]
    Xs, ts = [], []
    for h in train:
        H, cc, _, _ = _solve(h)
        X, t = U.mlp_features(H, with_targets=True)
        Xs.append(X)
        ts.append(t)
    net = U.MLP(seed=3)
    net.train(np.concatenate(Xs), np.concatenate(ts), epochs=12, batch=4096, lr=1e-3, seed=0)
    it_mp2, it_mlp = [], []
    for h in test:
        _, _, e0, n0 = _solve(h)
        _, _, e1, n1 = _solve(h, guess=net)
        assert abs(e1 - e0) < 1e-7  # the plain iteration decides the answer
        it_mp2.append(n0)
        it_mlp.append(n1)
    print("iterations MP2 guess", it_mp2, "learned guess", it_mlp)
    assert sum(it_mlp) < sum(it_mp2)


def test_family_workflow_batched_learned_guess():
    from ugacc_gb300 import family
    out = family.run(members=24, train=16, seed=11, r_conv=1e-8, epochs=8, row_fraction=1.0, no_range=(4, 8),
                     nv_range=(20, 48))
    print(out)
    assert out["all_members"]["converged"] == 24
    assert out["test_learned_guess"]["converged"] == out["test_mp2_guess"]["converged"] == 8
    assert out["max_abs_dE"] < 1e-7
    assert out["iterations_saved"] > 0
