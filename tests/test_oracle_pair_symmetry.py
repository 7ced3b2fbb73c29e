"""Why the mixed solve projects R2 onto the pair-symmetric subspace (oracle, CPU).

Around the converged amplitudes, a T2 perturbation that is antisymmetric under
(i,j,a,b) -> (j,i,b,a) is barely damped by the Jacobi step (the Fock terms of the
symmetrised residual cancel in that sector), while a symmetric one is damped strongly:
here one step keeps ~70 % of an antisymmetric perturbation and ~1 % of a symmetric one.
Rounding noise of tensor-core products lands in both sectors; left in R2 its
antisymmetric part accumulates instead of decaying.
"""
import numpy as np

from oracle import cc as O
from ugacc_gb300.generator import make_hamiltonian


def _jacobi_gain(cc, t1s, t2s, d2):
    cc.t1, cc.t2 = t1s.copy(), t2s + d2
    cc.build_tau()
    _, t2n, _ = cc.iterate_once()
    cc.t1, cc.t2 = t1s.copy(), t2s.copy()
    cc.build_tau()
    _, t2ref, _ = cc.iterate_once()
    return np.linalg.norm(t2n - t2ref) / np.linalg.norm(d2)


def test_antisymmetric_pair_sector_is_not_damped():
    h = make_hamiltonian(4, 18, 5)
    H = O.Hamiltonian(h)
    cc = O.CCWfn(H, r_convergence=1e-12)
    cc.compute_energy()
    t1s, t2s = cc.t1.copy(), cc.t2.copy()
    rng = np.random.default_rng(0)
    X = rng.standard_normal(t2s.shape) * 1e-6
    sym = 0.5 * (X + X.transpose(1, 0, 3, 2))
    anti = 0.5 * (X - X.transpose(1, 0, 3, 2))
    g_sym = _jacobi_gain(cc, t1s, t2s, sym)
    g_anti = _jacobi_gain(cc, t1s, t2s, anti)
    assert g_sym < 0.05
    assert g_anti > 0.5
    assert g_anti > 20.0 * g_sym
