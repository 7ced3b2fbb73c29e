"""CCSD(T) on the active space of an MO-integral file (frozen core and frozen virtual
orbitals, hamiltonian.cc:21-102) against the numpy oracle on the same active block."""
import dataclasses

import numpy as np
import pytest

import ugacc_gb300 as U
from oracle import cc as O
from oracle import fcidump as FD
from ugacc_gb300.generator import make_hamiltonian

pytestmark = pytest.mark.gpu


def test_frozen_orbitals_ccsd_t_from_fcidump(tmp_path):
    ham = make_hamiltonian(6, 22, seed=9)
    eri = ham.eri_chemist()
    h = FD.core_hamiltonian_for(ham.fock, eri, ham.no)
    path = str(tmp_path / "FCIDUMP")
    FD.write(path, h, eri, 2.5, 2 * ham.no, scramble=True)
    H = U.Hamiltonian.from_fcidump(path, nfzc=1, nfzv=3)
    assert (H.no, H.nv) == (5, 19)
    _, _, _, efzc, escf = FD.hamiltonian(h, eri, 2.5, ham.no, 1, 3)
    assert abs(H.efzc - efzc) < 1e-12 and abs(H.escf - escf) < 1e-12
    cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "MAXITER": 100})
    cc.compute_energy()
    # the same active block, from the generator's own factors
    act = dataclasses.replace(ham, no=5, nv=19, eps=ham.eps[1:-3].copy(), B=np.ascontiguousarray(ham.B[:, 1:-3, 1:-3]))
    ref = O.CCWfn(O.Hamiltonian(act), maxiter=100, r_convergence=1e-10)
    ref.compute_energy()
    assert abs(cc.eccsd - ref.eccsd) < 1e-10
    np.testing.assert_allclose(cc.t2, ref.t2, atol=1e-10, rtol=0)
    assert abs(cc.triples() - ref.tcorr_tjl()) < 1e-10
