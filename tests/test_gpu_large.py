"""GPU checks at the sizes of the larger workloads (minutes, not seconds).

* (T) in the mixed form against the FP64 form on the same converged amplitudes at
  no=24/nv=240 (the Lambda/response workload's Hamiltonian, seed 3), where |E(T)| is
  several mEh: the difference must stay below 1 uEh absolute; and the whole mixed
  CCSD(T) against the FP64 one to 1 uEh.
* The response pipeline (Lambda, densities, alpha at omega 0 and 0.0656) of the same
  generator at no=16/nv=160, seed 3: mixed against FP64.
* The batched solver on the 512-member family (no 4..12, nv 20..96): every member
  converged, and a sample of members against separate single-context solves.
"""
import numpy as np
import pytest

import ugacc_gb300 as U
from ugacc_gb300.generator import RESPONSE_OMEGAS, make_family, make_hamiltonian, make_perturbations

pytestmark = pytest.mark.gpu


def test_mixed_triples_within_one_microhartree_at_no24_nv240():
    h = make_hamiltonian(24, 240, 3)
    H = U.Hamiltonian.from_synthetic(h, precision="MIXED")
    c64 = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "PRECISION": "FP64"})
    e_ccsd64 = c64.compute_energy()
    e_t64 = c64.triples()
    # (T) in the mixed form on the same FP64 amplitudes
    e_tmx = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "PRECISION": "MIXED"}).triples()
    print("E(T) fp64 %.12e mixed %.12e diff %.2e" % (e_t64, e_tmx, abs(e_tmx - e_t64)))
    assert abs(e_t64) > 3e-3
    assert abs(e_tmx - e_t64) < 1e-6  # 1 uEh, absolute
    # the whole mixed CCSD(T) against FP64
    cmx = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "PRECISION": "MIXED", "WFN": "CCSD_T"})
    e_mx = cmx.compute_energy()
    assert abs(cmx.eccsd - e_ccsd64) < 1e-8
    assert abs(e_mx - (e_ccsd64 + e_t64)) < 1e-6


def _response(H, h, precision):
    cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "PRECISION": precision})
    cc.compute_energy()
    hb = U.HBAR(H, cc)
    lam = U.CCLambda(cc, hb)
    lam.compute_lambda()
    dens = U.CCDensity(cc, lam)
    out = {"eccsd": cc.eccsd, "pseudo": lam.pseudoenergy(), "e1": dens.onepdm(), "e2": dens.twopdm(), "alpha": {}}
    perts = make_perturbations(h.nact, h.seed)
    for w in RESPONSE_OMEGAS:
        mu = [U.CCPert(perts[x], w, cc, hb, lam) for x in range(3)]
        for m in mu:
            m.solve("right")
        a = np.zeros((3, 3))
        for p in range(3):
            for q in range(p + 1):
                r = U.CCResp(mu[p], mu[q])
                a[p, q] = a[q, p] = (r.linresp(mu[p], mu[q]) if p == q else
                                     0.5 * r.linresp(mu[p], mu[q]) + 0.5 * r.linresp(mu[q], mu[p]))
        out["alpha"][w] = a
    return out


def test_response_pipeline_mixed_vs_fp64_no16_nv160():
    h = make_hamiltonian(16, 160, 3)
    r64 = _response(U.Hamiltonian.from_synthetic(h), h, "FP64")
    rmx = _response(U.Hamiltonian.from_synthetic(h, precision="MIXED"), h, "MIXED")
    assert abs(rmx["eccsd"] - r64["eccsd"]) < 1e-9
    assert abs(rmx["pseudo"] - r64["pseudo"]) < 1e-9
    assert abs(rmx["e1"] - r64["e1"]) < 1e-9 and abs(rmx["e2"] - r64["e2"]) < 1e-9
    for w in RESPONSE_OMEGAS:
        a64, amx = r64["alpha"][w], rmx["alpha"][w]
        print("omega", w, "alpha_xx", a64[0, 0], amx[0, 0])
        np.testing.assert_allclose(amx, a64, rtol=1e-8, atol=1e-8 * np.abs(a64).max())


def test_batched_family_512_members_vs_single_solves():
    fam = make_family(512, 7, no_range=(4, 12), nv_range=(20, 96))
    opts = {"R_CONVERGENCE": 1e-8, "MAXITER": 100}
    bt = U.Batch()
    for h in fam:
        bt.add(h)
    e, it, cv = bt.ccsd(opts)
    info = bt.info()
    bt.close()
    assert cv.all(), int(cv.sum())
    assert info["graph_launches"] == 1
    print("512 members: %d sweeps, %.2f s" % (info["sweeps"], info["solve_ms"] / 1e3))
    for k in [0, 57, 130, 255, 301, 388, 444, 511]:
        h = fam[k]
        cc = U.CCWfn(U.Hamiltonian.from_synthetic(h), opts)
        e1 = cc.compute_energy()
        assert abs(e1 - e[k]) < 1e-9, (k, e1, e[k])
        assert abs(cc.iterations - it[k]) <= 1, (k, cc.iterations, it[k])
