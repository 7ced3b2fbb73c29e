"""Pins the numpy oracle against the reference's own outputs (tests/golden/)."""
import numpy as np
import pytest

from golden_util import cases, hamiltonian, load
from oracle import cc as O

ETOL = 1e-12   # Eh; the restatement agrees with the reference to ~1e-17
TTOL = 1e-11


def _pipeline(meta):
    h, perts = hamiltonian(meta)
    H = O.Hamiltonian(h)
    cc = O.CCWfn(H, maxiter=100, r_convergence=1e-10)
    cc.compute_energy()
    return h, perts, H, cc


@pytest.mark.parametrize("name", [c for c in cases() if c != "c2"])
def test_ccsd_and_triples(name):
    meta, arr = load(name)
    h, perts, H, cc = _pipeline(meta)
    for tag, run in meta["runs"].items():
        if run["options"].get("WFN") == "CCSD_T":  # compute_energy returned E_CCSD + E_(T)
            assert abs(cc.eccsd + cc.tcorr_tjl() - run["e_ccsd"]) < ETOL
        else:
            assert abs(cc.eccsd - run["e_ccsd"]) < ETOL
        # iteration-by-iteration energies of the reference's table (same DIIS procedure)
        ref_iters = [e for _, e in run["tables"]["ccsd"][1:]]
        assert len(ref_iters) == len(cc.iter_energies)
        np.testing.assert_allclose(cc.iter_energies, ref_iters, atol=5e-15, rtol=0)
        if f"{tag}/t1" in arr:
            np.testing.assert_allclose(cc.t1, arr[f"{tag}/t1"], atol=TTOL, rtol=0)
        if f"{tag}/t2" in arr:
            np.testing.assert_allclose(cc.t2, arr[f"{tag}/t2"], atol=TTOL, rtol=0)
        if "e_t_tjl" in run:
            et = cc.tcorr_tjl()
            assert abs(et - run["e_t_tjl"]) < ETOL
            # the reference's three (T) algorithms agree with one another
            assert abs(run["e_t_ooc"] - run["e_t_tjl"]) < ETOL
            assert abs(run["e_t_incore"] - run["e_t_tjl"]) < ETOL


@pytest.mark.parametrize("name", ["c1", "tiny", "one_occ"])
def test_hbar_lambda_density(name):
    meta, arr = load(name)
    h, perts, H, cc = _pipeline(meta)
    tag, run = next((t, r) for t, r in meta["runs"].items() if r["options"]["DERTYPE"] != "NONE")
    hb = O.HBAR(H, cc)
    for k in ["Hov", "Hoo", "Hvv", "Hoooo", "Hvvvv", "Hvovv", "Hooov", "Hovvo", "Hovov", "Hvvvo", "Hovoo"]:
        if f"{tag}/{k}" in arr:
            np.testing.assert_allclose(getattr(hb, k), arr[f"{tag}/{k}"], atol=TTOL, rtol=0, err_msg=k)
    lam = O.CCLambda(cc, hb)
    lam.compute_lambda()
    assert abs(lam.pseudoenergy() - run["pseudoenergy"]) < ETOL
    for k in ["l1", "l2"]:
        if f"{tag}/{k}" in arr:
            np.testing.assert_allclose(getattr(lam, k), arr[f"{tag}/{k}"], atol=TTOL, rtol=0)
    dens = O.CCDensity(cc, lam)
    e1, e2 = dens.onepdm(), dens.twopdm()
    assert abs(e1 - run["e_onepdm"]) < ETOL and abs(e2 - run["e_twopdm"]) < ETOL
    # the reference's own consistency check, ugacc.cc:133-139
    assert abs(e1 + e2 - run["e_ccsd"]) < 1e-9
    for k in ["Doo", "Dvv", "Dov", "Dvo"]:
        if f"{tag}/{k}" in arr:
            np.testing.assert_allclose(getattr(dens, k), arr[f"{tag}/{k}"], atol=TTOL, rtol=0)
    # the two-particle density block by block, and each block's energy as the reference
    # prints it (ccdensity.cc:153-339, 14 decimals)
    for k in ["Goooo", "Gvvvv", "Gooov", "Gvvvo", "Govov", "Goovv"]:
        if f"{tag}/{k}" in arr:
            np.testing.assert_allclose(dens.G[k], arr[f"{tag}/{k}"], atol=TTOL, rtol=0, err_msg=k)
    for blk, e in run.get("e_twopdm_parts", {}).items():
        assert abs(dens.E2[blk.lower()] - e) < 1e-13, (blk, dens.E2[blk.lower()], e)


@pytest.mark.parametrize("name", ["c1", "tiny"])
def test_response(name):
    meta, arr = load(name)
    h, perts, H, cc = _pipeline(meta)
    hb = O.HBAR(H, cc)
    lam = O.CCLambda(cc, hb)
    lam.compute_lambda()
    for tag, run in meta["runs"].items():
        if run["options"]["DERTYPE"] != "SECOND":
            continue
        omega = float(run["options"]["MY_OMEGA"])
        hand = run["options"]["MYHAND"].lower()
        alpha, rot, P = O.response(cc, hb, lam, perts, omega, hand)
        for k, v in alpha.items():
            assert abs(v - run["alpha_" + k]) < 1e-11, (tag, k)
        for k, v in rot.items():
            assert abs(v - run["rot_" + k]) < 1e-11, (tag, k)
        for key, ref in arr.items():
            t, nm = key.split("/")
            if t != tag or "_" not in nm or nm[0] not in "XY":
                continue
            amp, pert = nm.split("_")
            np.testing.assert_allclose(getattr(P[pert], amp), ref, atol=TTOL, rtol=0, err_msg=key)


def test_diis_matches_reference_procedure():
    """Same extrapolation as the shim's DIISManager (attic/diis.cc procedure)."""
    rng = np.random.default_rng(3)
    d = O.DIIS(8)
    for k in range(11):
        d.add(rng.standard_normal(20), rng.standard_normal(20))
    assert d.size() == 8
    out = d.extrapolate()
    E = np.array(d.err)
    B = E @ E.T
    B /= np.abs(B).max()
    M = np.block([[B, -np.ones((8, 1))], [-np.ones((1, 8)), np.zeros((1, 1))]])
    c = np.linalg.solve(M, np.r_[np.zeros(8), -1.0])
    assert abs(c[:8].sum() - 1.0) < 1e-12
    np.testing.assert_allclose(out, c[:8] @ np.array(d.vec), atol=1e-12)


def test_not_converged_raises():
    meta, _ = load("tiny")
    h, _ = hamiltonian(meta)
    cc = O.CCWfn(O.Hamiltonian(h), maxiter=1, r_convergence=1e-10)
    with pytest.raises(O.NotConverged):
        cc.compute_energy()


@pytest.mark.parametrize("tag,ooc", [("ccsd_t_first", True), ("ccsd_t_first_incore", False)])
def test_triples_gradient_pieces_lambda_and_densities(tag, ooc):
    """WFN=CCSD_T, DERTYPE=FIRST: the s1, s2 and (T) density pieces of tgrad_ooc
    (ccwfn.cc:1150-1316, OOC=1) and of the in-core tgrad (:854-1142, OOC=0, full Doo/Dvv),
    the Lambda equations with s1/s2 (cclambda.cc:181,243) and the densities that start
    from the (T) pieces (ccdensity.cc:44-69)."""
    meta, arr = load("tgrad")
    h, perts, H, cc = _pipeline(meta)
    run = meta["runs"][tag]
    tg = cc.tgrad(ooc=ooc)
    for k in ["s1", "s2", "Doo", "Dvv", "Dov", "Goovv", "Gooov", "Gvvvo"]:
        ref = arr[f"{tag}/{k}" if k in ("s1", "s2") else f"{tag}/{k}T"]
        np.testing.assert_allclose(tg[k], ref, atol=1e-16 + 1e-12 * np.abs(ref).max(), rtol=0, err_msg=k)
    hb = O.HBAR(H, cc)
    lam = O.CCLambda(cc, hb)
    lam.compute_lambda()
    assert abs(lam.pseudoenergy() - run["pseudoenergy"]) < ETOL
    np.testing.assert_allclose(lam.l1, arr[f"{tag}/l1"], atol=TTOL, rtol=0)
    np.testing.assert_allclose(lam.l2, arr[f"{tag}/l2"], atol=TTOL, rtol=0)
    dens = O.CCDensity(cc, lam)
    e1, e2 = dens.onepdm(), dens.twopdm()
    assert abs(e1 - run["e_onepdm"]) < ETOL and abs(e2 - run["e_twopdm"]) < ETOL
    # with the (T) pieces the density energy is the CCSD(T) energy
    assert abs(e1 + e2 - run["e_ccsd"]) < 1e-12
    # the blocks include the (T) pieces the reference starts them from
    for k in ["Goooo", "Gvvvv", "Gooov", "Gvvvo", "Govov", "Goovv"]:
        if f"{tag}/{k}" in arr:
            np.testing.assert_allclose(dens.G[k], arr[f"{tag}/{k}"], atol=TTOL, rtol=0, err_msg=k)
    for blk, e in run.get("e_twopdm_parts", {}).items():
        assert abs(dens.E2[blk.lower()] - e) < 1e-13, (blk, dens.E2[blk.lower()], e)
    for k in ["Doo", "Dvv", "Dov"]:
        np.testing.assert_allclose(getattr(dens, k), arr[f"{tag}/{k}"], atol=TTOL, rtol=0)
