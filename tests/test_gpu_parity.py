"""GPU path (through the C ABI) against the reference's golden outputs and the oracle."""
import numpy as np
import pytest

import ugacc_gb300 as U
from golden_util import cases, hamiltonian, load
from oracle import cc as O
from ugacc_gb300.generator import make_hamiltonian, make_perturbations

pytestmark = pytest.mark.gpu

ETOL = 1e-10   # Eh, FP64 path vs the reference's own code (|dE| <= 1e-8 required)
TTOL = 1e-10   # amplitudes / intermediates


def gpu_pipeline(h, use_ints=True, **opts):
    H = U.Hamiltonian.from_synthetic(h, use_ints=use_ints)
    cc = U.CCWfn(H, dict({"R_CONVERGENCE": 1e-10, "MAXITER": 100}, **opts))
    cc.compute_energy()
    return H, cc


@pytest.mark.parametrize("name", [c for c in cases() if c != "c2"])
def test_ccsd_triples_vs_reference(name):
    meta, arr = load(name)
    h, _ = hamiltonian(meta)
    H, cc = gpu_pipeline(h)
    tag, run = next(iter(meta["runs"].items()))
    if run["options"].get("WFN") == "CCSD_T":  # the reference returned E_CCSD + E_(T)
        assert abs(cc.eccsd + cc.triples() - run["e_ccsd"]) < ETOL
    else:
        assert abs(cc.eccsd - run["e_ccsd"]) < ETOL
    assert cc.iterations == len(run["tables"]["ccsd"])  # same DIIS, same iteration count
    if f"{tag}/t1" in arr:
        np.testing.assert_allclose(cc.t1, arr[f"{tag}/t1"], atol=TTOL, rtol=0)
    if f"{tag}/t2" in arr:
        np.testing.assert_allclose(cc.t2, arr[f"{tag}/t2"], atol=TTOL, rtol=0)
    if "e_t_tjl" in run:
        assert abs(cc.triples() - run["e_t_tjl"]) < ETOL


def test_df_and_ints_inputs_agree():
    meta, _ = load("c1")
    h, _ = hamiltonian(meta)
    _, a = gpu_pipeline(h, use_ints=True)
    _, b = gpu_pipeline(h, use_ints=False)
    assert abs(a.eccsd - b.eccsd) < 1e-12
    np.testing.assert_allclose(a.t2, b.t2, atol=1e-13, rtol=0)


@pytest.mark.parametrize("name", ["c1", "tiny", "one_occ"])
def test_hbar_lambda_density_vs_reference(name):
    meta, arr = load(name)
    h, _ = hamiltonian(meta)
    H, cc = gpu_pipeline(h)
    tag, run = next((t, r) for t, r in meta["runs"].items() if r["options"]["DERTYPE"] != "NONE")
    hb = U.HBAR(H, cc)
    for k in U.HBAR.SHAPES:
        if f"{tag}/{k}" in arr:
            np.testing.assert_allclose(hb.block(k), arr[f"{tag}/{k}"], atol=TTOL, rtol=0, err_msg=k)
    lam = U.CCLambda(cc, hb)
    lam.compute_lambda()
    assert abs(lam.pseudoenergy() - run["pseudoenergy"]) < ETOL
    for k in ["l1", "l2"]:
        if f"{tag}/{k}" in arr:
            np.testing.assert_allclose(getattr(lam, k), arr[f"{tag}/{k}"], atol=TTOL, rtol=0)
    dens = U.CCDensity(cc, lam)
    e1, e2 = dens.onepdm(), dens.twopdm()
    assert abs(e1 - run["e_onepdm"]) < ETOL and abs(e2 - run["e_twopdm"]) < ETOL
    assert abs(e1 + e2 - run["e_ccsd"]) < 1e-9  # ugacc.cc:133-139 consistency check
    for k in ["Doo", "Dvv", "Dov", "Dvo"]:
        if f"{tag}/{k}" in arr:
            np.testing.assert_allclose(dens.block(k), arr[f"{tag}/{k}"], atol=TTOL, rtol=0)
    _check_twopdm(dens, run, arr, tag)


def _check_twopdm(dens, run, arr, tag):
    """The six two-particle density blocks element by element and each block's energy as
    the reference prints it (ccdensity.cc:153-339, 14 decimals)."""
    for k in ["Goooo", "Gvvvv", "Gooov", "Gvvvo", "Govov", "Goovv"]:
        if f"{tag}/{k}" in arr:
            np.testing.assert_allclose(dens.block(k), arr[f"{tag}/{k}"], atol=TTOL, rtol=0, err_msg=k)
    parts = dens.twopdm_parts()
    for blk, e in run.get("e_twopdm_parts", {}).items():
        assert abs(parts[blk] - e) < 1e-12, (blk, parts[blk], e)


@pytest.mark.parametrize("name", ["c1", "tiny"])
def test_response_vs_reference(name):
    meta, arr = load(name)
    h, perts = hamiltonian(meta)
    H, cc = gpu_pipeline(h)
    hb = U.HBAR(H, cc)
    lam = U.CCLambda(cc, hb)
    lam.compute_lambda()
    for tag, run in meta["runs"].items():
        if run["options"]["DERTYPE"] != "SECOND":
            continue
        omega = float(run["options"]["MY_OMEGA"])
        hand = run["options"]["MYHAND"].lower()
        alpha, rot, P = U.response(cc, hb, lam, perts, omega, hand)
        for k, v in alpha.items():
            assert abs(v - run["alpha_" + k]) < 1e-9, (tag, k)
        for k, v in rot.items():
            assert abs(v - run["rot_" + k]) < 1e-9, (tag, k)
        for key, ref in arr.items():
            t, nm = key.split("/")
            if t != tag or nm[0] not in "XY":
                continue
            amp, pert = nm.split("_")
            np.testing.assert_allclose(P[pert].amp(amp), ref, atol=TTOL, rtol=0, err_msg=key)


def test_larger_case_vs_oracle():
    """Sizes past every 64-wide GEMM tile edge, against the numpy oracle."""
    h = make_hamiltonian(7, 70, 21)
    H, cc = gpu_pipeline(h, use_ints=False)
    ref = O.CCWfn(O.Hamiltonian(h), maxiter=100, r_convergence=1e-10)
    ref.compute_energy()
    assert abs(cc.eccsd - ref.eccsd) < ETOL
    np.testing.assert_allclose(cc.t2, ref.t2, atol=TTOL, rtol=0)
    assert abs(cc.triples() - ref.tcorr_tjl()) < ETOL


def test_not_converged_status():
    meta, _ = load("tiny")
    h, _ = hamiltonian(meta)
    H = U.Hamiltonian.from_synthetic(h)
    cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "MAXITER": 1})
    with pytest.raises(U.ConvergenceError):
        cc.compute_energy()


def test_stage_order_is_enforced():
    meta, _ = load("tiny")
    h, _ = hamiltonian(meta)
    H = U.Hamiltonian.from_synthetic(h)
    with pytest.raises(U.UccError) as e:
        H.ctx.check(H.ctx.lib.ucc_hbar(H.ctx.h))
    assert e.value.status == 5


@pytest.mark.parametrize("tag,ooc", [("ccsd_t_first", True), ("ccsd_t_first_incore", False)])
def test_triples_gradient_vs_reference(tag, ooc):
    """WFN=CCSD_T, DERTYPE=FIRST: s1, s2 and the (T) density pieces of tgrad_ooc
    (ccwfn.cc:1150-1316, OOC=1) or tgrad (:854-1142, OOC=0: full Doo/Dvv), then Lambda
    with s1/s2 and the densities starting from the (T) pieces."""
    meta, arr = load("tgrad")
    h, _ = hamiltonian(meta)
    run = meta["runs"][tag]
    H, cc = gpu_pipeline(h, WFN="CCSD_T", DERTYPE="FIRST", OOC=ooc)
    assert abs(cc.eccsd + cc.et - run["e_ccsd"]) < ETOL
    no, nv = h.no, h.nv
    shapes = {"s1": (no, nv), "s2": (no, no, nv, nv), "DooT": (no, no), "DvvT": (nv, nv), "DovT": (no, nv),
              "GoovvT": (no, no, nv, nv), "GooovT": (no, no, no, nv), "GvvvoT": (nv, nv, nv, no)}
    for name, shp in shapes.items():
        ref = arr[f"{tag}/{name}"]
        got = H.ctx.get(name, shp)
        np.testing.assert_allclose(got, ref, atol=1e-20 + 1e-10 * np.abs(ref).max(), rtol=0, err_msg=name)
    hb = U.HBAR(H, cc)
    lam = U.CCLambda(cc, hb)
    lam.compute_lambda()
    assert abs(lam.pseudoenergy() - run["pseudoenergy"]) < ETOL
    np.testing.assert_allclose(lam.l1, arr[f"{tag}/l1"], atol=TTOL, rtol=0)
    np.testing.assert_allclose(lam.l2, arr[f"{tag}/l2"], atol=TTOL, rtol=0)
    dens = U.CCDensity(cc, lam)
    e1, e2 = dens.onepdm(), dens.twopdm()
    assert abs(e1 - run["e_onepdm"]) < ETOL and abs(e2 - run["e_twopdm"]) < ETOL
    assert abs(e1 + e2 - (cc.eccsd + cc.et)) < 1e-10  # E(density) = E_CCSD(T)
    for k in ["Doo", "Dvv", "Dov"]:
        np.testing.assert_allclose(H.ctx.get(k, arr[f"{tag}/{k}"].shape), arr[f"{tag}/{k}"], atol=TTOL, rtol=0)
    _check_twopdm(dens, run, arr, tag)


def test_triples_gradient_vs_oracle_larger():
    """The same pieces at no=5, nv=24 (several tuple batches) against the oracle."""
    h = make_hamiltonian(5, 24, 31)
    H, cc = gpu_pipeline(h, WFN="CCSD_T", DERTYPE="FIRST")  # OOC false: full Doo/Dvv
    Ho = O.Hamiltonian(h)
    co = O.CCWfn(Ho, r_convergence=1e-10)
    co.compute_energy()
    tg = co.tgrad(ooc=False)
    no, nv = h.no, h.nv
    pairs = {"s1": ("s1", (no, nv)), "s2": ("s2", (no, no, nv, nv)), "Doo": ("DooT", (no, no)),
             "Dvv": ("DvvT", (nv, nv)), "Dov": ("DovT", (no, nv)), "Goovv": ("GoovvT", (no, no, nv, nv)),
             "Gooov": ("GooovT", (no, no, no, nv)), "Gvvvo": ("GvvvoT", (nv, nv, nv, no))}
    for k, (name, shp) in pairs.items():
        ref = tg[k]
        np.testing.assert_allclose(H.ctx.get(name, shp), ref, atol=1e-20 + 1e-9 * np.abs(ref).max(), rtol=0,
                                   err_msg=k)


@pytest.mark.skipif("c2" not in cases(), reason="the no=16/nv=160 reference run is not recorded")
def test_c2_workload_vs_reference():
    """The bench workload itself (no=16, nv=160, seed 1): E_CCSD and E_(T) of the
    reference's own compiled code (hours on one core) against the FP64 and the mixed form."""
    meta, arr = load("c2")
    h, _ = hamiltonian(meta)
    run = meta["runs"]["ccsd_t"]
    H = U.Hamiltonian.from_synthetic(h)
    cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "MAXITER": 100, "WFN": "CCSD_T"})
    cc.compute_energy()
    assert abs(cc.eccsd - run["e_ccsd"]) < ETOL
    assert abs(cc.et - run["e_t_tjl"]) < ETOL
    np.testing.assert_allclose(cc.t1, arr["ccsd_t/t1"], atol=TTOL, rtol=0)
    mx = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "MAXITER": 100, "WFN": "CCSD_T", "PRECISION": "MIXED"})
    mx.compute_energy()
    assert abs(mx.eccsd - run["e_ccsd"]) < 1e-10
    assert abs(mx.et - run["e_t_tjl"]) < 1e-8
