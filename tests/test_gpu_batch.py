"""Batched CCSD: every member must end where the one-context solver ends.

Members of one smooth family with uneven sizes are solved together (one graph launch
for the whole solve, the sweep loop on the device); each member's energy, iteration
count and amplitudes are compared with a separate single-context solve of the same
Hamiltonian.
"""
import numpy as np
import pytest

import ugacc_gb300 as U
from ugacc_gb300.generator import make_family

pytestmark = pytest.mark.gpu


def _single(h, opts):
    H = U.Hamiltonian.from_synthetic(h)
    cc = U.CCWfn(H, opts)
    e = cc.compute_energy()
    return e, cc.iterations, cc.t2


@pytest.mark.parametrize("diis", [True, False])
def test_batch_matches_single_solves(diis):
    fam = make_family(9, seed=21, no_range=(4, 7), nv_range=(20, 40))
    opts = {"R_CONVERGENCE": 1e-9, "DIIS": diis, "MAXITER": 60}
    bt = U.Batch()
    for h in fam:
        bt.add(h)
    e, it, cv = bt.ccsd(opts)
    assert cv.all()
    for k, h in enumerate(fam):
        e1, it1, t2 = _single(h, opts)
        assert abs(e[k] - e1) < 1e-10, (k, e[k], e1)
        assert abs(int(it[k]) - it1) <= 1, (k, it[k], it1)
        np.testing.assert_allclose(bt.t2(k), t2, atol=1e-7, rtol=0)
    info = bt.info()
    assert info["members"] == len(fam) and info["sweeps"] == it.max()
    assert info["grouped_ops"] > 10 and sum(info["shape_choice"]) > 0 and info["graph_kernels"] > info["grouped_ops"]
    # a second solve starts again from MP2 and repeats the first exactly
    e2, it2, _ = bt.ccsd(opts)
    np.testing.assert_array_equal(it2, it)
    np.testing.assert_allclose(e2, e, rtol=0, atol=1e-13)


def test_batch_iteration_limit():
    fam = make_family(3, seed=5, no_range=(4, 5), nv_range=(20, 24))
    bt = U.Batch()
    for h in fam:
        bt.add(h)
    e, it, cv = bt.ccsd({"R_CONVERGENCE": 1e-12, "MAXITER": 3})
    assert not cv.any() and (it == 3).all()


def test_batch_rejects_mixed_precision():
    fam = make_family(1, seed=5, no_range=(4, 4), nv_range=(20, 20))
    bt = U.Batch()
    bt.add(fam[0])
    with pytest.raises(U.UccError):
        bt.ccsd({"PRECISION": "MIXED"})


def test_batch_solve_is_one_graph_launch():
    fam = make_family(5, seed=8, no_range=(4, 6), nv_range=(20, 32))
    bt = U.Batch()
    for h in fam:
        bt.add(h)
    e, it, cv = bt.ccsd({"R_CONVERGENCE": 1e-9})
    info = bt.info()
    # all sweeps ran inside one host launch of the solve graph
    assert cv.all() and info["graph_launches"] == 1 and info["sweeps"] == it.max() > 3


def test_batch_device_time_limit_reports_timeout_and_batch_stays_usable():
    """The sweep loop runs on the device; its globaltimer limit ends it early with
    UCC_DEVICE_TIMEOUT, and the next solve with a normal limit converges as usual."""
    fam = make_family(6, seed=9, no_range=(4, 6), nv_range=(20, 32))
    opts = {"R_CONVERGENCE": 1e-10, "MAXITER": 60}
    ref = U.Batch()
    for h in fam:
        ref.add(h)
    e_ref, it_ref, _ = ref.ccsd(opts)
    ref.close()
    bt = U.Batch()
    for h in fam:
        bt.add(h)
    bt.set_time_limit(1e-6)  # runs out after the first sweep
    with pytest.raises(U.UccError) as err:
        bt.ccsd(opts)
    assert err.value.status == 7, err.value
    assert "time limit" in str(err.value)
    assert bt.info()["sweeps"] < it_ref.max()
    bt.set_time_limit(600.0)
    e, it, cv = bt.ccsd(opts)
    assert cv.all()
    np.testing.assert_array_equal(it, it_ref)
    np.testing.assert_allclose(e, e_ref, rtol=0, atol=1e-13)
    with pytest.raises(U.UccError):
        bt.set_time_limit(0.0)
