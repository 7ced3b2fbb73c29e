"""Tensor-core (tcgen05, BF16 hi+lo split, FP32 accumulate) path against FP64."""
import numpy as np
import pytest

import ugacc_gb300 as U
from ugacc_gb300.generator import make_hamiltonian

pytestmark = pytest.mark.gpu

# Two-term split products keep ~16 significant bits per operand: relative error of a
# GEMM element is bounded by ~2^-16 of the sum of |products|.
SPLIT_RTOL = 4e-5


@pytest.mark.parametrize("M,N,K,ta,tb", [(128, 256, 64, 0, 0), (300, 520, 777, 0, 1), (257, 129, 1000, 1, 0),
                                          (1000, 300, 96, 1, 1)])
def test_tc_gemm_against_fp64(M, N, K, ta, tb):
    rng = np.random.default_rng(M + N + K)
    A = rng.standard_normal((K, M) if ta else (M, K))
    B = rng.standard_normal((N, K) if tb else (K, N))
    C0 = rng.standard_normal((M, N))
    ctx = U.Context()
    ref = 0.7 * (A.T if ta else A) @ (B.T if tb else B) - 0.3 * C0
    got = ctx.gemm(A, B, C0, alpha=0.7, beta=-0.3, transa=ta, transb=tb, precision=U.MIXED)
    scale = 0.7 * np.abs(A.T if ta else A) @ np.abs(B.T if tb else B)
    assert np.all(np.abs(got - ref) <= SPLIT_RTOL * scale + 1e-12)
    f64 = ctx.gemm(A, B, C0, alpha=0.7, beta=-0.3, transa=ta, transb=tb, precision=U.FP64)
    np.testing.assert_allclose(f64, ref, rtol=1e-12, atol=1e-10)


def test_mixed_refined_ccsd_matches_fp64():
    h = make_hamiltonian(12, 64, 9)
    H = U.Hamiltonian.from_synthetic(h)
    cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10})
    e64 = cc.compute_energy()
    t2 = cc.t2
    H.ctx.reset_stats()
    mx = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "PRECISION": "MIXED", "REFINE_SWEEPS": 2})
    emx = mx.compute_energy()
    st = H.ctx.stats()
    assert st["tc_gemm_launches"] > 0 and st["fp64_iterations"] >= 2
    assert abs(emx - e64) < 1e-9
    np.testing.assert_allclose(mx.t2, t2, atol=1e-9, rtol=0)


def test_mixed_unrefined_within_one_microhartree():
    h = make_hamiltonian(12, 64, 9)
    H = U.Hamiltonian.from_synthetic(h)
    e64 = U.CCWfn(H, {"R_CONVERGENCE": 1e-8}).compute_energy()
    mx = U.CCWfn(H, {"R_CONVERGENCE": 1e-5, "PRECISION": "MIXED", "REFINE_SWEEPS": 0})
    emx = mx.compute_energy()
    assert H.ctx.stats()["fp64_iterations"] == 0
    assert abs(emx - e64) < 1e-6


@pytest.mark.parametrize("no,nv,seed", [(6, 80, 13), (5, 84, 7), (6, 78, 13)])
def test_mixed_triples_matches_fp64(no, nv, seed):
    """nv = 80 and 84 run the pipelined energy kernel (84: the last 8-wide virtual tile is half
    outside nv, zero-filled), nv = 78 the padded-tile kernel it falls back to when nv % 4 != 0."""
    h = make_hamiltonian(no, nv, seed)
    H = U.Hamiltonian.from_synthetic(h)
    cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10})
    cc.compute_energy()
    e64 = cc.triples()
    mx = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "PRECISION": "MIXED"})
    mx.compute_energy()
    H.ctx.reset_stats()
    emx = mx.triples()
    assert H.ctx.stats()["tc_gemm_launches"] == 3  # one batched launch per pair of W3 terms
    # split products carry ~2^-16 relative error into W3; E(T) is a weighted sum of W3*V3;
    # never looser than 1 uEh absolute (tests/test_gpu_large.py checks that bound where
    # |E(T)| is several mEh)
    assert abs(emx - e64) < min(1e-6, 1e-8 + 1e-4 * abs(e64))


def _lambda_response(h, precision, hand):
    from ugacc_gb300.generator import make_perturbations
    H = U.Hamiltonian.from_synthetic(h)
    cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "PRECISION": precision})
    cc.compute_energy()
    hb = U.HBAR(H, cc)
    lam = U.CCLambda(cc, hb)
    lam.compute_lambda()
    pseudo = lam.pseudoenergy()
    mu = U.CCPert(make_perturbations(h.nact, h.seed)[0], 0.0656, cc, hb, lam)
    mu.solve("right")
    if hand == "left":
        mu.solve("left")
    a = U.CCResp(mu, mu).linresp(mu, mu)
    return pseudo, a, H.ctx.stats()


@pytest.mark.parametrize("hand", ["right", "left"])
def test_mixed_lambda_and_response_match_fp64(hand):
    h = make_hamiltonian(10, 64, 12)
    p64, a64, _ = _lambda_response(h, "FP64", hand)
    pmx, amx, st = _lambda_response(h, "MIXED", hand)
    assert st["tc_gemm_launches"] > 0
    assert abs(pmx - p64) < 1e-9
    assert abs(amx - a64) < 1e-8 * max(1.0, abs(a64))


def _tgrad_pipeline(h, precision):
    H = U.Hamiltonian.from_synthetic(h)
    cc = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "PRECISION": precision, "WFN": "CCSD_T", "DERTYPE": "FIRST"})
    e = cc.compute_energy()
    no, nv = h.no, h.nv
    s1, s2 = H.ctx.get("s1", (no, nv)), H.ctx.get("s2", (no, no, nv, nv))
    hb = U.HBAR(H, cc)
    lam = U.CCLambda(cc, hb)
    lam.compute_lambda()
    dens = U.CCDensity(cc, lam)
    return e, s1, s2, dens.onepdm() + dens.twopdm(), H.ctx.stats()


def test_mixed_triples_gradient_matches_fp64():
    h = make_hamiltonian(6, 64, 21)
    e64, s1_64, s2_64, ed64, _ = _tgrad_pipeline(h, "FP64")
    emx, s1_mx, s2_mx, edmx, st = _tgrad_pipeline(h, "MIXED")
    assert st["tc_gemm_launches"] > 0
    assert abs(ed64 - e64) < 1e-9 and abs(edmx - emx) < 2e-8  # E(density) = E_CCSD(T)
    np.testing.assert_allclose(s1_mx, s1_64, atol=1e-4 * np.abs(s1_64).max(), rtol=0)
    np.testing.assert_allclose(s2_mx, s2_64, atol=1e-4 * np.abs(s2_64).max(), rtol=0)
    assert abs(edmx - ed64) < 1e-7


def test_fine_split_gemm_matches_fp64():
    """UCC_MIXED_FINE: three-part split, K in chunks summed in FP64 (in-kernel chunks)."""
    rng = np.random.default_rng(8)
    ctx = U.Context()
    for (M, N, K) in [(200, 300, 500), (256, 512, 4096)]:
        A, B = rng.standard_normal((M, K)), rng.standard_normal((K, N))
        C0 = rng.standard_normal((M, N))
        ref = 0.5 * A @ B + 0.25 * C0
        got = ctx.gemm(A, B, C0, alpha=0.5, beta=0.25, precision=U.MIXED_FINE)
        scale = 0.5 * np.abs(A) @ np.abs(B)
        assert np.all(np.abs(got - ref) <= SPLIT_RTOL * scale + 1e-12)


@pytest.mark.parametrize("M,N,K,ta,tb", [(128, 256, 64, 0, 0), (300, 520, 777, 0, 1), (257, 129, 1000, 1, 0),
                                          (40, 3000, 5000, 0, 1), (1000, 300, 96, 1, 1), (640, 768, 20000, 0, 0),
                                          (2200000, 40, 64, 0, 0), (2560, 2560, 16, 0, 0), (160, 40960, 16, 1, 0),
                                          (3000, 700, 24, 0, 1), (999, 1001, 40, 1, 1)])
def test_sliced_fp64_gemm(M, N, K, ta, tb):
    """UCC_FP64_SLICED: 9 exact bf16 slices per operand on the tensor cores, FP64-accurate
    (error of the order of FP64 rounding, relative to the row / column maxima).  The
    2200000-row shape exceeds one slicing launch and runs in row chunks; K = 16 ... 40 are
    zero-padded to the 64-wide K block."""
    rng = np.random.default_rng(M * 7 + N + K)
    A = rng.standard_normal((K, M) if ta else (M, K)) * np.exp(2.0 * rng.standard_normal((K, M) if ta else (M, K)))
    B = rng.standard_normal((N, K) if tb else (K, N))
    A[..., 3] = 0.0  # zero rows / columns and tiny entries
    B[..., 5] *= 1e-30
    C0 = rng.standard_normal((M, N))
    ctx = U.Context()
    Am, Bm = (A.T if ta else A), (B.T if tb else B)
    ref = 0.7 * Am @ Bm - 0.3 * C0
    got = ctx.gemm(A, B, C0, alpha=0.7, beta=-0.3, transa=ta, transb=tb, precision=U.FP64_SLICED)
    scale = 0.7 * np.abs(Am).max(axis=1)[:, None] * np.abs(Bm).max(axis=0)[None, :]
    err = np.abs(got - ref)
    assert np.all(err <= 1e-14 * np.sqrt(K) * scale + 1e-15 * np.abs(ref) + 1e-300), (err / scale).max()
    st = ctx.stats()
    assert st["sliced_gemm_launches"] == (2 if M > 2000000 else 1)


def test_mixed_record_sweeps_use_the_sliced_gemm():
    """The FP64 work of a MIXED solve (record sweeps, HBAR) runs on the sliced tensor-core
    GEMM and keeps the FP64 answer."""
    h = make_hamiltonian(12, 96, 9)
    H = U.Hamiltonian.from_synthetic(h)
    e64 = U.CCWfn(H, {"R_CONVERGENCE": 1e-10}).compute_energy()
    H.ctx.reset_stats()
    emx = U.CCWfn(H, {"R_CONVERGENCE": 1e-10, "PRECISION": "MIXED"}).compute_energy()
    st = H.ctx.stats()
    assert st["sliced_gemm_launches"] > 0 and st["fp64_iterations"] >= 2
    assert abs(emx - e64) < 1e-9


def test_sliced_gemm_reports_operands_out_of_range():
    """A row maximum beyond 2^498 sets the sliced form's range flag in the slicing kernel
    (which only reads and writes inside its buffers); the call then fails with UCC_BAD_ARGS
    instead of returning a wrong product, and the context stays usable."""
    ctx = U.Context()
    rng = np.random.default_rng(3)
    A = rng.standard_normal((128, 64))
    B = rng.standard_normal((64, 256))
    A[5, 3] = 1e160
    with pytest.raises(U.UccError) as e:
        ctx.gemm(A, B, precision=U.FP64_SLICED)
    assert e.value.status == 4
    A[5, 3] = 1.0
    got = ctx.gemm(A, B, precision=U.FP64_SLICED)
    np.testing.assert_allclose(got, A @ B, rtol=0, atol=1e-12)


def test_sliced_gemm_digits_set_the_error():
    """ucc_gemm_sliced with d digits per operand: the error per output element stays within
    the truncation bound ~(d + 5) 2^(2 - 6d) sqrt(K) max|A row| max|B col| (with a factor 4
    of margin), and each digit taken away raises it by far more than the 8x checked here
    (nominally 64x), so the digits asked for are the digits used."""
    M, N, K = 300, 520, 777
    rng = np.random.default_rng(17)
    A = rng.standard_normal((M, K)) * np.exp(rng.standard_normal((M, K)))
    B = rng.standard_normal((K, N))
    ref = A @ B
    scale = np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=0)[None, :]
    ctx = U.Context()
    worst = {}
    for d in range(4, 10):
        got = ctx.gemm(A, B, digits=d)
        rel = np.abs(got - ref) / scale
        bound = 16.0 * (d + 5) * 2.0 ** (-6 * d) * np.sqrt(K)
        assert rel.max() <= bound + 1e-15, (d, rel.max(), bound)
        worst[d] = rel.max()
    for d in range(4, 8):
        assert worst[d] >= 8.0 * worst[d + 1], worst
    np.testing.assert_array_equal(ctx.gemm(A, B, digits=9), ctx.gemm(A, B, precision=U.FP64_SLICED))
    with pytest.raises(U.UccError) as e:
        ctx.gemm(A, B, digits=10)
    assert e.value.status == 4
    ctx.close()
