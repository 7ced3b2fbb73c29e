"""Failure detection on the GPU without a GPU fault.

Every wait inside the tensor-core pipelines is bounded: when one runs out the kernel
raises a device flag and returns, and the C ABI call reports UCC_DEVICE_TIMEOUT.
ucc_wait_selftest runs that path on purpose (one thread waits on a barrier that nothing
completes), so the tests below check the status, that the wait ends near its limit, and
that the context and its stream keep working afterwards.
"""
import time

import numpy as np
import pytest

import ugacc_gb300 as U

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_survives():
    ctx = U.Context()
    rng = np.random.default_rng(3)
    A, B = rng.standard_normal((320, 512)), rng.standard_normal((512, 384))
    ref = A @ B
    C0 = ctx.gemm(A, B, precision=U.MIXED)  # the pipeline works before
    t0 = time.time()
    with pytest.raises(U.UccError) as e:
        ctx.wait_selftest(0.05)
    waited = time.time() - t0
    assert e.value.status == 7, e.value
    assert "timed out" in str(e.value)
    assert waited < 5.0, waited
    # the flag is cleared and the stream is usable: the same product again, bit-identical
    C1 = ctx.gemm(A, B, precision=U.MIXED)
    assert np.array_equal(C0, C1)
    assert np.abs(C1 - ref).max() < 1e-4 * np.abs(ref).max()
    # a second self-test reports again (the flag was reset, not left stuck)
    with pytest.raises(U.UccError) as e2:
        ctx.wait_selftest(1e-3)
    assert e2.value.status == 7
    ctx.close()


def test_wait_selftest_rejects_limits_out_of_range():
    ctx = U.Context()
    with pytest.raises(U.UccError) as e:
        ctx.wait_selftest(0.0)
    assert e.value.status == 4
    ctx.close()
