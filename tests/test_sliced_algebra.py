"""The sliced FP64 GEMM's arithmetic, restated in numpy (CPU).

tc_gemm.cu (slice_digits_kernel, sliced_gemm_kernel) writes each operand row as
2^e_r sum_s d_s 2^-6(s+1) with |d_s| <= 32 (e_r = ilogb(row max) + 2) and sums the slice
products order by order; products of one order are integers times 2^-6(s+t+2) of at most
2^10, so up to 2^14 of them add exactly in FP32.  The error-free splitting is the one of
Ozaki, Ogita, Oishi and Rump (Numer. Algorithms 59, 2012).
"""
import numpy as np


SB = 6  # bits per digit


def _slices(X, S):
    """Digits as slice_digits_kernel forms them: x 2^(SB S - e) rounded to an integer, then
    balanced base-2^SB digits from the least significant one up."""
    amax = np.abs(X).max(axis=1)
    e = np.where(amax > 0, np.frexp(np.where(amax > 0, amax, 1.0))[1] + 1, -500)  # ilogb + 2
    v = X * np.ldexp(1.0, -e)[:, None]
    assert np.all(np.abs(v) < 0.5)
    Xi = np.rint(np.ldexp(v, SB * S)).astype(np.int64)  # exact: |v 2^(SB S)| < 2^53
    H = 1 << (SB - 1)
    out = [None] * S
    for s in range(S - 1, 0, -1):
        d = ((Xi + H) & (2 * H - 1)) - H
        Xi = (Xi - d) >> SB
        out[s] = d.astype(np.float64)
    out[0] = Xi.astype(np.float64)
    return np.array(out), e


def test_digits_are_small_integers_and_reconstruct():
    rng = np.random.default_rng(0)
    X = rng.standard_normal((50, 300)) * np.exp(3.0 * rng.standard_normal((50, 300)))
    d, e = _slices(X, 9)
    assert np.all(np.abs(d) <= 32) and np.all(d == np.rint(d))
    # bf16 holds 8 significant bits: every digit times a power of two is exact
    rec = sum(d[s] * 2.0 ** (-SB * (s + 1)) for s in range(9)) * np.ldexp(1.0, e)[:, None]
    rowmax = np.abs(X).max(axis=1)[:, None]
    assert np.all(np.abs(rec - X) <= 2.0 ** -53 * rowmax)


def test_order_sums_are_exact_in_fp32():
    rng = np.random.default_rng(1)
    A = rng.standard_normal((8, 16384))
    B = rng.standard_normal((8, 16384))
    da, _ = _slices(A, 3)
    db, _ = _slices(B, 3)
    for s, t in [(0, 0), (1, 0), (2, 0)]:
        exact = da[s] @ db[t].T  # integers of magnitude <= 2^14 * 32 * 32 = 2^24
        assert np.all(np.abs(exact) <= 2.0 ** 24)
        assert np.array_equal(exact.astype(np.float32).astype(np.float64), exact)


def test_truncated_order_sum_is_fp64_accurate():
    rng = np.random.default_rng(2)
    A = rng.standard_normal((64, 2000)) * np.exp(2.0 * rng.standard_normal((64, 2000)))
    B = rng.standard_normal((48, 2000))
    S = 9
    da, ea = _slices(A, S)
    db, eb = _slices(B, S)
    acc = np.zeros((64, 48))
    for g in range(S):  # orders s + t = g < S; higher orders are dropped
        for s in range(g + 1):
            acc += (da[s] @ db[g - s].T) * 2.0 ** (-SB * (g + 2))
    got = acc * np.ldexp(1.0, ea)[:, None] * np.ldexp(1.0, eb)[None, :]
    ref = A @ B.T
    scale = np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=1)[None, :]
    assert np.all(np.abs(got - ref) <= 1e-14 * np.sqrt(2000) * scale)


def _digits_64(X, S):
    """slice_digits_kernel's balanced base-2^SB digits of one integer, least significant
    first extracted (tc_gemm.cu, 64-bit form)."""
    H, out = 1 << (SB - 1), [0] * S
    for s in range(S - 1, -1, -1):
        if s > 0:
            d = ((X + H) & (2 * H - 1)) - H
            X = (X - d) >> SB
        else:
            d = X
        out[s] = d
    return out


def _digits_32(X, S):
    """The same in 32-bit parts (the kernel's form for S >= 6): the low 30 bits give the 5
    least significant digits and a carry of 0 or 1 into the high part."""
    H, out = 1 << (SB - 1), [0] * S
    lo, hi = X & ((1 << 30) - 1), X >> 30
    s = S - 1
    for _ in range(5):
        d = ((lo + H) & (2 * H - 1)) - H
        lo = (lo - d) >> SB
        out[s] = d
        s -= 1
    assert lo in (0, 1)
    hi += lo
    for s in range(s, 0, -1):
        d = ((hi + H) & (2 * H - 1)) - H
        hi = (hi - d) >> SB
        out[s] = d
    out[0] = hi
    for v in [lo, hi] + out:
        assert -(2 ** 31) <= v < 2 ** 31  # every intermediate fits an int
    return out


def test_32bit_digit_extraction_equals_the_64bit_form():
    rng = np.random.default_rng(5)
    for S in (6, 7, 8, 9):
        lim = 1 << (SB * S - 1)
        xs = [0, 1, -1, lim - 1, -(lim - 1), 2 ** 30, -(2 ** 30), 2 ** 30 - 1, -(2 ** 29) - 1]
        xs += [int(v) for v in rng.integers(-lim + 1, lim, size=20000)]
        for X in xs:
            assert _digits_32(X, S) == _digits_64(X, S), (S, X)
