"""The packed pair ladder's algebra, in numpy (CPU).

The particle ladders run on packed pairs (kernels_fp64.cu pack_vvvv / pack_tau /
unpack_ladder): with amplitudes Z invariant under (i,j,e,f) -> (j,i,f,e) and an operator
W_abef invariant under (a,b,e,f) -> (b,a,f,e),

    sum_ef W_abef Z_ijef = S[ij][ab] + sign A[ij][ab],
    S = Zp Wp^T over (i<=j, a<=b, e<=f),  A = Zm Wm^T over (i<j, a<b, e<f),

sign = -1 when exactly one of (i > j), (a > b) holds.  The HBAR ladders of the
Lambda (cclambda.cc) and response (ccpert.cc) residuals use Hvvvv, which is not
pair-symmetric; they enter symmetrised residuals Q + Q(ji,ba), whose ladder part is the
packed ladder of W = Hvvvv_efab + Hvvvv_feba (mode 1) or Hvvvv_abef + Hvvvv_bafe (mode 2).
"""
import numpy as np


def _pairs_le(n):
    return [(p, q) for q in range(n) for p in range(q + 1)]


def _pairs_lt(n):
    return [(p, q) for q in range(n) for p in range(q)]


def _op(H, mode):
    if mode == 1:
        return np.einsum("efab->abef", H) + np.einsum("feba->abef", H)
    if mode == 2:
        return H + np.einsum("bafe->abef", H)
    return H


def _packed_ladder(Z, H, mode):
    no, nv = Z.shape[0], Z.shape[2]
    W = _op(H, mode)
    vp, vm, op_, om = _pairs_le(nv), _pairs_lt(nv), _pairs_le(no), _pairs_lt(no)
    Wp = np.array([[W[a, b, e, e] if e == f else W[a, b, e, f] + W[a, b, f, e] for e, f in vp] for a, b in vp])
    Wm = np.array([[W[a, b, e, f] - W[a, b, f, e] for e, f in vm] for a, b in vm])
    Zp = np.array([[Z[i, j, e, e] if e == f else 0.5 * (Z[i, j, e, f] + Z[i, j, f, e]) for e, f in vp] for i, j in op_])
    Zm = np.array([[0.5 * (Z[i, j, e, f] - Z[i, j, f, e]) for e, f in vm] for i, j in om])
    S, A = Zp @ Wp.T, Zm @ Wm.T
    out = np.zeros_like(Z)
    ip = {p: k for k, p in enumerate(op_)}
    im = {p: k for k, p in enumerate(om)}
    ap = {p: k for k, p in enumerate(vp)}
    am = {p: k for k, p in enumerate(vm)}
    for i in range(no):
        for j in range(no):
            for a in range(nv):
                for b in range(nv):
                    ij, ab = (min(i, j), max(i, j)), (min(a, b), max(a, b))
                    v = S[ip[ij], ap[ab]]
                    if i != j and a != b:
                        sign = -1.0 if (i > j) != (a > b) else 1.0
                        v += sign * A[im[ij], am[ab]]
                    out[i, j, a, b] = v
    return out


def _sym_amps(rng, no, nv):
    X = rng.standard_normal((no, no, nv, nv))
    return X + X.transpose(1, 0, 3, 2)


def test_ground_ladder_mode0():
    rng = np.random.default_rng(1)
    no, nv = 3, 5
    H = rng.standard_normal((nv,) * 4)
    H = H + H.transpose(1, 0, 3, 2)  # <ab|ef> = <ba|fe>
    Z = _sym_amps(rng, no, nv)
    ref = np.einsum("ijef,abef->ijab", Z, H)
    assert np.allclose(_packed_ladder(Z, H, 0), ref, atol=1e-12)


def test_lambda_and_y2_ladder_mode1():
    rng = np.random.default_rng(2)
    no, nv = 3, 5
    H = rng.standard_normal((nv,) * 4)  # no pair symmetry, like Hvvvv with its t1 term
    Z = _sym_amps(rng, no, nv)
    Q = 0.5 * np.einsum("ijef,efab->ijab", Z, H)
    ref = Q + Q.transpose(1, 0, 3, 2)
    assert np.allclose(0.5 * _packed_ladder(Z, H, 1), ref, atol=1e-12)


def test_x2_ladder_mode2():
    rng = np.random.default_rng(3)
    no, nv = 3, 5
    H = rng.standard_normal((nv,) * 4)
    Z = _sym_amps(rng, no, nv)
    Q = 0.5 * np.einsum("ijef,abef->ijab", Z, H)
    ref = Q + Q.transpose(1, 0, 3, 2)
    assert np.allclose(0.5 * _packed_ladder(Z, H, 2), ref, atol=1e-12)
