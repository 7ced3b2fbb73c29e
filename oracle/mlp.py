"""numpy restatement of the learned-guess MLP (test infrastructure).

Mirrors ugacc_gb300/csrc/mlp.cu: 15 features -> 256 -> 256 -> 1 with SiLU, parameters in
the order W1[8][256] b1[256] W2[256][256] b2[256] w3[256] b3, mean-squared-error loss.
The GPU stores the three weight matrices in FP16 for its forward and backward products
(biases stay FP32), so the comparison rounds them the same way.
"""
import numpy as np

F, H = 15, 256
F_COUNT = F
SIZES = [("W1", (F, H)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("w3", (H,)), ("b3", (1,))]


def unpack(p):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape).astype(np.float64)
        o += n
    return out


def num_params():
    return sum(int(np.prod(s)) for _, s in SIZES)


def _fp16(x):
    return x.astype(np.float16).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, X, half_weights=True, half_activations=False):
    """half_activations: the first layer's activations rounded to FP16, as the fused
    tensor-core guess kernel feeds them to its second-layer MMA."""
    q = unpack(p)
    W1, W2, w3 = (q["W1"], q["W2"], q["w3"])
    if half_weights:
        W1, W2, w3 = _fp16(W1), _fp16(W2), _fp16(w3)
    Z1 = X @ W1 + q["b1"]
    A1 = silu(Z1)
    if half_activations:
        A1 = _fp16(A1)
    Z2 = A1 @ W2 + q["b2"]
    A2 = silu(Z2)
    y = A2 @ w3 + q["b3"][0]
    return y, (Z1, A1, Z2, A2, W1, W2, w3)


def loss_grad(p, X, t, half_weights=True):
    X = X.astype(np.float64)
    y, (Z1, A1, Z2, A2, W1, W2, w3) = forward(p, X, half_weights)
    n = X.shape[0]
    d = y - t
    loss = float(np.mean(d * d))
    dy = 2.0 * d / n
    g = {"w3": A2.T @ dy, "b3": np.array([dy.sum()])}
    dZ2 = np.outer(dy, w3) * dsilu(Z2)
    g["W2"] = A1.T @ dZ2
    g["b2"] = dZ2.sum(0)
    dZ1 = (dZ2 @ W2.T) * dsilu(Z1)
    g["W1"] = X.T @ dZ1
    g["b1"] = dZ1.sum(0)
    return loss, np.concatenate([g[name].ravel() for name, _ in SIZES])


SCALE = 100.0     # scale of the integral-valued features
TARGET = 1000.0   # targets and the network's output are TARGET * (t2 - t2_mp2)


def _denominators(no, nv, eps):
    eo, ev = eps[:no], eps[no:]
    return ((eo[:, None, None, None] + eo[None, :, None, None]) - ev[None, None, :, None]) - ev[None, None, None, :]


def features(no, nv, V):
    """Pair features of every T2 element (i, j, a, b), row-major, from the <pq|rs> blocks
    of `V` (a dict with "oovv", "oooo", "ovov", "vvvv" and "eps"): the MP2 amplitude and its
    exchange partner, the integral, -1/D, the mean occupied and virtual orbital energies,
    the i == j and a == b flags, the diagonal ladder and ring elements <ab|ab>, <ij|ij>,
    <ia|ia> + <jb|jb>, <ia|ai> + <jb|bj>, and the orbital-energy splittings |e_i - e_j|/2,
    |e_a - e_b|/2, (e_i - e_j)(e_a - e_b)/4 (all invariant under (i,j,a,b) -> (j,i,b,a))."""
    eps = V["eps"]
    D = _denominators(no, nv, eps)
    Voovv, Voooo, Vovov, Vvvvv = V["oovv"], V["oooo"], V["ovov"], V["vvvv"]
    eo, ev = eps[:no], eps[no:]
    i, j, a, b = np.meshgrid(np.arange(no), np.arange(no), np.arange(nv), np.arange(nv), indexing="ij")
    F = np.empty((no, no, nv, nv, F_COUNT))
    F[..., 0] = SCALE * Voovv / D
    F[..., 1] = SCALE * Voovv.transpose(0, 1, 3, 2) / D
    F[..., 2] = SCALE * Voovv
    F[..., 3] = -1.0 / D
    F[..., 4] = 0.5 * (eo[:, None, None, None] + eo[None, :, None, None])
    F[..., 5] = 0.5 * (ev[None, None, :, None] + ev[None, None, None, :])
    F[..., 6] = (i == j)
    F[..., 7] = (a == b)
    F[..., 8] = SCALE * Vvvvv[a, b, a, b]
    F[..., 9] = SCALE * Voooo[i, j, i, j]
    F[..., 10] = SCALE * (Vovov[i, a, i, a] + Vovov[j, b, j, b])
    F[..., 11] = SCALE * (Voovv[i, i, a, a] + Voovv[j, j, b, b])
    dij = eo[:, None, None, None] - eo[None, :, None, None]
    dab = ev[None, None, :, None] - ev[None, None, None, :]
    F[..., 12] = 0.5 * np.abs(dij)
    F[..., 13] = 0.5 * np.abs(dab)
    F[..., 14] = 0.25 * dij * dab
    return F.reshape(-1, F_COUNT)


def blocks(ints, no):
    """The <pq|rs> blocks features() reads, from a full [nact]^4 array."""
    o, v = slice(0, no), slice(no, None)
    return {"oovv": ints[o, o, v, v], "oooo": ints[o, o, o, o], "ovov": ints[o, v, o, v], "vvvv": ints[v, v, v, v]}


def targets(no, nv, Voovv, eps, t2):
    D = _denominators(no, nv, eps)
    return (TARGET * (t2.reshape(no, no, nv, nv) - Voovv.reshape(no, no, nv, nv) / D)).ravel()
