"""numpy restatement of the learned-guess MLP (test infrastructure).

Mirrors ugacc_gb300/csrc/mlp.cu: 8 features -> 256 -> 256 -> 1 with SiLU, parameters in
the order W1[8][256] b1[256] W2[256][256] b2[256] w3[256] b3, mean-squared-error loss.
The GPU stores the three weight matrices in FP16 for its forward and backward products
(biases stay FP32), so the comparison rounds them the same way.
"""
import numpy as np

F, H = 8, 256
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


def forward(p, X, half_weights=True):
    q = unpack(p)
    W1, W2, w3 = (q["W1"], q["W2"], q["w3"])
    if half_weights:
        W1, W2, w3 = _fp16(W1), _fp16(W2), _fp16(w3)
    Z1 = X @ W1 + q["b1"]
    A1 = silu(Z1)
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


SCALE = 100.0  # targets and the correction carried by the network are S * (t2 - t2_mp2)


def _denominators(no, nv, eps):
    eo, ev = eps[:no], eps[no:]
    return ((eo[:, None, None, None] + eo[None, :, None, None]) - ev[None, None, :, None]) - ev[None, None, None, :]


def features(no, nv, Voovv, eps):
    """Pair features of every T2 element (i, j, a, b), row-major: the MP2 amplitude and
    its exchange partner, the integral, -1/D, the mean occupied and virtual orbital
    energies and the i == j, a == b flags (the first three scaled by S)."""
    D = _denominators(no, nv, eps)
    V = Voovv.reshape(no, no, nv, nv)
    Vx = V.transpose(0, 1, 3, 2)
    eo, ev = eps[:no], eps[no:]
    F = np.empty((no, no, nv, nv, 8))
    F[..., 0] = SCALE * V / D
    F[..., 1] = SCALE * Vx / D
    F[..., 2] = SCALE * V
    F[..., 3] = -1.0 / D
    F[..., 4] = 0.5 * (eo[:, None, None, None] + eo[None, :, None, None])
    F[..., 5] = 0.5 * (ev[None, None, :, None] + ev[None, None, None, :])
    F[..., 6] = np.eye(no)[:, :, None, None]
    F[..., 7] = np.eye(nv)[None, None, :, :]
    return F.reshape(-1, 8)


def targets(no, nv, Voovv, eps, t2):
    D = _denominators(no, nv, eps)
    return (SCALE * (t2.reshape(no, no, nv, nv) - Voovv.reshape(no, no, nv, nv) / D)).ravel()
