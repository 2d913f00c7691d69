"""Float64 numpy MLP -- TEST INFRASTRUCTURE ONLY.

The reference has no learned controller; this is the CPU oracle for the
project's own MLP (9 -> 64 -> 64 -> 1, SiLU, mean-squared error), used to
check the GPU training kernels' loss and gradients and the tensor-core
inference.  Flat parameter layout as in particles_gb300/csrc/pt_mlp_train.cu:
W1[9][64], b1[64], W2[64][64], b2[64], W3[64], b3.
"""
import numpy as np

NIN, NH = 9, 64
SIZES = [("W1", (NIN, NH)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NH,)),
         ("b3", (1,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    p = np.asarray(p, np.float64)
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, X):
    w = unpack(p)
    z1 = X @ w["W1"] + w["b1"]
    h1 = _silu(z1)
    z2 = h1 @ w["W2"] + w["b2"]
    h2 = _silu(z2)
    return h2 @ w["W3"] + w["b3"][0], (z1, h1, z2, h2)


def loss_grad(p, X, T):
    """Mean-squared error and its gradient (float64)."""
    X = np.asarray(X, np.float64)
    T = np.asarray(T, np.float64)
    w = unpack(p)
    y, (z1, h1, z2, h2) = forward(p, X)
    n = X.shape[0]
    r = y - T
    loss = float((r * r).mean())
    dy = 2.0 * r / n
    g = {"W3": h2.T @ dy, "b3": np.array([dy.sum()])}
    dz2 = np.outer(dy, w["W3"]) * _dsilu(z2)
    g["W2"] = h1.T @ dz2
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ w["W2"].T) * _dsilu(z1)
    g["W1"] = X.T @ dz1
    g["b1"] = dz1.sum(0)
    flat = np.concatenate([g[name].ravel() for name, _ in SIZES])
    return loss, flat


def init_params(seed):
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in SIZES:
        if name.startswith("W"):
            fan_in = shape[0]
            parts.append(rng.normal(0.0, 1.0 / np.sqrt(fan_in), shape).ravel())
        else:
            parts.append(np.zeros(int(np.prod(shape))))
    return np.concatenate(parts)
