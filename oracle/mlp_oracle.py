"""FP64 restatement of the control-variate network (test infrastructure).

Forward and hand-derived backward of x -> tanh(W1 x + b1) -> tanh(W2 h1 + b2) -> W3 h2 + b3
with loss mean (y - t)^2, in numpy FP64, on the same parameter layout as the GPU kernels:
W1 [128][4], b1 [128], W2 [128][128], b2 [128], W3 [128], b3. The GPU computes with the
BF16-rounded weights, so callers pass those here.
"""
import numpy as np

H = 128
SIZES = [("W1", (H, 4)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H,)), ("b3", (1,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = p[o:o + n].reshape(shape)
        o += n
    return out


def forward(p, x):
    w = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    h1 = np.tanh(x @ w["W1"].T + w["b1"])
    h2 = np.tanh(h1 @ w["W2"].T + w["b2"])
    return h2 @ w["W3"] + w["b3"][0], (x, h1, h2)


def gradient(p, x, t):
    """(grad [NPARAMS], loss) of mean (y - t)^2."""
    w = unpack(p)
    y, (x, h1, h2) = forward(p, x)
    t = np.asarray(t, dtype=np.float64)
    n = len(t)
    dy = 2.0 * (y - t) / n
    g = {"W3": h2.T @ dy, "b3": np.array([dy.sum()])}
    dz2 = np.outer(dy, w["W3"]) * (1.0 - h2 ** 2)
    g["W2"] = dz2.T @ h1
    g["b2"] = dz2.sum(axis=0)
    dz1 = (dz2 @ w["W2"]) * (1.0 - h1 ** 2)
    g["W1"] = dz1.T @ x
    g["b1"] = dz1.sum(axis=0)
    return np.concatenate([g[name].ravel() for name, _ in SIZES]), float(np.mean((y - t) ** 2))
