"""FP64 restatement of the control-variate network (test infrastructure).

Forward and hand-derived backward of x -> tanh(W1 x + b1) -> tanh(W2 h1 + b2) -> W3 h2 + b3
with loss mean (y - t)^2, in numpy FP64, on the same parameter layout as the GPU kernels:
W1 [128][4], b1 [128], W2 [128][128], b2 [128], W3 [128], b3. The GPU computes with the
BF16-rounded weights, so callers pass those here. Its 128 x 128 layer runs on the tensor
cores with BF16 operands, so the operands of those products (h1 in the forward and the
weight gradient, dz2 in both gradients) are rounded to BF16 here as well (round to nearest
even, from FP32); everything else stays FP64.
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


def bf16(v):
    """Round to BF16 (nearest even) through FP32, as the GPU forms its tensor-core operands."""
    u = np.ascontiguousarray(np.asarray(v, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(p, x):
    w = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    h1 = np.tanh(x @ w["W1"].T + w["b1"])
    h2 = np.tanh(bf16(h1) @ w["W2"].T + w["b2"])
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
    g["W2"] = bf16(dz2).T @ bf16(h1)
    g["b2"] = dz2.sum(axis=0)
    dz1 = (bf16(dz2) @ w["W2"]) * (1.0 - h1 ** 2)
    g["W1"] = dz1.T @ x
    g["b1"] = dz1.sum(axis=0)
    return np.concatenate([g[name].ravel() for name, _ in SIZES]), float(np.mean((y - t) ** 2))
