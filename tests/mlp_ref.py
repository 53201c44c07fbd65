"""Float64 numpy restatement of the estimator network (80 -> 64 -> 64 -> 2,
ReLU hidden layers, MSE loss averaged over batch and outputs) used to check
the GPU forward/backward kernels. Parameter layout as in include/qeg.h:
W1[64][80] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]."""
import numpy as np

IN, HID, OUT = 80, 64, 2
SIZES = [("W1", (HID, IN)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)), ("W3", (OUT, HID)), ("b3", (OUT,))]
NPARAMS = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(p):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([d[name].reshape(-1) for name, _ in SIZES])


def to_bf16(x):
    """Rounds float32 values to bfloat16 precision (round to nearest even)."""
    b = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def forward(p, x):
    w = unpack(p)
    z1 = x @ w["W1"].T + w["b1"]
    h1 = np.maximum(z1, 0)
    z2 = h1 @ w["W2"].T + w["b2"]
    h2 = np.maximum(z2, 0)
    y = h2 @ w["W3"].T + w["b3"]
    return y, (z1, h1, z2, h2)


def loss_and_grad(p, x, t):
    x = np.asarray(x, np.float64)
    t = np.asarray(t, np.float64)
    w = unpack(p)
    y, (z1, h1, z2, h2) = forward(p, x)
    n = x.shape[0] * OUT
    loss = float(((y - t) ** 2).sum() / n)
    dy = 2 * (y - t) / n
    g = {"W3": dy.T @ h2, "b3": dy.sum(0)}
    dz2 = (dy @ w["W3"]) * (z2 > 0)
    g["W2"] = dz2.T @ h1
    g["b2"] = dz2.sum(0)
    dz1 = (dz2 @ w["W2"]) * (z1 > 0)
    g["W1"] = dz1.T @ x
    g["b1"] = dz1.sum(0)
    return loss, pack(g)
