"""Oracle of the learned-site network (TEST INFRASTRUCTURE: the parity reference
of the library's MLP kernels, never part of them): float64 numpy forward pass, mean
squared error and its gradient by the chain rule, for the parameter layout of
bn_mlp_* (W1[64][6] b1 W2[64][64] b2 W3[64][64] b3 W4[6][64] b4)."""
import numpy as np

IN, H, OUT = 6, 64, 6
SIZES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
         ("W4", (OUT, H)), ("b4", (OUT,))]


def unpack(p):
    out, o = {}, 0
    for name, shp in SIZES:
        n = int(np.prod(shp))
        out[name] = np.asarray(p[o:o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def num_params():
    return sum(int(np.prod(s)) for _, s in SIZES)


def forward(p, x):
    w = unpack(p)
    h1 = np.tanh(x @ w["W1"].T + w["b1"])
    h2 = np.tanh(h1 @ w["W2"].T + w["b2"])
    h3 = np.tanh(h2 @ w["W3"].T + w["b3"])
    return h3 @ w["W4"].T + w["b4"], (h1, h2, h3)


def loss_grad(p, x, t):
    """loss = sum (o - t)^2 / (n * OUT) and its gradient, flat in the layout above."""
    w = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    o, (h1, h2, h3) = forward(p, x)
    n = x.shape[0]
    r = o - t
    loss = float(np.sum(r * r) / (n * OUT))
    d4 = 2.0 * r / (n * OUT)
    d3 = (d4 @ w["W4"]) * (1 - h3 * h3)
    d2 = (d3 @ w["W3"]) * (1 - h2 * h2)
    d1 = (d2 @ w["W2"]) * (1 - h1 * h1)
    g = {"W1": d1.T @ x, "b1": d1.sum(0), "W2": d2.T @ h1, "b2": d2.sum(0), "W3": d3.T @ h2, "b3": d3.sum(0),
         "W4": d4.T @ h3, "b4": d4.sum(0)}
    return loss, np.concatenate([g[name].ravel() for name, _ in SIZES])
