"""numpy restatement of the warm-start network -- TEST INFRASTRUCTURE ONLY.

No reference counterpart (the network is new).  Forward, mean-squared-error loss and
backward of 96 -> 128 -> 128 -> 16 (3 outputs used) with SiLU, in float64.  With
``bf16=True`` the values the GPU kernels round to bfloat16 are rounded the same way (inputs,
weights, hidden activations and the deltas that feed the tensor-core GEMMs), so the GPU's
float32-accumulated results can be compared tightly.  Parameter layout: one float32 array,
W1 [96][128] | W2 [128][128] | W3 [128][16] | b1 [128] | b2 [128] | b3 [16].
"""

import numpy as np

IN, H, OUT, NOUT = 96, 128, 16, 3
SIZES = [("W1", (IN, H)), ("W2", (H, H)), ("W3", (H, OUT)), ("b1", (H,)), ("b2", (H,)), ("b3", (OUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SIZES)


def unpack(P):
    out, o = {}, 0
    for name, shp in SIZES:
        n = int(np.prod(shp))
        out[name] = np.asarray(P[o : o + n], dtype=np.float64).reshape(shp)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).reshape(-1) for name, _ in SIZES])


def bf16(x):
    """Round to bfloat16 (round to nearest even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(P, X, bf=True):
    p = unpack(P)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    x = r(X)
    z1 = x @ r(p["W1"])
    h1 = r(silu(z1 + p["b1"]))
    z2 = h1 @ r(p["W2"])
    h2 = r(silu(z2 + p["b2"]))
    y = h2 @ r(p["W3"]) + p["b3"]
    return dict(x=x, z1=z1, h1=h1, z2=z2, h2=h2, y=y)


def loss_and_grad(P, X, T, bf=True):
    """Mean over samples of sum over the 3 outputs of (y - t)^2, and its gradient."""
    p = unpack(P)
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    f = forward(P, X, bf)
    n = len(X)
    e = np.zeros_like(f["y"])
    e[:, :NOUT] = f["y"][:, :NOUT] - np.asarray(T, dtype=np.float64)[:, :NOUT]
    loss = float(np.sum(e * e) / n)
    dy = 2.0 * e / n
    dyr = r(dy)
    dh2 = dyr @ r(p["W3"]).T
    dz2 = dh2 * silu_grad(f["z2"] + p["b2"])
    dz2r = r(dz2)
    dh1 = dz2r @ r(p["W2"]).T
    dz1 = dh1 * silu_grad(f["z1"] + p["b1"])
    g = dict(
        W1=f["x"].T @ r(dz1),
        W2=f["h1"].T @ dz2r,
        W3=f["h2"].T @ dyr,
        b1=dz1.sum(0),
        b2=dz2.sum(0),
        b3=dy.sum(0),
    )
    return loss, pack(g)


def adam(P, G, M, V, lr, t):
    M = 0.9 * M + 0.1 * G
    V = 0.999 * V + 0.001 * G * G
    mh = M / (1 - 0.9**t)
    vh = V / (1 - 0.999**t)
    return P - lr * mh / (np.sqrt(vh) + 1e-8), M, V
