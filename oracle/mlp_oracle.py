"""FP64 NumPy oracle of the learned-correction MLP (forward and backward).

TEST INFRASTRUCTURE ONLY (the checker of the tcgen05 kernels in
barnes-hut_gb300/csrc/bh_mlp.cu; the product never calls it).  The network has
no reference counterpart.  To compare with the GPU kernels it reproduces their
rounding points: weights and the layer inputs of every GEMM are rounded to
BF16 (round to nearest even), everything else is FP64.  GELU is the tanh form
(Hendrycks & Gimpel) used by the kernels.

Parameter layout (float, length 10448): W1[16][64] (rows >= 6 zero), b1[64],
W2[64][64], b2[64], W3[64][64], b3[64], W4[64][16] (columns >= 2 zero), b4[16];
W_l[in][out].
"""
import numpy as np

OFF = dict(W1=(0, (16, 64)), b1=(1024, (64,)), W2=(1088, (64, 64)), b2=(5184, (64,)),
           W3=(5248, (64, 64)), b3=(9344, (64,)), W4=(9408, (64, 16)), b4=(10432, (16,)))
P_TOTAL = 10448
C0, C1 = 0.7978845608028654, 0.044715


def bf16(a):
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return {k: p[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in OFF.items()}


def pack(d):
    p = np.zeros(P_TOTAL)
    for k, (o, s) in OFF.items():
        p[o:o + int(np.prod(s))] = np.asarray(d[k]).reshape(-1)
    return p


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(C0 * (x + C1 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(C0 * (x + C1 * x ** 3))
    return 0.5 * (1 + t) + 0.5 * x * (1 - t * t) * C0 * (1 + 3 * C1 * x * x)


def forward(p, feats, emulate_bf16=True):
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    w = unpack(p)
    x = np.zeros((len(feats), 16))
    x[:, :6] = feats[:, :6]
    cache = {"a0": r(x)}
    h1 = cache["a0"] @ r(w["W1"])
    a1 = r(gelu(h1 + w["b1"]))
    h2 = a1 @ r(w["W2"])
    a2 = r(gelu(h2 + w["b2"]))
    h3 = a2 @ r(w["W3"])
    a3 = r(gelu(h3 + w["b3"]))
    y = a3 @ r(w["W4"]) + w["b4"]
    cache.update(h1=h1, a1=a1, h2=h2, a2=a2, h3=h3, a3=a3)
    return y[:, :2], cache


def loss_and_grad(p, feats, targets, emulate_bf16=True):
    """loss = mean((y - t)^2) over rows and the 2 outputs; gradient w.r.t. p."""
    r = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    w = unpack(p)
    y, c = forward(p, feats, emulate_bf16)
    P = len(feats)
    e = y - targets
    loss = float(np.mean(e ** 2))
    dy = np.zeros((P, 16))
    dy[:, :2] = 2.0 * e / (P * 2)
    g = {}
    g["W4"] = c["a3"].T @ r(dy)
    g["b4"] = dy.sum(0)
    da3 = r(dy) @ r(w["W4"]).T
    dh3 = da3 * gelu_grad(c["h3"] + w["b3"])
    g["W3"] = c["a2"].T @ r(dh3)
    g["b3"] = dh3.sum(0)
    da2 = r(dh3) @ r(w["W3"]).T
    dh2 = da2 * gelu_grad(c["h2"] + w["b2"])
    g["W2"] = c["a1"].T @ r(dh2)
    g["b2"] = dh2.sum(0)
    da1 = r(dh2) @ r(w["W2"]).T
    dh1 = da1 * gelu_grad(c["h1"] + w["b1"])
    g["W1"] = c["a0"].T @ r(dh1)
    g["b1"] = dh1.sum(0)
    g["W1"][6:] = 0
    g["W4"][:, 2:] = 0
    g["b4"][2:] = 0
    return loss, pack(g)
