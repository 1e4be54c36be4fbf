"""CPU restatement of the learned-correction network (test infrastructure
only: the tests use it as the checker of the library's tensor-core forward
and backward kernels; nothing in the product imports it).

The network has no counterpart in the reference (Teton accelerates source
iteration only with grey transport, rt/GTASolver.F90).  What is restated
here is the library's own definition (umt_gb300/csrc/learn.cu):

    h1 = bf16(relu(bf16(X) bf16(W1)^T + b1))
    h2 = bf16(relu(h1 bf16(W2)^T + b2))
    h3 = bf16(relu(h2 bf16(W3)^T + b3))
    o  = h3 bf16(W4)^T + b4

with products accumulated exactly here (float64) and in FP32 on the GPU.
The backward pass rounds at the same points the kernels do: dO = bf16(dY),
dZ3 = bf16((dO bf16(W4)) * [h3 > 0]), dZ2, dZ1 likewise; dW_l = dZ_l^T X_l,
db_l = sum of dZ_l.  `exact=True` skips the BF16 rounding of the backward
quantities (the float64 gradient of the forward as computed).

Parameter vector (FP32 master copy, row-major out x in):
    W1[128][F], b1[128], W2[128][128], b2[128], W3[128][128], b3[128],
    W4[G][128], b4[G],  F = 4G + 4.
"""
from __future__ import annotations

import numpy as np

H = 128


def bf16(x):
    """Round to bfloat16 (nearest, ties to even), returned as float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def features(G):
    return 4 * G + 4


def unpack(p, G):
    F = features(G)
    p = np.asarray(p, dtype=np.float64)
    shapes = [("W1", (H, F)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
              ("W4", (G, H)), ("b4", (G,))]
    out, o = {}, 0
    for name, shp in shapes:
        n = int(np.prod(shp))
        out[name] = p[o:o + n].reshape(shp)
        o += n
    assert o == p.size, (o, p.size)
    return out


def pack(d):
    return np.concatenate([d[k].ravel() for k in ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4")])


def forward(p, X, G):
    w = unpack(p, G)
    x = bf16(X)
    h1 = bf16(np.maximum(x @ bf16(w["W1"]).T + w["b1"], 0.0))
    h2 = bf16(np.maximum(h1 @ bf16(w["W2"]).T + w["b2"], 0.0))
    h3 = bf16(np.maximum(h2 @ bf16(w["W3"]).T + w["b3"], 0.0))
    o = h3 @ bf16(w["W4"]).T + w["b4"]
    return o, (x, h1, h2, h3)


def gradient(p, X, dY, G, exact=False):
    """Gradient of sum(dY * o) with respect to the parameter vector."""
    w = unpack(p, G)
    q = (lambda a: a) if exact else bf16
    o, (x, h1, h2, h3) = forward(p, X, G)
    dO = q(dY)
    dZ3 = q((dO @ bf16(w["W4"])) * (h3 > 0))
    dZ2 = q((dZ3 @ bf16(w["W3"])) * (h2 > 0))
    dZ1 = q((dZ2 @ bf16(w["W2"])) * (h1 > 0))
    g = {"W1": dZ1.T @ x, "b1": dZ1.sum(0), "W2": dZ2.T @ h1, "b2": dZ2.sum(0),
         "W3": dZ3.T @ h2, "b3": dZ3.sum(0), "W4": dO.T @ h3, "b4": dO.sum(0)}
    return pack(g)


def multiplier(o, lo=-12.0, hi=8.0):
    """The correction multiplier m = exp(clamp(o))."""
    return np.exp(np.clip(o, lo, hi))
