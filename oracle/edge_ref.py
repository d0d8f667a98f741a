"""CPU oracle of the learned absorbing edge's networks (test infrastructure).

A numpy restatement of what include/fdp_edge.h specifies and
2d-vqsp-fd-sim_gb300/csrc/fdp_edge.cu computes: per set, a 96 -> 64 -> 64
-> 8 network with tanh hidden layers; inputs, weights and hidden activations
rounded to bfloat16 (round to nearest even), products accumulated exactly
here (float64) where the GPU accumulates in FP32 in its own order, so
comparisons carry a tolerance; loss = mean over samples and outputs of
(y - target)^2 and its gradient, back-propagated as the kernels do on the
tensor cores: each layer's error rounded to bfloat16 before it multiplies
the weights (the previous layer's error) or the layer's inputs (the weight
gradient), bias gradients summed from the unrounded errors; Adam with beta1
0.9, beta2 0.999, eps 1e-8.

`exact=True` drops every rounding, which makes the forward pass a smooth
function whose gradient the tests check against central differences --
that pins the backward formulas this oracle and the kernels share.  The
learned edge has no counterpart in the reference, so nothing here follows a
reference file.  Only tests may use this module.
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT, SETS = 96, 64, 8, 12
# parameter layout of one set: W1[64][96], b1, W2[64][64], b2, W3[8][64], b3
OFF = {}
_o = 0
for _name, _size in (("W1", HID * IN), ("b1", HID), ("W2", HID * HID), ("b2", HID), ("W3", OUT * HID), ("b3", OUT)):
    OFF[_name] = (_o, _size)
    _o += _size
SET_PARAMS = _o
assert SET_PARAMS == 10888


def bf16(x) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + (((u >> 16) & 1) + 0x7FFF)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(params: np.ndarray, s: int) -> dict:
    p = params[s * SET_PARAMS:(s + 1) * SET_PARAMS]
    shapes = {"W1": (HID, IN), "b1": (HID,), "W2": (HID, HID), "b2": (HID,), "W3": (OUT, HID), "b3": (OUT,)}
    return {k: p[o:o + n].reshape(shapes[k]) for k, (o, n) in OFF.items()}


def _forward_set(w: dict, x: np.ndarray, exact: bool):
    r = (lambda v: np.asarray(v, np.float64)) if exact else (lambda v: bf16(v).astype(np.float64))
    X = r(x)
    W1, W2, W3 = r(w["W1"]), r(w["W2"]), r(w["W3"])
    b1, b2, b3 = (np.asarray(w[k], np.float64) for k in ("b1", "b2", "b3"))
    H1 = r(np.tanh(b1 + X @ W1.T))
    H2 = r(np.tanh(b2 + H1 @ W2.T))
    Y = b3 + H2 @ W3.T
    return X, H1, H2, Y, (W1, W2, W3)


def forward(params: np.ndarray, sets: np.ndarray, x: np.ndarray, exact: bool = False) -> np.ndarray:
    y = np.zeros((len(sets), OUT))
    for s in np.unique(sets):
        idx = np.nonzero(sets == s)[0]
        y[idx] = _forward_set(unpack(params, int(s)), x[idx], exact)[3]
    return y


def gradients(params: np.ndarray, sets: np.ndarray, x: np.ndarray, target: np.ndarray, exact: bool = False):
    """(gradient with the parameters' layout, loss)."""
    n = len(sets)
    grad = np.zeros(SETS * SET_PARAMS)
    loss = 0.0
    for s in np.unique(sets):
        idx = np.nonzero(sets == s)[0]
        w = unpack(params, int(s))
        X, H1, H2, Y, (W1, W2, W3) = _forward_set(w, x[idx], exact)
        r = Y - np.asarray(target[idx], np.float64)
        loss += float(np.sum(r * r))
        dY = 2.0 * r / (n * OUT)
        # the tensor-core operands: errors rounded to bf16 (none with exact)
        q = (lambda v: np.asarray(v, np.float64)) if exact else (lambda v: bf16(v).astype(np.float64))
        dZ2 = (q(dY) @ W3) * (1.0 - H2 * H2)
        dZ1 = (q(dZ2) @ W2) * (1.0 - H1 * H1)
        g = {"W1": q(dZ1).T @ X, "b1": dZ1.sum(0), "W2": q(dZ2).T @ H1, "b2": dZ2.sum(0), "W3": q(dY).T @ H2,
             "b3": dY.sum(0)}
        for k, (o, m) in OFF.items():
            grad[s * SET_PARAMS + o:s * SET_PARAMS + o + m] = g[k].ravel()
    return grad, loss / (n * OUT)


class Adam:
    """The optimizer the kernels run, on FP32 parameters."""

    def __init__(self, params: np.ndarray):
        self.w = np.asarray(params, np.float32).copy()
        self.m = np.zeros_like(self.w)
        self.v = np.zeros_like(self.w)
        self.t = 0

    def step(self, grad: np.ndarray, lr: float) -> np.ndarray:
        self.t += 1
        g = np.asarray(grad, np.float32)
        self.m = np.float32(0.9) * self.m + np.float32(0.1) * g
        self.v = np.float32(0.999) * self.v + np.float32(0.001) * g * g
        c1, c2 = np.float32(1 - 0.9 ** self.t), np.float32(1 - 0.999 ** self.t)
        self.w = self.w - np.float32(lr) * (self.m / c1) / (np.sqrt(self.v / c2) + np.float32(1e-8))
        return self.w
