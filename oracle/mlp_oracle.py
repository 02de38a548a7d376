"""CPU oracle of the learned warm start (test infrastructure only).

Only the tests, `__graft_entry__.smoke()` and the bench's CPU leg use this
module, as the checker of the library's MLP kernels; the library never calls
it.

The reference (evoc-rs 0.2.7) has no learned initialisation: this network is
the warm-start form that sits beside the plain method. The oracle restates
the published algorithm the library implements:

  * a multilayer perceptron  x -> GELU(x W1^T + b1) -> GELU(. W2^T + b2)
    -> . W3^T + b3, GELU in its tanh form x/2 (1 + tanh(sqrt(2/pi)
    (x + 0.044715 x^3))) (Hendrycks & Gimpel, 2016);
  * mean squared error L = mean((y - t)^2) over all n * out_dim entries;
  * its gradients by back-propagation;
  * Adam with bias correction (Kingma & Ba, 2015);
  * orthogonal Procrustes alignment R = U V^T of M = U S V^T
    (Schoenemann, 1966).

Where the library rounds to BF16 (the GEMM operands: the points, W1..W3, the
hidden activations and the back-propagated hidden-layer gradients) the oracle
rounds at the same places, to nearest even; everything else is float64 here
and float32 on the GPU, so the two agree to accumulation-order error.
`exact=True` turns the rounding off, for the finite-difference check of the
gradient formulas themselves.
"""
from __future__ import annotations

import math

import numpy as np


def bf16(x) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


_GELU_C = math.sqrt(2.0 / math.pi)
_GELU_A = 0.044715


def gelu(x: np.ndarray) -> np.ndarray:
    """GELU, tanh form: x/2 (1 + tanh(c (x + a x^3)))."""
    return 0.5 * x * (1.0 + np.tanh(_GELU_C * (x + _GELU_A * x ** 3)))


def gelu_grad(x: np.ndarray) -> np.ndarray:
    t = np.tanh(_GELU_C * (x + _GELU_A * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * _GELU_C * (1.0 + 3.0 * _GELU_A * x * x)


def unpack(flat: np.ndarray, in_dim: int, hidden: int, out_dim: int) -> dict:
    """Packed parameters: W1 (h x in), b1, W2 (h x h), b2, W3 (out x h), b3."""
    sizes = [("w1", (hidden, in_dim)), ("b1", (hidden,)), ("w2", (hidden, hidden)),
             ("b2", (hidden,)), ("w3", (out_dim, hidden)), ("b3", (out_dim,))]
    out, at = {}, 0
    for name, shape in sizes:
        cnt = int(np.prod(shape))
        out[name] = np.asarray(flat[at:at + cnt], dtype=np.float64).reshape(shape)
        at += cnt
    assert at == len(flat)
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([np.ravel(d[k]) for k in ("w1", "b1", "w2", "b2", "w3", "b3")])


def n_params(in_dim: int, hidden: int, out_dim: int) -> int:
    return hidden * in_dim + hidden + hidden * hidden + hidden + out_dim * hidden + out_dim


def forward(params: dict, x, exact: bool = False) -> dict:
    r = (lambda a: np.asarray(a, dtype=np.float64)) if exact else bf16
    xb = r(x)
    w1, w2, w3 = r(params["w1"]), r(params["w2"]), r(params["w3"])
    h1 = xb @ w1.T + params["b1"]
    a1 = r(gelu(h1))
    h2 = a1 @ w2.T + params["b2"]
    a2 = r(gelu(h2))
    y = a2 @ w3.T + params["b3"]
    return {"x": xb, "w1": w1, "w2": w2, "w3": w3, "h1": h1, "a1": a1, "h2": h2, "a2": a2,
            "y": y}


def loss_and_gradients(params: dict, x, target, exact: bool = False):
    """Mean squared error and its gradient for every parameter (a dict)."""
    r = (lambda a: np.asarray(a, dtype=np.float64)) if exact else bf16
    f = forward(params, x, exact)
    t = np.asarray(target, dtype=np.float64)
    n, out = t.shape
    d = f["y"] - t
    loss = float(np.mean(d * d))
    dy = 2.0 * d / (n * out)
    g = {"w3": dy.T @ f["a2"], "b3": dy.sum(0)}
    dh2 = r((dy @ f["w3"]) * gelu_grad(f["h2"]))
    g["w2"] = dh2.T @ f["a1"]
    g["b2"] = dh2.sum(0)
    dh1 = r((dh2 @ f["w2"]) * gelu_grad(f["h1"]))
    g["w1"] = dh1.T @ f["x"]
    g["b1"] = dh1.sum(0)
    return loss, g


def loss_only(params: dict, x, target, exact: bool = True) -> float:
    y = forward(params, x, exact)["y"]
    d = y - np.asarray(target, dtype=np.float64)
    return float(np.mean(d * d))


def adam(p, m, v, g, t: int, lr: float, beta1: float, beta2: float, eps: float):
    """One Adam step (bias-corrected) on float arrays; returns (p, m, v)."""
    m = beta1 * m + (1.0 - beta1) * g
    v = beta2 * v + (1.0 - beta2) * g * g
    mh = m / (1.0 - beta1 ** t)
    vh = v / (1.0 - beta2 ** t)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def procrustes(m: np.ndarray) -> np.ndarray:
    """Orthogonal R maximising trace(R^T M): U V^T from the SVD M = U S V^T."""
    u, _, vt = np.linalg.svd(np.asarray(m, dtype=np.float64))
    return u @ vt


def align(layout: np.ndarray, pred: np.ndarray) -> np.ndarray:
    """The layout rotated (and shifted) onto the prediction: centre both,
    rotate the layout by the Procrustes solution, add the prediction's mean."""
    t = np.asarray(layout, dtype=np.float64)
    p = np.asarray(pred, dtype=np.float64)
    tm, pm = t.mean(0), p.mean(0)
    r = procrustes((t - tm).T @ (p - pm))
    return (t - tm) @ r + pm
