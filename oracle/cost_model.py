"""CPU restatement (numpy, float64) of the tile cost model that the library
trains and evaluates on the GPU (newman_gb300/csrc/schedule.cu).

Test infrastructure only: the tests check the GPU forward pass and gradient
against these functions; nothing in the library calls them.  The model has no
counterpart in the reference (mandelbrot.cpp renders its rows in a fixed
order); it decides the order of the tiles, and the tests also check that the
image does not depend on that order.

Model: x (18) -> 64 -> 64 -> 64 -> 1, ReLU between layers, y = W4 h3 + b4.
Parameter vector layout (as the library's): W1[64][18] b1[64] W2[64][64]
b2[64] W3[64][64] b3[64] W4[64] b4[1], weights row-major [out][in].  The GPU
reads FP16 copies of the weights and FP32 biases; `unpack(p, fp16=True)`
gives the same numbers in float64.
"""
import numpy as np

N_IN, N_H = 18, 64
SHAPES = [("W1", (N_H, N_IN)), ("b1", (N_H,)), ("W2", (N_H, N_H)), ("b2", (N_H,)),
          ("W3", (N_H, N_H)), ("b3", (N_H,)), ("W4", (N_H,)), ("b4", (1,))]
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(p, fp16=True):
    """Parameter vector -> dict of float64 arrays.  With fp16, the numbers the
    GPU computes with: FP32 biases and FP16 weights; without, p as it is."""
    p = np.asarray(p)
    out, k = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        a = p[k:k + n]
        if fp16:
            a = a.astype(np.float32)
            if name.startswith("W"):
                a = a.astype(np.float16)
        out[name] = a.astype(np.float64).reshape(shape)
        k += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SHAPES])


def forward(P, X):
    """Predictions for the rows of X, and the cache for backward."""
    X = np.asarray(X, np.float64)
    a1 = X @ P["W1"].T + P["b1"]
    h1 = np.maximum(a1, 0.0)
    a2 = h1 @ P["W2"].T + P["b2"]
    h2 = np.maximum(a2, 0.0)
    a3 = h2 @ P["W3"].T + P["b3"]
    h3 = np.maximum(a3, 0.0)
    y = h3 @ P["W4"] + P["b4"][0]
    return y, (X, a1, h1, a2, h2, a3, h3)


def loss_and_grad(P, X, T):
    """mean((y - T)^2) and its gradient (dict like P)."""
    y, (X, a1, h1, a2, h2, a3, h3) = forward(P, X)
    n = len(y)
    diff = y - np.asarray(T, np.float64)
    loss = float(np.mean(diff * diff))
    dy = 2.0 * diff / n
    g = {"W4": h3.T @ dy, "b4": np.array([dy.sum()])}
    g3 = np.outer(dy, P["W4"]) * (a3 > 0)
    g["W3"], g["b3"] = g3.T @ h2, g3.sum(0)
    g2 = (g3 @ P["W3"]) * (a2 > 0)
    g["W2"], g["b2"] = g2.T @ h1, g2.sum(0)
    g1 = (g2 @ P["W2"]) * (a1 > 0)
    g["W1"], g["b1"] = g1.T @ X, g1.sum(0)
    return loss, g
