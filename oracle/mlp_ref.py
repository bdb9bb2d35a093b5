"""ORACLE — TEST INFRASTRUCTURE ONLY.

FP64 numpy forward and backward of the contact-parameter MLP
(16 -> 64 -> 64 -> 64 -> 1, ReLU, sigmoid, MSE), rounding operands to BF16 at
the points where the device kernels do, so that the device gradients can be
checked against it. bf16=False gives the exact FP64 network for a
finite-difference check of the formulas themselves.
"""
import numpy as np

OFF_W1, OFF_B1 = 0, 1024
OFF_W2, OFF_B2 = 1088, 5184
OFF_W3, OFF_B3 = 5248, 9344
OFF_W4, OFF_B4 = 9408, 9472
NPARAM = 9473


def bf16(a):
    """Round-to-nearest-even to bfloat16, returned as float64."""
    a = np.asarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w):
    w = np.asarray(w, dtype=np.float64)
    return (w[OFF_W1:OFF_B1].reshape(64, 16), w[OFF_B1:OFF_W2], w[OFF_W2:OFF_B2].reshape(64, 64), w[OFF_B2:OFF_W3],
            w[OFF_W3:OFF_B3].reshape(64, 64), w[OFF_B3:OFF_W4], w[OFF_W4:OFF_B4], w[OFF_B4])


def forward_backward(w, X, y, bf=True):
    r = bf16 if bf else (lambda a: np.asarray(a, dtype=np.float64))
    W1, b1, W2, b2, W3, b3, w4, b4 = unpack(w)
    X = r(X)
    W1r, W2r, W3r = r(W1), r(W2), r(W3)
    Z1 = X @ W1r.T
    H1 = r(np.maximum(Z1 + b1, 0.0))
    Z2 = H1 @ W2r.T
    H2 = r(np.maximum(Z2 + b2, 0.0))
    Z3 = H2 @ W3r.T
    H3 = np.maximum(Z3 + b3, 0.0)
    z4 = H3 @ w4 + b4
    p = 1.0 / (1.0 + np.exp(-z4))
    B = len(y)
    loss = np.mean((p - y) ** 2)
    d4 = 2.0 * (p - y) * p * (1.0 - p) / B
    g = np.zeros(NPARAM)
    g[OFF_W4:OFF_B4] = H3.T @ d4
    g[OFF_B4] = d4.sum()
    D3 = r(np.outer(d4, w4) * (H3 > 0))
    g[OFF_W3:OFF_B3] = (D3.T @ H2).ravel()
    g[OFF_B3:OFF_W4] = D3.sum(0)
    D2 = r((D3 @ W3r) * (H2 > 0))
    g[OFF_W2:OFF_B2] = (D2.T @ H1).ravel()
    g[OFF_B2:OFF_W3] = D2.sum(0)
    D1 = r((D2 @ W2r) * (H1 > 0))
    g[OFF_W1:OFF_B1] = (D1.T @ X).ravel()
    g[OFF_B1:OFF_W2] = D1.sum(0)
    return loss, g, p
