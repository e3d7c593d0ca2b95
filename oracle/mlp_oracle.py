"""CPU oracle for the learned rank predictor -- TEST INFRASTRUCTURE ONLY.

Float64 NumPy restatement of the math the GPU kernels of
``tncontract_gb300/csrc/tnc_mlp.cu`` implement: dense layers with ReLU /
sigmoid, the mean-squared-error gradient through the sigmoid, backward
passes, and Adam (Kingma & Ba 2015).  The reference library has no learned
component; this is the checker for the gradients the GPU training computes.
Also restates the discarded-weight truncation rule used with the predictor
(a rule the reference lacks: smallest k with sum_{j>=k} s_j^2 <= tol * sum s^2).
"""
from __future__ import annotations

import numpy as np


def unpack(params, n_in, width):
    sizes = [width * n_in, width, width * width, width, width, 1]
    offs = np.cumsum([0] + sizes)
    p = [params[offs[i]:offs[i + 1]] for i in range(6)]
    return (p[0].reshape(width, n_in), p[1], p[2].reshape(width, width), p[3], p[4].reshape(1, width), p[5])


def forward(params, X, n_in, width):
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(params, np.float64), n_in, width)
    X = np.asarray(X, np.float64)
    h1 = np.maximum(X @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    z = h2 @ W3.T + b3
    y = 1.0 / (1.0 + np.exp(-z))
    return y.reshape(-1), (X, h1, h2)


def grads(params, X, T, n_in, width):
    """Gradient of mean((y - T)^2) with respect to the flat parameters."""
    W1, b1, W2, b2, W3, b3 = unpack(np.asarray(params, np.float64), n_in, width)
    y, (X, h1, h2) = forward(params, X, n_in, width)
    B = X.shape[0]
    g3 = (2.0 * (y - T) * y * (1.0 - y) / B).reshape(B, 1)
    dW3 = g3.T @ h2
    db3 = g3.sum(0)
    gh2 = (g3 @ W3) * (h2 > 0)
    dW2 = gh2.T @ h1
    db2 = gh2.sum(0)
    gh1 = (gh2 @ W2) * (h1 > 0)
    dW1 = gh1.T @ X
    db1 = gh1.sum(0)
    return np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3.ravel(), db3])


def adam(p, g, m, v, lr, b1, b2, eps, step):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v


def dw_keep(s, tol, chi=0):
    """Discarded-weight rule: smallest k with sum_{j>=k} s_j^2 <= tol * sum s_j^2."""
    s2 = np.asarray(s, np.float64) ** 2
    tot = s2.sum()
    tail = tot - np.concatenate([[0.0], np.cumsum(s2)])
    ok = np.nonzero(tail <= tol * tot)[0]
    k = max(int(ok[0]) if ok.size else len(s2), 1)
    return min(k, chi) if chi else k


def svd_compress_dw(sites, chi, tol):
    """MatrixProductState.svd_compress with the discarded-weight rule in the
    truncating sweep (QR left sweep, normalise, SVD right sweep, restore the
    norm), sites (phys, left, right)."""
    import tn_oracle as O
    s1 = O.left_canonise_qr(sites)
    nrm = np.linalg.norm(s1[-1])
    s1[-1] = s1[-1] / nrm
    rev = O.mps_reverse(s1)
    N = len(rev)
    norm = 1.0
    for i in range(N - 1):
        a = rev[i]
        d, l, r = a.shape
        u, s, vh = np.linalg.svd(a.reshape(d * l, r), full_matrices=False)
        k = dw_keep(s, tol, chi)
        norm *= s[0]
        rev[i] = u[:, :k].reshape(d, l, k)
        sv = (s[:k] / s[0])[:, None] * vh[:k]
        nxt = np.tensordot(sv, rev[i + 1], (1, 1))
        rev[i + 1] = np.ascontiguousarray(nxt.transpose(1, 0, 2))
    rev[-1] = rev[-1] * norm
    out = O.mps_reverse(rev)
    out[0] = out[0] * nrm
    return out
