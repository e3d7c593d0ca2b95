"""Learned rank predictor for the truncating SVD sweep.

A 3-layer perceptron (width 128, ReLU, sigmoid output) maps per-bond features
-- the bond's position, its local maximal rank, the bond-dimension cap, the
tolerance, and moments of the singular spectrum of the neighbouring bond
that the sweep has just computed -- to the fraction of the local maximal rank
that the discarded-weight rule keeps.  The sweep engine uses the prediction
to size a randomized SVD (sketch of k + oversampling columns, power
iterations) instead of the full Jacobi SVD, and falls back to the full SVD
when the sketch's residual weight exceeds the tolerance.

Training runs on the GPU with the library's own kernels (dense forward /
backward, MSE-through-sigmoid gradient, Adam); the samples come from sweeps
of the plain method (full SVD).  Nothing here has a counterpart in the
reference, which always runs the full SVD (tncontract/onedim/onedim_core.py:317).
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _ops

N_FEATURES = 8


def spectrum_features(bond_pos, kmax_local, chi_cap, dw_tol, s_neighbour):
    """Feature vector of one bond.  ``s_neighbour``: singular values of the
    adjacent bond already factorised (host array, descending)."""
    s = np.asarray(s_neighbour, dtype=np.float64)
    if s.size == 0 or s[0] <= 0:
        s = np.ones(1)
    p = s * s
    p = p / p.sum()
    n = p.size
    ent = float(-(p * np.log(np.maximum(p, 1e-300))).sum() / max(math.log(n), 1e-12)) if n > 1 else 0.0
    pr = float(1.0 / (p * p).sum() / n)
    top = float(p[: max(1, n // 10)].sum())
    tail = np.cumsum(p[::-1])[::-1]
    k_nb = int(np.count_nonzero(tail > dw_tol))
    return np.array([bond_pos, math.log2(max(kmax_local, 1)) / 12.0, math.log2(max(chi_cap, 1)) / 12.0,
                     ent, pr, top, k_nb / n, -math.log10(max(dw_tol, 1e-300)) / 16.0], dtype=np.float32)


def dw_rank(S_host, dw_tol, chi=0, total=None):
    """Smallest k with sum_{j>=k} s_j^2 <= dw_tol * total (total defaults to
    sum s^2), capped at chi (0 = no cap)."""
    s2 = np.asarray(S_host, dtype=np.float64) ** 2
    tot = float(s2.sum()) if total is None else float(total)
    if tot <= 0:
        return 1
    tail = tot - np.cumsum(np.concatenate([[0.0], s2]))  # weight left after keeping j values
    k = int(np.argmax(tail <= dw_tol * tot)) if np.any(tail <= dw_tol * tot) else len(s2)
    k = max(k, 1)
    if chi:
        k = min(k, chi)
    return k


class RankMLP:
    """in -> 128 -> 128 -> 1, parameters in one flat FP32 device buffer."""

    def __init__(self, width=128, seed=0, n_in=N_FEATURES):
        self.n_in, self.width = n_in, width
        rng = np.random.default_rng(seed)
        shapes = [(width, n_in), (width,), (width, width), (width,), (1, width), (1,)]
        parts = []
        for shp in shapes:
            if len(shp) == 2:
                lim = math.sqrt(6.0 / shp[1])  # He-uniform for ReLU layers
                parts.append(rng.uniform(-lim, lim, shp).astype(np.float32).ravel())
            else:
                parts.append(np.zeros(shp, np.float32))
        self.shapes = shapes
        self.sizes = [int(np.prod(s)) for s in shapes]
        self.offsets = np.cumsum([0] + self.sizes)
        self.params = torch.from_numpy(np.concatenate(parts)).to(_ops.device())
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0

    def _view(self, buf, i):
        return buf[self.offsets[i]:self.offsets[i + 1]]

    def _dense(self, W, b, x, nin, nout, act):
        return _ops.dense_forward(W, b, x, nin, nout, act)

    def forward(self, X):
        """X: (batch, n_in) device float32 -> (y, activations)."""
        X = X.contiguous()
        P = self.params
        h1 = self._dense(self._view(P, 0), self._view(P, 1), X, self.n_in, self.width, 1)
        h2 = self._dense(self._view(P, 2), self._view(P, 3), h1, self.width, self.width, 1)
        y = self._dense(self._view(P, 4), self._view(P, 5), h2, self.width, 1, 2)
        return y.reshape(-1), (X, h1, h2)

    def backward(self, X, T):
        """Gradients of mean((y - T)^2) into self.grads; returns the loss."""
        y, (X, h1, h2) = self.forward(X)
        B = X.shape[0]
        g3 = _ops.mse_sigmoid_grad(y, T)
        P, G = self.params, self.grads
        gh2 = _ops.empty((B, self.width), torch.float32)
        _ops.dense_backward(self._view(P, 4), h2, h2, g3.reshape(B, 1), self._view(G, 4), self._view(G, 5), gh2,
                            self.width, 1, 1)
        gh1 = _ops.empty((B, self.width), torch.float32)
        _ops.dense_backward(self._view(P, 2), h1, h1, gh2, self._view(G, 2), self._view(G, 3), gh1,
                            self.width, self.width, 1)
        _ops.dense_backward(self._view(P, 0), X, None, gh1, self._view(G, 0), self._view(G, 1), None,
                            self.n_in, self.width, 0)
        d = (y - T).float()
        return float((d * d).mean().item())

    def adam(self, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step += 1
        _ops.adam_step(self.params, self.grads, self.m, self.v, lr, b1, b2, eps, self.step)

    def fit(self, X, T, steps=400, lr=2e-3, batch=256, seed=0):
        """Adam on minibatches of (X, T) (host or device arrays); returns the
        loss history."""
        X = torch.as_tensor(np.asarray(X, np.float32)).to(_ops.device())
        T = torch.as_tensor(np.asarray(T, np.float32)).to(_ops.device())
        rng = np.random.default_rng(seed)
        n = X.shape[0]
        hist = []
        for _ in range(steps):
            idx = torch.from_numpy(rng.integers(0, n, size=min(batch, n))).to(X.device)
            hist.append(self.backward(X[idx].contiguous(), T[idx].contiguous()))
            self.adam(lr)
        return hist

    def predict(self, feats):
        X = torch.as_tensor(np.asarray(feats, np.float32).reshape(-1, self.n_in)).to(_ops.device())
        y, _ = self.forward(X)
        return y.cpu().numpy()

    def save(self, path):
        np.savez(path, params=self.params.cpu().numpy(), width=self.width, n_in=self.n_in)

    @classmethod
    def load(cls, path):
        z = np.load(path)
        m = cls(width=int(z["width"]), n_in=int(z["n_in"]))
        m.params.copy_(torch.from_numpy(z["params"]))
        return m
