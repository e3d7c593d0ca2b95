"""Test-only CPU stand-in for ``tncontract_gb300._ops``.

The product has no CPU path: every ``_ops`` function calls the native CUDA
library.  To test the HOST logic (label resolution, axis-move simulation,
control flow of the MPS / PEPS routines) in the CPU test suite, this module
temporarily replaces the ``_ops`` functions with CPU ``torch`` versions.  It
is used only by ``-m "not gpu"`` tests; GPU tests never patch anything.
"""
from __future__ import annotations

import contextlib

import numpy as np
import torch

import tncontract_gb300._ops as ops


def _permute(x, perm, conj=False):
    y = x.permute(*[int(p) for p in perm]).contiguous()
    if conj and y.is_complex():
        y = y.conj().resolve_conj()
    return y


def _tensordot(a, b, axes_a, axes_b):
    dt = torch.promote_types(a.dtype, b.dtype)
    return torch.tensordot(a.to(dt), b.to(dt), dims=(list(axes_a), list(axes_b))).contiguous()


def _svd(M, max_sweeps=0, tol=0.0, check=True, info_out=None):
    u, s, vh = np.linalg.svd(M.numpy(), full_matrices=False)
    return torch.from_numpy(u), torch.from_numpy(s), torch.from_numpy(vh)


def _qr(M):
    q, r = np.linalg.qr(M.numpy(), mode="reduced")
    return torch.from_numpy(q), torch.from_numpy(r)


def _qr_r(M, adjoint=False, check=True):
    X = M.numpy()
    X = np.conj(X).T if adjoint else X
    return torch.from_numpy(np.ascontiguousarray(np.linalg.qr(X, mode="r")))


def _trunc(S, chi, threshold, relative, with_smax=False, kdev_out=None):
    s = S.numpy()
    keep = s[:chi] if chi else s
    thr = s[0] * threshold if relative else threshold
    k = int(np.count_nonzero(keep > thr))
    if kdev_out is not None:
        kdev_out.append(torch.tensor([k], dtype=torch.int64))
    disc = float(np.sum(s[k:].astype(np.float64) ** 2))
    if with_smax:
        return k, disc, float(s[0]) if s.size else 0.0
    return k, disc


def _strided(t, off, rows, cols, ld):
    return torch.as_strided(t, (rows, cols), (ld, 1), t.storage_offset() + off)


def _gemm(opA, opB, m, n, k, A, lda, B, ldb, Cm, ldc, alpha=1.0, beta=0.0, batch=1, sA=0, sB=0, sC=0):
    ops_ = {0: lambda x: x, 1: lambda x: x.T, 2: lambda x: x.conj().T, 3: lambda x: x.conj()}
    a_shape = (k, m) if opA in (1, 2) else (m, k)
    b_shape = (n, k) if opB in (1, 2) else (k, n)
    for b in range(batch):
        a = ops_[opA](_strided(A, b * sA, a_shape[0], a_shape[1], lda))
        bb = ops_[opB](_strided(B, b * sB, b_shape[0], b_shape[1], ldb))
        c = _strided(Cm, b * sC, m, n, ldc)
        r = complex(alpha) * (a @ bb) if Cm.is_complex() else float(complex(alpha).real) * (a @ bb)
        if complex(beta) != 0:
            r = r + (complex(beta) if Cm.is_complex() else complex(beta).real) * c
        c.copy_(r)
    return Cm


def _svd_rows(M, max_sweeps=0, tol=0.0):
    m, n = M.shape
    u, s, vh = np.linalg.svd(M.numpy(), full_matrices=False)
    W = s[:, None] * vh if m <= n else s[:, None] * np.conj(u).T
    return (torch.from_numpy(np.ascontiguousarray(W)), torch.from_numpy(s),
            torch.arange(len(s), dtype=torch.int64), torch.zeros(4, dtype=torch.int32))


def _svd_rows_stage(M, max_sweeps, tol, stop_tol, block_rows=0):
    return _svd_rows(M, max_sweeps, tol)


def _gather(W, order, kdev, kmax, S=None, mode=0):
    k = min(int(kdev.reshape(-1)[0]), kmax)
    rows = W[order[:k]]
    if mode == 0:
        return rows.contiguous()
    return (rows.conj().T / S[:k].to(W.dtype)[None, :]).contiguous()


def _sort_rows(M):
    nrm = (M.abs() ** 2).sum(1).double()
    order = torch.from_numpy(np.argsort(-nrm.numpy(), kind="stable").copy())
    rank = torch.empty_like(order)
    rank[order] = torch.arange(len(order))
    return M[order].contiguous(), order, rank


def _permute_rows(X, idx):
    return X[idx].contiguous()


def _copy2d(src, rows, cols, lds, dst, ldd, src_off=0, dst_off=0):
    s = src.reshape(-1)
    d = dst.reshape(-1)
    for i in range(rows):
        d[dst_off + i * ldd: dst_off + i * ldd + cols] = s[src_off + i * lds: src_off + i * lds + cols]
    return dst


def _mps_mpo_site(A, W, layout):
    dt = torch.promote_types(A.dtype, W.dtype)
    t = torch.tensordot(A.to(dt), W.to(dt), dims=([0], [1]))  # (l, r, po, wl, wr)
    l, r, po, wl, wr = t.shape
    if layout == 0:
        return t.permute(0, 3, 2, 1, 4).reshape(l * wl, po, r * wr).contiguous()
    return t.permute(2, 0, 3, 1, 4).reshape(po, l * wl, r * wr).contiguous()


def _scale_rows(A, d, mode=0):
    A.mul_(_mode(d, mode).to(A.dtype)[:, None])
    return A


def _mode(d, mode):
    if mode == 1:
        return torch.sqrt(d)
    if mode == 2:
        return torch.where(d > 0, 1 / d, torch.zeros_like(d))
    if mode == 3:
        return torch.where(d > 0, 1 / (d * d), torch.zeros_like(d))
    return d


def _scale_cols(A, d, mode=0):
    A.mul_(_mode(d, mode).to(A.dtype)[None, :])
    return A


def _diag_matrix(s, dtype):
    return torch.diag(s).to(dtype)


def _trace(x, a1, a2):
    return torch.from_numpy(np.array(np.trace(x.numpy(), axis1=a1, axis2=a2)))


def _scale(x, alpha, conj=False, out=None):
    y = x.conj().resolve_conj() if (conj and x.is_complex()) else x
    z = complex(alpha)
    r = y * (z if x.is_complex() else z.real)
    if out is not None:
        out.copy_(r)
        return out
    return r.contiguous()


def _axpby(alpha, x, beta, y):
    a, b = complex(alpha), complex(beta)
    if not y.is_complex():
        a, b = a.real, b.real
    y.copy_(a * x + b * y)
    return y


def _fill_gaussian(shape, dtype, seed):
    rng = np.random.default_rng(int(seed) & 0xFFFFFFFF)
    a = rng.standard_normal(shape)
    if dtype.is_complex:
        a = a + 1j * rng.standard_normal(shape)
    return torch.from_numpy(a).to(dtype)


def _dense_forward(W, b, x, nin, nout, act):
    y = x @ W.reshape(nout, nin).T + b
    if act == 1:
        y = torch.relu(y)
    elif act == 2:
        y = torch.sigmoid(y)
    return y.contiguous()


def _dense_backward(W, x, act_in, g, dW, db, gin, nin, nout, relu_mask):
    g = g.reshape(-1, nout)
    dW.copy_((g.T @ x).reshape(-1))
    db.copy_(g.sum(0))
    if gin is not None:
        r = g @ W.reshape(nout, nin)
        if relu_mask:
            r = r * (act_in > 0)
        gin.copy_(r)


def _mse_sigmoid_grad(y, t):
    return (2 * (y - t) * y * (1 - y) / y.shape[0]).contiguous()


def _adam_step(p, g, m, v, lr, b1, b2, eps, step):
    m.mul_(b1).add_((1 - b1) * g)
    v.mul_(b2).add_((1 - b2) * g * g)
    p.sub_(lr * (m / (1 - b1 ** step)) / (torch.sqrt(v / (1 - b2 ** step)) + eps))


def _tensordot_many(items):
    return [_tensordot(a, b, aa, ab) for a, b, aa, ab in items]


PATCH = {
    "tensordot_many": _tensordot_many,
    "fill_gaussian": _fill_gaussian,
    "dense_forward": _dense_forward,
    "dense_backward": _dense_backward,
    "mse_sigmoid_grad": _mse_sigmoid_grad,
    "adam_step": _adam_step,
    "device": lambda: torch.device("cpu"),
    "permute": _permute,
    "tensordot": _tensordot,
    "svd": _svd,
    "qr": _qr,
    "qr_r": _qr_r,
    "truncation_rank": _trunc,
    "gemm": _gemm,
    "svd_rows": _svd_rows,
    "svd_rows_stage": _svd_rows_stage,
    "gather_rows": _gather,
    "sort_rows": _sort_rows,
    "permute_rows": _permute_rows,
    "copy2d": _copy2d,
    "mps_mpo_site": _mps_mpo_site,
    "scale_rows": _scale_rows,
    "scale_cols": _scale_cols,
    "diag_matrix": _diag_matrix,
    "trace": _trace,
    "scale": _scale,
    "axpby": _axpby,
    "conj": lambda x: x.conj().resolve_conj() if x.is_complex() else x,
    "cast": lambda x, dt: x if x.dtype == dt else x.to(dt),
    "nrm2": lambda x: float(torch.linalg.vector_norm(x.reshape(-1).to(torch.complex128)).item()),
    "nrm2_device": lambda x: torch.linalg.vector_norm(x.reshape(-1).to(torch.complex128)).reshape(1),
    "matmul": lambda a, b, opA=0, opB=0, out=None: (
        {0: a, 1: a.T, 2: a.conj().T, 3: a.conj()}[opA] @ {0: b, 1: b.T, 2: b.conj().T, 3: b.conj()}[opB]
    ).contiguous(),
}


@contextlib.contextmanager
def cpu_ops():
    saved = {k: getattr(ops, k) for k in PATCH}
    saved_slice = ops.slice_last
    try:
        for k, v in PATCH.items():
            setattr(ops, k, v)
        yield
    finally:
        for k, v in saved.items():
            setattr(ops, k, v)
        ops.slice_last = saved_slice
