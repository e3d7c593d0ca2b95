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


def _trunc(S, chi, threshold, relative):
    s = S.numpy()
    keep = s[:chi] if chi else s
    thr = s[0] * threshold if relative else threshold
    k = int(np.count_nonzero(keep > thr))
    return k, float(np.sum(s[k:].astype(np.float64) ** 2))


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
    f = torch.sqrt(d) if mode == 1 else d
    A.mul_(f.to(A.dtype)[:, None])
    return A


def _scale_cols(A, d, mode=0):
    f = torch.sqrt(d) if mode == 1 else d
    A.mul_(f.to(A.dtype)[None, :])
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


PATCH = {
    "device": lambda: torch.device("cpu"),
    "permute": _permute,
    "tensordot": _tensordot,
    "svd": _svd,
    "qr": _qr,
    "truncation_rank": _trunc,
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
