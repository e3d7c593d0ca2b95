"""Device operations on CUDA ``torch.Tensor`` storage, each one call into the
native C ABI (``include/tncontract_gb300.h``).

PyTorch provides device memory and the current stream only; every
arithmetic / data-movement step of the hot path runs in the library's own
sm_103a kernels.  All tensors handled here are dense and C-contiguous.
"""
from __future__ import annotations

import ctypes as C
import math
import threading

import numpy as np
import torch

from . import _lib as L

_CODE = {torch.float32: L.F32, torch.float64: L.F64,
         torch.complex64: L.C64, torch.complex128: L.C128}
_REAL = {torch.float32: torch.float32, torch.float64: torch.float64,
         torch.complex64: torch.float32, torch.complex128: torch.float64}
_NP2TORCH = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
             np.dtype(np.complex64): torch.complex64, np.dtype(np.complex128): torch.complex128}


class LinAlgError(np.linalg.LinAlgError):
    pass


def device():
    return torch.device("cuda", torch.cuda.current_device())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return C.c_void_p(t.data_ptr())


def code(dtype):
    try:
        return _CODE[dtype]
    except KeyError:
        raise TypeError("unsupported dtype %s (float32/float64/complex64/complex128)" % dtype)


def real_dtype(dtype):
    return _REAL[dtype]


def is_complex(dtype):
    return dtype in (torch.complex64, torch.complex128)


def _pair(x):
    z = complex(x)
    return (C.c_double * 2)(z.real, z.imag)


def _arr(ctype, seq):
    seq = list(seq)
    return (ctype * max(1, len(seq)))(*seq)


# When set to a dict, every C-ABI call is bracketed by CUDA events on the
# current stream: PROFILE[name] -> list of (start, end, algorithmic flops).
# PROFILE_ONLY (a set of names) restricts the bracketing to those calls.
PROFILE = None
PROFILE_ONLY = None


def _call(name, *args, flops=0.0):
    fn = getattr(L.lib(), name)
    prof = PROFILE
    if prof is None or (PROFILE_ONLY is not None and name not in PROFILE_ONLY):
        L.check(name, fn(*args))
        return
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record()
    st = fn(*args)
    e.record()
    prof.setdefault(name, []).append((s, e, float(flops)))
    L.check(name, st)


def profile_summary(prof):
    """{name: (launches, total ms, total flops)} after a synchronize."""
    out = {}
    for name, recs in prof.items():
        ms = sum(s.elapsed_time(e) for s, e, _ in recs)
        out[name] = (len(recs), ms, sum(f for _, _, f in recs))
    return out


def empty(shape, dtype):
    return torch.empty(tuple(int(s) for s in shape), dtype=dtype, device=device())


def zeros(shape, dtype):
    # a zero fill is allocation plumbing (a memset), not hot-path arithmetic
    return torch.zeros(tuple(int(s) for s in shape), dtype=dtype, device=device())


_WS = {}


def workspace(nbytes):
    """Per-stream reusable workspace (stream ordering makes reuse safe)."""
    key = (torch.cuda.current_device(), torch.cuda.current_stream().cuda_stream)
    buf = _WS.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 1 << 20), dtype=torch.uint8, device=device())
        _WS[key] = buf
    return buf


# ------------------------------------------------------------------ creation


def to_device(x, dtype=None):
    """Copy array-like ``x`` to a new contiguous device tensor.  Integer and
    boolean inputs become float64 (the engine computes in floating point)."""
    if isinstance(x, torch.Tensor):
        t = x
        if dtype is not None and t.dtype != dtype:
            t = t.to(dtype)
        if t.dtype not in _CODE:
            t = t.to(torch.complex128 if t.is_complex() else torch.float64)
        if t.device.type != "cuda" or t.device.index != torch.cuda.current_device():
            return t.contiguous().to(device())
        return t.contiguous().clone()
    a = np.asarray(x)
    if a.dtype not in _NP2TORCH:
        a = a.astype(np.complex128 if np.iscomplexobj(a) else np.float64)
    if dtype is not None:
        a = a.astype({v: k for k, v in _NP2TORCH.items()}[dtype])
    return torch.from_numpy(np.ascontiguousarray(a)).to(device())


def copy(t):
    return t.clone()


# ------------------------------------------------------------------ movement


MAX_KERNEL_RANK = 8  # tnc_permute / tnc_trace take at most this many axes


def fuse_permutation(shape, perm):
    """The same data movement on fewer axes: unit axes dropped, and input axes
    that stay adjacent and in order in the output fused into one.  Returns
    (fused input shape, fused permutation)."""
    keep = [a for a in range(len(shape)) if shape[a] != 1]
    index = {a: i for i, a in enumerate(keep)}
    dims = [int(shape[a]) for a in keep]
    p = [index[a] for a in perm if shape[a] != 1]
    groups = []
    for a in p:
        if groups and groups[-1][-1] + 1 == a:
            groups[-1].append(a)
        else:
            groups.append([a])
    by_input = sorted(range(len(groups)), key=lambda g: groups[g][0])
    fused_shape = [int(np.prod([dims[a] for a in groups[g]], dtype=np.int64)) for g in by_input]
    position = {g: i for i, g in enumerate(by_input)}
    return fused_shape, [position[g] for g in range(len(groups))]


def permutation_steps(shape, perm, max_rank=MAX_KERNEL_RANK):
    """Permutations of at most ``max_rank`` axes whose succession is
    transpose(., perm): the fused permutation itself when it is small
    enough, else single-axis moves (each a fused permutation of at most four
    axes, one pass over the data) until the rest fits.  Each step is
    (input shape, permutation) on the current contiguous layout."""
    n = len(shape)
    fs, fp = fuse_permutation(shape, perm)
    if len(fs) <= max_rank:
        return [(fs, fp)]
    order = list(range(n))   # original axis at each current position
    steps = []
    for t in range(n):
        current = [int(shape[a]) for a in order]
        rest = [order.index(perm[k]) for k in range(n)]
        fs, fp = fuse_permutation(current, rest)
        if len(fs) <= max_rank:
            steps.append((fs, fp))
            return steps
        pos = order.index(perm[t])
        if pos == t:
            continue
        move = list(range(t)) + [pos] + list(range(t, pos)) + list(range(pos + 1, n))
        steps.append(fuse_permutation(current, move))
        order = [order[i] for i in move]
    return steps


def _permute_kernel(x, shape, perm, conj):
    out = empty([shape[p] for p in perm], x.dtype)
    _call("tnc_permute", code(x.dtype), _p(x), _p(out), len(shape),
          _arr(C.c_int64, shape), _arr(C.c_int, perm), int(conj), _stream())
    return out


def permute(x, perm, conj=False):
    """Return transpose(x, perm) (optionally conjugated) as a new tensor;
    ``x`` itself when the permutation is the identity and no conj is asked.
    Tensors of more than ``MAX_KERNEL_RANK`` axes are moved in fused steps of
    at most that many (``permutation_steps``)."""
    perm = [int(p) for p in perm]
    conj = bool(conj) and is_complex(x.dtype)
    if perm == list(range(x.dim())) and not conj:
        return x
    x = x.contiguous()
    shape = [x.shape[p] for p in perm]
    moving = [p for p in perm if x.shape[p] != 1]
    if not conj and moving == sorted(moving):
        return x.reshape(shape)  # only unit axes move: a view suffices
    if x.numel() == 0:
        return empty(shape, x.dtype)
    if x.dim() <= MAX_KERNEL_RANK:
        return _permute_kernel(x, list(x.shape), perm, conj)
    cur = x
    for i, (s, p) in enumerate(permutation_steps(list(x.shape), perm)):
        if not s:
            s, p = [cur.numel()], [0]
        cur = _permute_kernel(cur.reshape(s), s, p, conj and i == 0)
    return cur.reshape(shape)


def rollaxis(x, axis, start):
    """np.rollaxis semantics (used by the reference's axis moves)."""
    n = x.dim()
    axis = axis % n if n else 0
    if start < 0:
        start += n
    order = list(range(n))
    order.remove(axis)
    if start > axis:
        start -= 1
    order.insert(start, axis)
    return permute(x, order)


def cast(x, dtype):
    if x.dtype == dtype:
        return x
    out = empty(x.shape, dtype)
    if x.numel():
        _call("tnc_cast", code(x.dtype), code(dtype), x.numel(), _p(x.contiguous()), _p(out), _stream())
    return out


def scale(x, alpha, conj=False, out=None):
    x = x.contiguous()
    if out is None:
        out = empty(x.shape, x.dtype)
    if x.numel():
        _call("tnc_scale", code(x.dtype), x.numel(), _pair(alpha), _p(x), _p(out),
              int(bool(conj) and is_complex(x.dtype)), _stream())
    return out


def conj(x):
    if not is_complex(x.dtype):
        return x
    return scale(x, 1.0, conj=True)


def axpby(alpha, x, beta, y):
    """y <- alpha x + beta y (in place on y)."""
    if x.numel():
        _call("tnc_axpby", code(x.dtype), x.numel(), _pair(alpha), _p(x.contiguous()),
              _pair(beta), _p(y), _stream())
    return y


def add(x, y):
    out = y.clone()
    return axpby(1.0, x, 1.0, out)


def copy2d(src, rows, cols, lds, dst, ldd, src_off=0, dst_off=0):
    """dst[i, j] = src[i, j] for a rows x cols block (element offsets)."""
    if rows * cols:
        es = src.element_size()
        _call("tnc_copy2d", code(src.dtype), rows, cols, C.c_void_p(src.data_ptr() + src_off * es),
              lds, C.c_void_p(dst.data_ptr() + dst_off * es), ldd, _stream())
    return dst


def slice_last(data, k):
    """Contiguous copy of data[..., :k] (``data`` itself when k is the full extent)."""
    n = data.shape[-1]
    if k == n:
        return data
    rows = data.numel() // n if n else 0
    out = empty(tuple(data.shape[:-1]) + (k,), data.dtype)
    copy2d(data.contiguous(), rows, k, n, out, k)
    return out


def slice_axis(data, axis, k):
    """Contiguous copy of ``data`` with axis ``axis`` cut to its first k
    entries (``data`` itself when k is the full extent): one 2-D block copy
    of the (before, axis x after) view."""
    data = data.contiguous()
    n = data.shape[axis]
    if k == n:
        return data
    after = int(np.prod(data.shape[axis + 1:], dtype=np.int64))
    rows = int(np.prod(data.shape[:axis], dtype=np.int64))
    out = empty(tuple(data.shape[:axis]) + (k,) + tuple(data.shape[axis + 1:]), data.dtype)
    if out.numel():
        copy2d(data, rows, k * after, n * after, out, k * after)
    return out


def diag_matrix(s, dtype):
    n = s.shape[0]
    out = empty((n, n), dtype)
    if n:
        _call("tnc_diag_matrix", code(dtype), n, _p(s.contiguous()), _p(out), _stream())
    return out


def scale_rows(A, d, mode=0):
    """A[i, :] *= d[i] (mode 0) or sqrt(d[i]) (mode 1), in place; A 2-D."""
    r, c = A.shape
    if r * c:
        _call("tnc_scale_rows", code(A.dtype), r, c, _p(d.contiguous()), int(mode), _p(A), c, _stream())
    return A


def scale_cols(A, d, mode=0):
    r, c = A.shape
    if r * c:
        _call("tnc_scale_cols", code(A.dtype), r, c, _p(d.contiguous()), int(mode), _p(A), c, _stream())
    return A


def trace(x, a1, a2):
    """Trace over axes a1 and a2.  More than ``MAX_KERNEL_RANK`` axes: the
    untouched axes before, between and after the pair are fused first (five
    axes; the trace does not reorder them)."""
    x = x.contiguous()
    out = empty([s for i, s in enumerate(x.shape) if i not in (a1, a2)], x.dtype)
    if not out.numel():
        return out
    shape = list(x.shape)
    if x.dim() > MAX_KERNEL_RANK:
        shape, a1, a2 = fuse_trace(shape, a1, a2)
    _call("tnc_trace", code(x.dtype), len(shape), _arr(C.c_int64, shape), int(a1), int(a2),
          _p(x), _p(out), _stream())
    return out


def fuse_trace(shape, a1, a2):
    """(shape, a1, a2) of the same trace on five axes: the axes before,
    between and after the traced pair fused."""
    lo, hi = min(a1, a2), max(a1, a2)
    prod = lambda d: int(np.prod(d, dtype=np.int64))
    fused = [prod(shape[:lo]), int(shape[lo]), prod(shape[lo + 1:hi]), int(shape[hi]), prod(shape[hi + 1:])]
    return (fused, 1, 3) if a1 < a2 else (fused, 3, 1)


# ------------------------------------------------------------------ reductions


def nrm2_device(x):
    out = torch.empty(1, dtype=torch.float64, device=device())
    _call("tnc_nrm2", code(x.dtype), x.numel(), _p(x.contiguous()), _p(out), _stream())
    return out


def nrm2(x):
    """Frobenius norm as a Python float (synchronises)."""
    return float(nrm2_device(x).item())


def dot_device(x, y, conj_x=False):
    out = torch.empty(2, dtype=torch.float64, device=device())
    _call("tnc_dot", code(x.dtype), x.numel(), _p(x.contiguous()), _p(y.contiguous()),
          int(bool(conj_x)), _p(out), _stream())
    return out


# ------------------------------------------------------------------ contraction


# FP32-class GEMMs at least this large (m*n*k*batch) run on the tcgen05
# tensor-core kernel (TF32 split products); smaller ones and FP64 use the
# CUDA-core kernel.
USE_TC = True
TC_MIN_WORK = 1 << 21
_TC_WS = {}


def _tc_workspace(nbytes):
    key = (torch.cuda.current_device(), torch.cuda.current_stream().cuda_stream)
    buf = _TC_WS.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 1 << 20), dtype=torch.uint8, device=device())
        _TC_WS[key] = buf
    return buf


def gemm(opA, opB, m, n, k, A, lda, B, ldb, Cm, ldc, alpha=1.0, beta=0.0,
         batch=1, sA=0, sB=0, sC=0, tc=None):
    flops = 2.0 * m * n * k * batch * (4 if is_complex(Cm.dtype) else 1)
    dt = code(Cm.dtype)
    use_tc = (USE_TC if tc is None else tc) and dt in (L.F32, L.C64) and min(m, n) >= 64 and k >= 32 \
        and m * n * k * batch >= TC_MIN_WORK and batch <= 65535
    if use_tc:
        sz = C.c_size_t()
        _call("tnc_gemm_tc_workspace_size", dt, m, n, k, batch, C.byref(sz))
        ws = _tc_workspace(sz.value)
        _call("tnc_gemm_tc", dt, opA, opB, m, n, k, _pair(alpha), _p(A), lda, sA,
              _p(B), ldb, sB, _pair(beta), _p(Cm), ldc, sC, batch, _p(ws), sz.value, _stream(), flops=flops)
        return Cm
    _call("tnc_gemm", dt, opA, opB, m, n, k, _pair(alpha), _p(A), lda, sA,
          _p(B), ldb, sB, _pair(beta), _p(Cm), ldc, sC, batch, _stream(), flops=flops)
    return Cm


def matmul(a, b, opA=L.OP_N, opB=L.OP_N, out=None):
    """out = op(a) @ op(b) for 2-D tensors."""
    m = a.shape[1] if opA in (L.OP_T, L.OP_C) else a.shape[0]
    k = a.shape[0] if opA in (L.OP_T, L.OP_C) else a.shape[1]
    n = b.shape[0] if opB in (L.OP_T, L.OP_C) else b.shape[1]
    if out is None:
        out = empty((m, n), a.dtype)
    if m * n:
        gemm(opA, opB, m, n, k, a.contiguous(), a.shape[1], b.contiguous(), b.shape[1], out, n)
    return out


def tensordot(a, b, axes_a, axes_b):
    """np.tensordot(a, b, (axes_a, axes_b)) on device: at most one permute per
    operand (none when the contracted axes are already leading or trailing),
    then one GEMM."""
    axes_a = [int(x) % a.dim() for x in axes_a] if a.dim() else []
    axes_b = [int(x) % b.dim() for x in axes_b] if b.dim() else []
    dt = torch.promote_types(a.dtype, b.dtype)
    a = cast(a.contiguous(), dt)
    b = cast(b.contiguous(), dt)
    free_a = [i for i in range(a.dim()) if i not in axes_a]
    free_b = [i for i in range(b.dim()) if i not in axes_b]
    ma = int(np.prod([a.shape[i] for i in free_a], dtype=np.int64))
    nb = int(np.prod([b.shape[i] for i in free_b], dtype=np.int64))
    kk = int(np.prod([a.shape[i] for i in axes_a], dtype=np.int64))
    out = empty([a.shape[i] for i in free_a] + [b.shape[i] for i in free_b], dt)
    if ma == 0 or nb == 0:
        return out
    if free_a + axes_a == list(range(a.dim())):
        opA, Am, lda = L.OP_N, a, kk
    elif axes_a + free_a == list(range(a.dim())):
        opA, Am, lda = L.OP_T, a, ma
    else:
        opA, Am, lda = L.OP_N, permute(a, free_a + axes_a), kk
    if axes_b + free_b == list(range(b.dim())):
        opB, Bm, ldb = L.OP_N, b, nb
    elif free_b + axes_b == list(range(b.dim())):
        opB, Bm, ldb = L.OP_T, b, kk
    else:
        opB, Bm, ldb = L.OP_N, permute(b, axes_b + free_b), nb
    gemm(opA, opB, ma, nb, kk, Am, max(lda, 1), Bm, max(ldb, 1), out, nb)
    return out


def _tensordot_prepare(a, b, axes_a, axes_b):
    """Operands of np.tensordot(a, b, (axes_a, axes_b)) as one GEMM: at most
    one permute per operand.  Returns (out, gemm arguments or None)."""
    axes_a = [int(x) % a.dim() for x in axes_a] if a.dim() else []
    axes_b = [int(x) % b.dim() for x in axes_b] if b.dim() else []
    dt = torch.promote_types(a.dtype, b.dtype)
    a = cast(a.contiguous(), dt)
    b = cast(b.contiguous(), dt)
    free_a = [i for i in range(a.dim()) if i not in axes_a]
    free_b = [i for i in range(b.dim()) if i not in axes_b]
    ma = int(np.prod([a.shape[i] for i in free_a], dtype=np.int64))
    nb = int(np.prod([b.shape[i] for i in free_b], dtype=np.int64))
    kk = int(np.prod([a.shape[i] for i in axes_a], dtype=np.int64))
    out = empty([a.shape[i] for i in free_a] + [b.shape[i] for i in free_b], dt)
    if ma == 0 or nb == 0:
        return out, None
    if free_a + axes_a == list(range(a.dim())):
        opA, Am, lda = L.OP_N, a, kk
    elif axes_a + free_a == list(range(a.dim())):
        opA, Am, lda = L.OP_T, a, ma
    else:
        opA, Am, lda = L.OP_N, permute(a, free_a + axes_a), kk
    if axes_b + free_b == list(range(b.dim())):
        opB, Bm, ldb = L.OP_N, b, nb
    elif free_b + axes_b == list(range(b.dim())):
        opB, Bm, ldb = L.OP_T, b, kk
    else:
        opB, Bm, ldb = L.OP_N, permute(b, axes_b + free_b), nb
    return out, (opA, opB, ma, nb, kk, Am, max(lda, 1), Bm, max(ldb, 1), out, nb)


def gemm_grouped(problems):
    """Independent products (opA, opB, m, n, k, A, lda, B, ldb, C, ldc) of
    one dtype, C = op(A) op(B), as one launch per TNC_GEMM_GROUP_MAX of them
    (``tnc_gemm_grouped``)."""
    if not problems:
        return
    dt = code(problems[0][9].dtype)
    for i in range(0, len(problems), L.GEMM_GROUP_MAX):
        chunk = problems[i:i + L.GEMM_GROUP_MAX]
        arr = (L.GemmProblem * len(chunk))()
        flops = 0.0
        for slot, (opA, opB, m, n, k, A, lda, B, ldb, Cm, ldc) in zip(arr, chunk):
            slot.opA, slot.opB, slot.m, slot.n, slot.k = opA, opB, m, n, k
            slot.A, slot.lda, slot.B, slot.ldb, slot.C, slot.ldc = A.data_ptr(), lda, B.data_ptr(), ldb, \
                Cm.data_ptr(), ldc
            slot.alpha[0], slot.alpha[1], slot.beta[0], slot.beta[1] = 1.0, 0.0, 0.0, 0.0
            flops += 2.0 * m * n * k * (4 if is_complex(Cm.dtype) else 1)
        _call("tnc_gemm_grouped", dt, len(chunk), arr, _stream(), flops=flops)


def tensordot_many(items):
    """np.tensordot for several independent (a, b, axes_a, axes_b): operand
    permutes where needed, then the products of each dtype as one grouped
    GEMM launch.  Returns the results in order."""
    outs, by_dtype = [], {}
    for a, b, axes_a, axes_b in items:
        out, g = _tensordot_prepare(a, b, axes_a, axes_b)
        outs.append(out)
        if g is not None:
            by_dtype.setdefault(out.dtype, []).append(g)
    for probs in by_dtype.values():
        gemm_grouped(probs)
    return outs


def mps_mpo_site(A, W, layout):
    """Fused MPO-MPS site product; A (din, chl, chr), W (dout, din, Dl, Dr)."""
    din, chl, chr_ = A.shape
    dout, din2, Dl, Dr = W.shape
    assert din == din2
    dt = torch.promote_types(A.dtype, W.dtype)
    A = cast(A.contiguous(), dt)
    W = cast(W.contiguous(), dt)
    shape = (chl * Dl, dout, chr_ * Dr) if layout == 0 else (dout, chl * Dl, chr_ * Dr)
    out = empty(shape, dt)
    _call("tnc_mps_mpo_site", code(dt), din, dout, chl, chr_, Dl, Dr, _p(A), _p(W), _p(out),
          int(layout), _stream())
    return out


# ------------------------------------------------------------------ factorisations


def set_spin_limit(polls=0):
    """Polls every bounded device-side wait makes before giving up
    (``tnc_set_spin_limit``; 0 restores the default), current device."""
    _call("tnc_set_spin_limit", int(polls))


def wait_selftest(kind):
    """Run one CTA whose bounded wait nothing completes (0 grid barrier,
    1 step counter, 2 flag) and return its error word (``TNC_ERR_TIMEOUT``
    when the wait gave up as designed)."""
    ws = workspace(256)
    info = torch.zeros(1, dtype=torch.int32, device=device())
    _call("tnc_wait_selftest", int(kind), _p(ws), 256, _p(info), _stream())
    return int(info[0].item())


def svd(M, max_sweeps=0, tol=0.0, check=True, info_out=None):
    """Thin SVD of a 2-D device matrix: (U, S, VH), S real descending.
    Raises LinAlgError on non-convergence and ValueError on non-finite input,
    like np.linalg.svd / scipy gesvd."""
    M = M.contiguous()
    m, n = M.shape
    k = min(m, n)
    dt = M.dtype
    U = empty((m, k), dt)
    S = empty((k,), real_dtype(dt))
    VH = empty((k, n), dt)
    if k == 0:
        return U, S, VH
    sz = C.c_size_t()
    _call("tnc_svd_workspace_size", code(dt), m, n, C.byref(sz))
    ws = workspace(sz.value)
    info = torch.empty(4, dtype=torch.int32, device=device())
    mm, nn = max(m, n), min(m, n)
    _call("tnc_svd", code(dt), m, n, _p(M), n, _p(U), _p(S), _p(VH), int(max_sweeps), float(tol),
          _p(ws), sz.value, _p(info), _stream(),
          flops=(6.0 * mm * nn * nn + 20.0 * nn ** 3) * (4 if is_complex(dt) else 1))
    if info_out is not None:
        info_out.append(info)
    if check:
        st = int(info[0].item())
        if st == L.ERR_NONFINITE:
            raise ValueError("array must not contain infs or NaNs")
        if st == L.ERR_NOT_CONVERGED:
            raise LinAlgError("SVD did not converge")
        if st != L.OK:
            raise L.NativeError("tnc_svd", st)
    return U, S, VH


def qr(M, check=True):
    """Reduced QR of a 2-D device matrix: (Q, R)."""
    M = M.contiguous()
    m, n = M.shape
    k = min(m, n)
    Q = empty((m, k), M.dtype)
    R = empty((k, n), M.dtype)
    if k == 0:
        return Q, R
    sz = C.c_size_t()
    _call("tnc_qr_workspace_size", code(M.dtype), m, n, C.byref(sz))
    ws = workspace(sz.value)
    info = torch.empty(1, dtype=torch.int32, device=device())
    mm, nn = max(m, n), min(m, n)
    _call("tnc_qr", code(M.dtype), m, n, _p(M), n, _p(Q), _p(R), _p(ws), sz.value, _p(info), _stream(),
          flops=(2.0 * mm * nn * nn - 2.0 / 3.0 * nn ** 3) * (4 if is_complex(M.dtype) else 1))
    if check:
        st = int(info.item())
        if st != L.OK:
            raise L.NativeError("tnc_qr", st)
    return Q, R


def qr_r(M, adjoint=False, check=True):
    """R factor of the QR of M (m x n; R is min(m, n) x n) or, with
    ``adjoint``, of M^H (R is min(m, n) x m); Q is not formed."""
    M = M.contiguous()
    m, n = M.shape
    k = min(m, n)
    R = empty((k, m if adjoint else n), M.dtype)
    if k == 0:
        return R
    sz = C.c_size_t()
    _call("tnc_qr_r_workspace_size", code(M.dtype), m, n, int(bool(adjoint)), C.byref(sz))
    ws = workspace(sz.value)
    info = torch.empty(1, dtype=torch.int32, device=device())
    mm, nn = max(m, n), min(m, n)
    _call("tnc_qr_r", code(M.dtype), m, n, _p(M), int(bool(adjoint)), _p(R), _p(ws), sz.value, _p(info),
          _stream(), flops=(2.0 * mm * nn * nn - 2.0 / 3.0 * nn ** 3) * (4 if is_complex(M.dtype) else 1))
    if check:
        st = int(info.item())
        if st != L.OK:
            raise L.NativeError("tnc_qr_r", st)
    return R


def truncation_rank(S, chi, threshold, relative, with_smax=False, kdev_out=None):
    """(k, discarded weight[, s_max]) for descending singular values S, read
    back with one synchronising copy.  ``kdev_out`` (list) receives the device
    int64 holding k."""
    buf = torch.empty(3, dtype=torch.float64, device=device())
    kbuf = buf[0:1].view(torch.int64)
    _call("tnc_truncation_rank", code(S.dtype), S.numel(), _p(S), int(chi or 0), float(threshold),
          int(bool(relative)), _p(kbuf), C.c_void_p(buf.data_ptr() + 8), _stream())
    if with_smax and S.numel():
        _call("tnc_cast", code(S.dtype), L.F64, 1, _p(S), C.c_void_p(buf.data_ptr() + 16), _stream())
    if kdev_out is not None:
        kdev_out.append(kbuf)
    h = buf.cpu()
    k, disc = int(h[0:1].view(torch.int64).item()), float(h[1].item())
    if with_smax:
        return k, disc, (float(h[2].item()) if S.numel() else 0.0)
    return k, disc


_TUNE = {}            # (dtype, m, n) -> half-block height chosen by the autotuner
_TUNE_LOCK = threading.Lock()
TUNE_CANDIDATES = (L.ROWS_GRAM, 4, 8)


def _svd_rows_call(M, W, S, order, info, h, max_sweeps, tol):
    m, n = M.shape
    sz = C.c_size_t()
    _call("tnc_svd_rows_workspace_size", code(M.dtype), m, n, C.byref(sz))
    ws = workspace(sz.value)
    mm, nn = max(m, n), min(m, n)
    _call("tnc_svd_rows", code(M.dtype), m, n, _p(M), _p(W), _p(S), _p(order), int(max_sweeps), float(tol),
          int(h), _p(ws), sz.value, _p(info), _stream(),
          flops=(6.0 * mm * nn * nn + 20.0 * nn ** 3) * (4 if is_complex(M.dtype) else 1))


def tune_svd_rows(M, max_sweeps=0, tol=0.0):
    """Autotuner: time each half-block height once on this shape (device
    synchronised, CUDA events) and remember the fastest."""
    m, n = M.shape
    key = (M.dtype, m, n)
    with _TUNE_LOCK:
        if key in _TUNE:
            return _TUNE[key]
        nr, Lr = min(m, n), max(m, n)
        W = empty((nr, Lr), M.dtype)
        S = empty((nr,), real_dtype(M.dtype))
        order = torch.empty(nr, dtype=torch.int64, device=device())
        info = torch.empty(4, dtype=torch.int32, device=device())
        best, best_ms = 8, None
        global PROFILE
        saved, PROFILE = PROFILE, None
        try:
            for h in TUNE_CANDIDATES:
                torch.cuda.synchronize()
                s = torch.cuda.Event(enable_timing=True)
                e = torch.cuda.Event(enable_timing=True)
                s.record()
                _svd_rows_call(M, W, S, order, info, h, max_sweeps, tol)
                e.record()
                torch.cuda.synchronize()
                ms = s.elapsed_time(e)
                if best_ms is None or ms < best_ms:
                    best, best_ms = h, ms
        finally:
            PROFILE = saved
        _TUNE[key] = best
        return best


def svd_rows(M, max_sweeps=0, tol=0.0, block_rows=None):
    """Jacobi stage of the sweep SVD (``tnc_svd_rows``): returns (W, S,
    order, info) with W = orthogonalised rows of M (wide) or M^H (tall).
    ``block_rows`` None = the committed tuning table's choice for this
    shape's bucket (``tuning.lookup``), else the run-time autotuner's."""
    M = M.contiguous()
    m, n = M.shape
    nr, Lr = min(m, n), max(m, n)
    if block_rows is None:
        from . import tuning
        block_rows = (tuning.lookup(str(M.dtype).replace("torch.", ""), min(m, n), max(m, n))
                      or _TUNE.get((M.dtype, m, n)) or tune_svd_rows(M, max_sweeps, tol))
    W = empty((nr, Lr), M.dtype)
    S = empty((nr,), real_dtype(M.dtype))
    order = torch.empty(nr, dtype=torch.int64, device=device())
    info = torch.empty(4, dtype=torch.int32, device=device())
    _svd_rows_call(M, W, S, order, info, block_rows, max_sweeps, tol)
    return W, S, order, info


def svd_rows_stage(M, max_sweeps, tol, stop_tol, block_rows=0):
    """``svd_rows`` as the first stage of a finished core
    (``tnc_svd_rows_stage``): also stops after the first sweep without a
    rotation above ``stop_tol`` (info[3] = 1)."""
    M = M.contiguous()
    m, n = M.shape
    nr, Lr = min(m, n), max(m, n)
    W = empty((nr, Lr), M.dtype)
    S = empty((nr,), real_dtype(M.dtype))
    order = torch.empty(nr, dtype=torch.int64, device=device())
    info = torch.empty(4, dtype=torch.int32, device=device())
    sz = C.c_size_t()
    _call("tnc_svd_rows_workspace_size", code(M.dtype), m, n, C.byref(sz))
    ws = workspace(sz.value)
    _call("tnc_svd_rows_stage", code(M.dtype), m, n, _p(M), _p(W), _p(S), _p(order), int(max_sweeps), float(tol),
          float(stop_tol), int(block_rows), _p(ws), sz.value, _p(info), _stream())
    return W, S, order, info


def sort_rows(M):
    """(M', order, rank): M's rows in decreasing-norm order (``tnc_sort_rows``;
    M'[i] = M[order[i]], M[j] = M'[rank[j]])."""
    M = M.contiguous()
    m, L = M.shape
    out = empty((m, L), M.dtype)
    order = torch.empty(m, dtype=torch.int64, device=device())
    rank = torch.empty(m, dtype=torch.int64, device=device())
    norms2 = torch.empty(m, dtype=torch.float64, device=device())
    _call("tnc_sort_rows", code(M.dtype), m, L, _p(M), _p(out), _p(order), _p(rank), _p(norms2), _stream())
    return out, order, rank


def permute_rows(X, idx):
    """dst[i] = X[idx[i]] (``tnc_permute_rows``)."""
    X = X.contiguous()
    n = int(idx.shape[0])
    out = empty((n, X.shape[1]), X.dtype)
    _call("tnc_permute_rows", code(X.dtype), n, X.shape[1], _p(X), _p(idx), _p(out), _stream())
    return out


def svd_rows_df(M, max_sweeps=0, tol=0.0, block_rows=0, nkeep=None):
    """Double-float Jacobi of the rows of a wide single-precision M
    (``tnc_svd_rows_df``): returns (W, S, order, info) as ``svd_rows`` of M
    widened to FP64 (W complex128 / float64, S float64); ``nkeep``: only the
    first nkeep rows need be orthogonal to every row (None: all)."""
    M = M.contiguous()
    m, n = M.shape
    wide = torch.complex128 if is_complex(M.dtype) else torch.float64
    W = empty((m, n), wide)
    S = empty((m,), torch.float64)
    order = torch.empty(m, dtype=torch.int64, device=device())
    info = torch.empty(4, dtype=torch.int32, device=device())
    sz = C.c_size_t()
    _call("tnc_svd_rows_workspace_size", code(wide), m, n, C.byref(sz))
    ws = workspace(sz.value)
    _call("tnc_svd_rows_df", code(M.dtype), m, n, _p(M), _p(W), _p(S), _p(order), int(max_sweeps), float(tol),
          int(block_rows), m if nkeep is None else int(nkeep), _p(ws), sz.value, _p(info), _stream())
    return W, S, order, info


def fill_gaussian(shape, dtype, seed):
    out = empty(shape, dtype)
    if out.numel():
        _call("tnc_fill_gaussian", code(dtype), out.numel(), int(seed) & ((1 << 63) - 1), _p(out), _stream())
    return out


def dense_forward(W, b, x, nin, nout, act):
    out = empty((x.shape[0], nout), torch.float32)
    _call("tnc_dense_forward", _p(W), _p(b), _p(x), _p(out), x.shape[0], nin, nout, int(act), _stream())
    return out


def dense_backward(W, x, act_in, g, dW, db, gin, nin, nout, relu_mask):
    _call("tnc_dense_backward", _p(W), _p(x), _p(act_in) if act_in is not None else C.c_void_p(0), _p(g),
          _p(dW), _p(db), _p(gin) if gin is not None else C.c_void_p(0), g.shape[0], nin, nout,
          int(relu_mask), _stream())


def mse_sigmoid_grad(y, t):
    g = empty((y.shape[0],), torch.float32)
    _call("tnc_mse_sigmoid_grad", _p(y), _p(t.contiguous()), _p(g), y.shape[0], _stream())
    return g


def adam_step(p, g, m, v, lr, b1, b2, eps, step):
    _call("tnc_adam_step", _p(p), _p(g), _p(m), _p(v), p.numel(), float(lr), float(b1), float(b2), float(eps),
          int(step), _stream())


def gather_rows(W, order, kdev, kmax, S=None, mode=0):
    """Rows order[:k] of W (mode 0: k x L) or conj(W[order[:k]])^T / S (mode 1: L x k)."""
    Lr = W.shape[1]
    out = empty((kmax, Lr) if mode == 0 else (Lr, kmax), W.dtype)
    _call("tnc_gather_rows", code(W.dtype), _p(W), Lr, _p(order), _p(kdev), int(kmax),
          _p(S) if S is not None else C.c_void_p(0), int(mode), _p(out), _stream())
    return out


def prod(shape):
    return int(math.prod(int(s) for s in shape))
