"""Sweep engine: MPO-MPS apply + SVD compression on device-resident site
arrays, batched over independent instances.

This is the fast path behind the drop-in API.  It computes exactly what
``contract_mps_mpo`` followed by ``MatrixProductState.svd_compress``
(tncontract/onedim/onedim_core.py:1691-1708, 463-484) compute -- a QR left
sweep, normalisation, a truncating SVD right sweep with the reference's rank
rule (s/s_max > threshold, then at most chi, onedim_core.py:332-339) and the
norm restored -- but on sites kept in one fixed layout (phys, left, right)
so that no label bookkeeping or relayout runs per site, and with a precision
option:

* ``precision="fp64"``: complex128 / float64 storage and arithmetic;
* ``precision="fp32"``: complex64 / float32 storage and arithmetic (the FP32
  pipe of GB300 is 64x its FP64 pipe).  Fidelity error against the FP64
  result is reported by the benchmark and checked by the tests.

The truncating SVD of each site factors M^H = Q R (R only, ``tnc_qr_r``),
runs the block one-sided Jacobi of ``tnc_svd_rows`` on the rows of R
(rotations not accumulated; the rotated rows are S U^H of M) and forms
S V^H = U^H M with one GEMM.  Directions at the storage type's rounding-noise
floor are never kept (``noise_rank``).  ``apply_compress_batch`` runs several instances at once, one
CUDA stream and one host thread each (the native calls release the GIL), so
the per-site latency chains of different instances overlap on the GPU.
"""
from __future__ import annotations

import math
import threading
import time

import numpy as np
import torch

from . import _lib as L
from . import _ops

_DT = {"fp32": (torch.complex64, torch.float32), "fp64": (torch.complex128, torch.float64),
       "mixed": (torch.complex64, torch.float32)}
# The finish of the "mixed" precision's bond cores: "df" runs it in
# double-float arithmetic on the FP32 pipe (tnc_svd_rows_df), "fp64" in FP64.
MIXED_CORE = "df"
# precision -> how the native sweep factors each bond core
CORE = {"fp32": L.CORE_STORAGE, "fp64": L.CORE_STORAGE, "mixed": L.CORE_DF}


def mixed_core(precision):
    """The ``core`` argument of a precision: MIXED_CORE for "mixed", else None."""
    return MIXED_CORE if precision == "mixed" else None


def compute_dtype(precision, is_complex):
    """Storage dtype of a precision: "fp64" complex128 / float64; "fp32" and
    "mixed" complex64 / float32 ("mixed" finishes every bond core's Jacobi
    to FP64-level orthogonality, in double-float arithmetic, and decides the
    truncation on those singular values, see ``apply_compress_native``)."""
    return _DT[precision][0 if is_complex else 1]


def to_sites(arrays, dtype):
    """Host or device arrays (phys, left, right) -> contiguous device tensors of ``dtype``."""
    return [_ops.cast(_ops.to_device(a), dtype) for a in arrays]


def balance(arrays):
    """Rescale every site to unit Frobenius norm (in the arrays' own
    precision) and return (arrays, log_norm) with
    state = exp(log_norm) * product of the rescaled sites.  A normalised
    random MPS keeps a factor ~1e-86 (N=64, chi=256) in one site, below the
    FP32 range; balanced sites keep every entry O(1)."""
    out, log_norm = [], 0.0
    for a in arrays:
        if isinstance(a, torch.Tensor):
            n = float(torch.linalg.vector_norm(a.reshape(-1).to(torch.complex128)).item()) if a.device.type == "cpu" \
                else _ops.nrm2(a)
            out.append(a / n if n > 0 else a)
        else:
            n = float(np.linalg.norm(a))
            out.append(a / n if n > 0 else a)
        log_norm += float(np.log(n)) if n > 0 else 0.0
    return out, log_norm


class SweepStats:
    def __init__(self):
        self.bonds = []
        self.discarded = []      # per right-sweep bond, sum of discarded s^2 (normalised state)
        self.jacobi_sweeps = []
        self.norm = 1.0
        self.log_norm = 0.0      # natural log of the output state's norm factor


def apply_mpo(sites, mpo):
    """contract_mps_mpo in (phys, left, right) layout: fused bond a*D + b."""
    out = []
    for A, W in zip(sites, mpo):
        out.append(_ops.mps_mpo_site(A, _ops.cast(W, A.dtype) if W.dtype != A.dtype else W, layout=1))
    return out


def qr_left_sweep(P):
    """QR branch of left_canonise (onedim_core.py:267-294), in place on P.
    R is divided by its norm before it is absorbed (the gauge freedom makes
    this exact); returns log of the state norm (sum of the removed log-norms
    plus the last site's)."""
    N = len(P)
    log_norm = 0.0
    for i in range(N - 1):
        d, l, r = P[i].shape
        Q, R = _ops.qr(P[i].reshape(d * l, r))
        k = Q.shape[1]
        P[i] = Q.reshape(d, l, k)
        rn = _ops.nrm2(R)
        if rn > 0:
            log_norm += float(np.log(rn))
        d2, l2, r2 = P[i + 1].shape
        nxt = _ops.empty((d2, k, r2), P[i].dtype)
        _ops.gemm(L.OP_N, L.OP_N, k, r2, r, R, r, P[i + 1], r2, nxt, r2,
                  alpha=(1.0 / rn if rn > 0 else 1.0), batch=d2, sA=0, sB=r * r2, sC=k * r2)
        P[i + 1] = nxt
    last = _ops.nrm2(P[-1])
    if last == 0.0:
        raise ValueError("zero state in the QR sweep")
    P[-1] = _ops.scale(P[-1], 1.0 / last)
    return log_norm + float(np.log(last))


def _rows_limit(dtype):
    # register-resident rows of the Jacobi: 1024 entries of up to 8 bytes, 512 of complex128
    return 512 if dtype == torch.complex128 else 1024


def _check_info(info):
    st = int(info[0].item())
    if st != L.OK:
        if st == L.ERR_NONFINITE:
            raise ValueError("array must not contain infs or NaNs")
        raise _ops.LinAlgError("SVD did not converge (status %d)" % st)


# Core finish (the "mixed" precision of single-precision sites): the
# tolerances of the storage-precision Jacobi stage and of the finishing
# (double-float or FP64) stage, as in the native sweep (tnc_sweep.cu)
CORE_FP32_TOL, CORE_FP32_SWEEPS, CORE_FP64_TOL = 3e-6, 14, 1e-7
# the FP32 stage also stops after a sweep whose rotations were all below this
CORE_STOP_TOL = 1e-3
_WIDE = {torch.float32: torch.float64, torch.complex64: torch.complex128}


def _factor_full(M, core=None):
    """Full SVD of M (m x n) -> (S device, factors(k) -> (U_k, SV_k)).

    Columns up to the register limit (m rows) use the QR-preconditioned,
    non-accumulating block Jacobi: M^H = Q R, the rows of R (min(m, n) x m)
    are orthogonalised, which leaves them equal to S U^H of M (M = R^H Q^H),
    so U is the normalised rows and S V^H = U^H M is one GEMM.  U is then
    orthonormal to the Jacobi tolerance for every kept direction, however
    small its singular value (recovering U = M V / S instead divides the
    Jacobi's residual non-orthogonality by s_j and fails for spectra that
    fall below the storage precision), and the triangular start needs fewer
    sweeps on graded matrices (Drmac & Veselic 2008).  Longer columns run
    the accumulating SVD on the same R (its VH rows are then U^H of M)."""
    m, n = M.shape
    wide = _WIDE.get(M.dtype)
    rank = None
    if m <= _rows_limit(M.dtype):
        # rows in decreasing-norm order (a static column pivoting of the QR of
        # M^H: fewer Jacobi sweeps); U's rows go back in M's order at the end
        M, _order, rank = _ops.sort_rows(M)
    R = _ops.qr_r(M, adjoint=True)                                         # min(m, n) x m

    def unsort(U):
        return U if rank is None else _ops.permute_rows(U, rank)
    if core in ("fp64", "df") and wide is not None and m <= _rows_limit(wide):
        # FP32 Jacobi to near its rounding floor (a stall is handed over), then
        # the double-float (or FP64) Jacobi finishes the rows; S, the rank
        # decision and U come from the finished rows, U is stored back in the
        # sites' precision
        W32, _s, _o, info = _ops.svd_rows_stage(R, CORE_FP32_SWEEPS, CORE_FP32_TOL, CORE_STOP_TOL)
        if int(info[0].item()) not in (L.OK, L.ERR_NOT_CONVERGED):
            _check_info(info)
        if core == "df":
            kall = torch.tensor([W32.shape[0]], dtype=torch.int64, device=W32.device)
            rows = _ops.gather_rows(W32, _o, kall, W32.shape[0])                # FP32 norm order
            W, S, order, info = _ops.svd_rows_df(rows, tol=CORE_FP64_TOL)
        else:
            W, S, order, info = _ops.svd_rows(_ops.cast(W32, wide), tol=CORE_FP64_TOL)
        _check_info(info)

        def factors(k, kdev):
            U = _ops.cast(_ops.gather_rows(W, order, kdev, k, S=S, mode=1), M.dtype)   # m x k
            SV = _ops.empty((k, n), M.dtype)
            _ops.gemm(L.OP_C, L.OP_N, k, n, m, U, k, M, n, SV, n)     # U^H M
            return unsort(U), SV
        return S, factors
    if m <= _rows_limit(M.dtype):
        W, S, order, info = _ops.svd_rows(R)                               # W rows = S U^H
        _check_info(info)

        def factors(k, kdev):
            U = _ops.gather_rows(W, order, kdev, k, S=S, mode=1)          # m x k
            SV = _ops.empty((k, n), M.dtype)
            _ops.gemm(L.OP_C, L.OP_N, k, n, m, U, k, M, n, SV, n)         # U^H M
            return unsort(U), SV
        return S, factors
    _u, S, VH = _ops.svd(R)                                                # VH rows = U^H of M

    def factors(k, kdev):
        U = _ops.permute(VH[:k].contiguous(), (1, 0), conj=True)          # m x k
        SV = _ops.empty((k, n), M.dtype)
        _ops.gemm(L.OP_C, L.OP_N, k, n, m, U, k, M, n, SV, n)             # U^H M
        return U, SV
    return S, factors


def _factor_sketch(M, l, power_iters, seed, core=None):
    """Randomized range finder (Halko, Martinsson & Tropp 2011, alg. 4.4):
    Q = orth((M M^H)^q M Omega) with Omega n x l Gaussian, re-orthonormalised
    after every product; then the SVD of B = Q^H M (l x n).  Returns
    (S, factors, captured weight fraction residual) with factors mapping to
    (U = Q U_B, S V^H)."""
    m, n = M.shape
    dt = M.dtype
    Om = _ops.fill_gaussian((n, l), dt, seed)
    Y = _ops.empty((m, l), dt)
    _ops.gemm(L.OP_N, L.OP_N, m, l, n, M, n, Om, l, Y, l)
    for _ in range(power_iters):
        Q, _r = _ops.qr(Y)
        Z = _ops.empty((n, l), dt)
        _ops.gemm(L.OP_C, L.OP_N, n, l, m, M, n, Q, l, Z, l)     # M^H Q
        Q2, _r = _ops.qr(Z)
        _ops.gemm(L.OP_N, L.OP_N, m, l, n, M, n, Q2, l, Y, l)    # M Q2
    Q, _r = _ops.qr(Y)                                            # m x l
    B = _ops.empty((l, n), dt)
    _ops.gemm(L.OP_C, L.OP_N, l, n, m, Q, l, M, n, B, n)          # Q^H M
    # residual weight |M - Q Q^H M|_F^2, formed explicitly: the difference of
    # |M|^2 and |B|^2 would sit below FP32 resolution at small tolerances
    E = M.clone()
    _ops.gemm(L.OP_N, L.OP_N, m, n, l, Q, l, B, n, E, n, alpha=-1.0, beta=1.0)
    residual = _ops.nrm2(E) ** 2
    S, fB = _factor_full(B, core)

    def factors(k, kdev):
        UB, SV = fB(k, kdev)                                       # l x k, k x n
        U = _ops.empty((m, k), dt)
        _ops.gemm(L.OP_N, L.OP_N, m, k, l, Q, l, UB, k, U, k)
        return U, SV
    return S, factors, residual


def reference_rank(s, chi, threshold):
    """The reference's truncation rule on descending singular values s: keep
    s / s_max > threshold, then at most chi (onedim_core.py:332-339)."""
    if s.size == 0 or s[0] <= 0:
        return 0
    k = int(np.count_nonzero(s > threshold * s[0]))
    return min(k, chi) if chi else k


_EPS = {torch.float32: 2.0 ** -23, torch.complex64: 2.0 ** -23,
        torch.float64: 2.0 ** -52, torch.complex128: 2.0 ** -52}


def noise_rank(s, dtype):
    """Number of singular values above the rounding-noise floor of the
    storage type, 4 eps |M|_F.  The Jacobi stages leave rows at or below
    eps |M|_F out of their rotations (their directions are rounding noise),
    so directions there are never kept, whatever the rank rule asks (in FP64
    the floor sits below the reference's 1e-14 threshold for all but very
    flat spectra)."""
    floor = 4.0 * _EPS[dtype] * float(np.sqrt(np.sum(s ** 2)))
    return max(1, int(np.count_nonzero(s > floor))) if s.size and s[0] > 0 else 0


class RankStats:
    def __init__(self):
        self.features = []   # per bond, the predictor's input
        self.targets = []    # per bond, k / min(m, n) chosen by the rule (full SVD only)
        self.sketched = 0
        self.fallbacks = 0
        self.full = 0
        self.declined = 0    # bonds whose neighbour was cut by the bond cap: no sketch tried
        self.rows_factored = 0   # sum over bonds of (rows of the Jacobi problem)^2 * row length


def svd_right_sweep(P, chi, threshold, stats=None, dw_tol=None, rank_model=None, oversample=16,
                    power_iters=2, rank_stats=None, seed=1234, core=None):
    """Truncating SVD branch of right_canonise (reverse, left_canonise,
    reverse; onedim_core.py:296-378) with normalise=False, in place on P.

    Rank rule: the reference's (s/s_max > threshold, then at most chi) when
    ``dw_tol`` is None; otherwise the smallest rank whose discarded weight
    sum_{j>=k} s_j^2 is at most dw_tol * sum_j s_j^2 (capped at chi).  With a
    ``rank_model`` (and ``dw_tol``), each bond's rank is predicted from the
    neighbouring spectrum and a randomized SVD of that size + ``oversample``
    replaces the full SVD; when the sketch leaves more than dw_tol of the
    weight uncaptured the full SVD runs instead (fallback)."""
    from . import rank_model as RM
    N = len(P)
    norm_acc = 1.0
    s_prev = None
    prev_disc = None   # discarded fraction of the previous bond's spectrum
    for i in range(N - 1, 0, -1):
        d, l, r = P[i].shape
        M = _ops.permute(P[i], (0, 2, 1)).reshape(d * r, l)  # rows (phys, right), cols left
        m, n = M.shape
        kmax = min(m, n)
        used_sketch = False
        feats = None
        if dw_tol is not None and rank_stats is not None or rank_model is not None:
            feats = RM.spectrum_features((i - 1) / max(N - 2, 1), kmax, chi or kmax, dw_tol or 1e-16,
                                         s_prev if s_prev is not None else np.ones(1))
        # a sketch can only be accepted where the tolerance, not the bond cap,
        # decides the rank: the uncaptured weight must stay below dw_tol; where
        # the neighbouring bond discarded more than 10 dw_tol (its cut set by
        # chi) the full SVD runs without a sketch
        cap_bound = prev_disc is not None and dw_tol is not None and prev_disc > 10.0 * dw_tol
        if rank_model is not None and dw_tol is not None and s_prev is not None and cap_bound:
            if rank_stats is not None:
                rank_stats.declined += 1
        elif rank_model is not None and dw_tol is not None and s_prev is not None:
            frac = float(rank_model.predict(feats)[0])
            lsk = min(kmax, int(math.ceil(frac * kmax)) + oversample)
            if lsk < 0.75 * kmax:
                total = _ops.nrm2(M) ** 2
                S, factors, residual = _factor_sketch(M, lsk, power_iters, seed + i, core)
                s_host = S.cpu().numpy().astype(np.float64)
                if residual <= dw_tol * total:
                    used_sketch = True
                    # rank by the same rule, the uncaptured weight counted as discarded
                    k = RM.dw_rank(s_host, dw_tol, chi or 0, total=float((s_host ** 2).sum()) + residual)
                    k = min(k, noise_rank(s_host, M.dtype))
                    smax = float(s_host[0])
                    disc = float((s_host[k:] ** 2).sum()) + residual
                    kd = torch.tensor([k], dtype=torch.int64, device=M.device)
                    if rank_stats is not None:
                        rank_stats.sketched += 1
                        rank_stats.rows_factored += lsk * lsk * max(lsk, n)
                elif rank_stats is not None:
                    rank_stats.fallbacks += 1
        if not used_sketch:
            S, factors = _factor_full(M, core)
            s_host = S.cpu().numpy().astype(np.float64)
            if dw_tol is None:
                k = reference_rank(s_host, chi or 0, threshold)
            else:
                k = RM.dw_rank(s_host, dw_tol, chi or 0)
            k = min(k, noise_rank(s_host, M.dtype))
            smax = float(s_host[0])
            disc = float((s_host[k:] ** 2).sum())
            kd = torch.tensor([k], dtype=torch.int64, device=M.device)
            if rank_stats is not None:
                rank_stats.full += 1
                rank_stats.rows_factored += kmax * kmax * max(m, n)
                if feats is not None and s_prev is not None:
                    rank_stats.features.append(feats)
                    rank_stats.targets.append(k / kmax)
        if smax == 0.0:
            raise ValueError("zero state in the SVD sweep")
        if rank_stats is not None or rank_model is not None:
            s_prev = s_host
            tot2 = float(np.sum(s_host ** 2))
            prev_disc = disc / tot2 if tot2 > 0 else 0.0
        U, SV = factors(k, kd)
        P[i] = _ops.permute(U.reshape(d, r, k), (0, 2, 1))             # (phys, k, right)
        dp, lp, rp = P[i - 1].shape                                      # rp == l
        nxt = _ops.empty((dp, lp, k), M.dtype)
        _ops.gemm(L.OP_N, L.OP_T, dp * lp, k, rp, P[i - 1], rp, SV, n, nxt, k, alpha=1.0 / smax)
        P[i - 1] = nxt
        norm_acc *= smax
        if stats is not None:
            stats.bonds.append(k)
            stats.discarded.append(disc / (smax * smax))
    P[0] = _ops.scale(P[0], norm_acc)
    return norm_acc


_FOLD_LIMIT = {torch.complex64: 60.0, torch.float32: 60.0}  # |log| folded into FP32 sites


def apply_compress(sites, mpo, chi, threshold=1e-15, stats=None, log_norm_in=0.0, dw_tol=None,
                   rank_model=None, rank_stats=None, oversample=16, power_iters=2, core=None):
    """One unit: contract_mps_mpo then svd_compress(chi, threshold,
    normalise=False).  ``sites`` / ``mpo`` are device tensors in (phys,
    left, right) / (physout, physin, left, right) layout, all of the compute
    dtype; the input state is exp(log_norm_in) times the product of
    ``sites``.  Returns the compressed sites (phys, left, right) carrying the
    state's norm in the first site, as svd_compress does; when that factor is
    outside the storage range (FP32: |log| > 60) it is left out of the sites
    and only reported in ``stats.log_norm``.  ``dw_tol``, ``rank_model``,
    ``rank_stats``, ``oversample``, ``power_iters``: see svd_right_sweep.
    ``core="fp64"`` (single-precision sites): every bond core's Jacobi is
    finished in FP64 and the spectrum, the rank decision and U come from the
    FP64 rows (the "mixed" precision, as ``apply_compress_native`` does)."""
    P = apply_mpo(sites, mpo)
    log_norm = qr_left_sweep(P) + log_norm_in
    norm_acc = svd_right_sweep(P, chi, threshold, stats, dw_tol=dw_tol, rank_model=rank_model,
                               oversample=oversample, power_iters=power_iters, rank_stats=rank_stats, core=core)
    total = log_norm + (float(np.log(norm_acc)) if norm_acc > 0 else 0.0)
    # svd_right_sweep already folded norm_acc into P[0]
    lim = _FOLD_LIMIT.get(P[0].dtype, 600.0)
    if abs(log_norm) <= lim:
        P[0] = _ops.scale(P[0], float(np.exp(log_norm)))
        folded = True
    else:
        folded = False
    if stats is not None:
        stats.norm = float(np.exp(total)) if abs(total) < 700 else float("inf")
        stats.log_norm = total
        stats.norm_folded = folded
    return P


def apply_compress_native(sites, mpo, chi, threshold=1e-15, log_norm_in=0.0, stats=None, block_rows=0,
                          profile=None, core=None, core_tol=0.0):
    """``apply_compress`` as one native call (``tnc_sweep_apply_compress``):
    the same algorithm, rank rule and norm handling, with the whole sweep run
    by the library so the calling thread stays out of the interpreter (and
    off its lock) until the sweep ends.  Sites and MPO as for
    ``apply_compress``; returns the compressed sites (compact copies; the
    sweep's workspace is released), ``stats.log_norm`` / ``stats.bonds`` /
    ``stats.norm_folded`` / ``stats.discarded`` (per bond, the discarded
    fraction of the squared singular values, bonds left to right) when
    ``stats`` is given.  ``profile``: a ctypes array of 12 doubles
    accumulating per-op CUDA-event time, calls and algorithmic flops (QR,
    R-only QR, Jacobi, its finish), or None.  ``core``: "df" (double-float
    arithmetic on the FP32 pipe) or "fp64" finishes the Jacobi of every bond
    core to FP64-level orthogonality and takes the spectrum, the
    truncation decision and U from it (single-precision sites only; the
    "mixed" precision), None / "storage" factors in the storage precision;
    ``core_tol``: the finishing Jacobi's tolerance (0: its default)."""
    import ctypes as C
    N = len(sites)
    dt = sites[0].dtype
    sites = [s.contiguous() for s in sites]
    mpo = [_ops.cast(w, dt).contiguous() for w in mpo]
    d = int(sites[0].shape[0])
    bonds = [int(sites[0].shape[1])] + [int(s.shape[2]) for s in sites]
    mbonds = [int(mpo[0].shape[2])] + [int(w.shape[3]) for w in mpo]
    b_arr = (C.c_int64 * (N + 1))(*bonds)
    m_arr = (C.c_int64 * (N + 1))(*mbonds)
    code = _ops.code(dt)
    core_code = {None: L.CORE_STORAGE, "storage": L.CORE_STORAGE, "fp64": L.CORE_FP64, "df": L.CORE_DF}[core]
    sz = C.c_size_t()
    L.check("tnc_sweep_workspace_size",
            L.lib().tnc_sweep_workspace_size(code, N, d, b_arr, m_arr, core_code, C.byref(sz)))
    ws = torch.empty(int(sz.value), dtype=torch.uint8, device=sites[0].device)
    s_arr = (C.c_void_p * N)(*[s.data_ptr() for s in sites])
    w_arr = (C.c_void_p * N)(*[w.data_ptr() for w in mpo])
    out_b = (C.c_int64 * (N + 1))()
    out_o = (C.c_int64 * N)()
    out_d = (C.c_double * (N - 1))()
    lnorm = C.c_double(float(log_norm_in))
    folded = C.c_int(0)
    st = L.lib().tnc_sweep_apply_compress(code, N, d, s_arr, b_arr, w_arr, m_arr, int(chi or 0), float(threshold),
                                          int(block_rows), core_code, float(core_tol), C.c_void_p(ws.data_ptr()),
                                          sz.value, out_b, out_o, out_d, C.byref(lnorm), C.byref(folded), profile,
                                          C.c_void_p(torch.cuda.current_stream().cuda_stream))
    if st == L.ERR_ARG:
        raise ValueError("zero state in the sweep (or bad arguments)")
    if st == L.ERR_NONFINITE:
        raise ValueError("array must not contain infs or NaNs")
    if st == L.ERR_NOT_CONVERGED:
        raise _ops.LinAlgError("SVD did not converge")
    L.check("tnc_sweep_apply_compress", st)
    es = torch.empty(0, dtype=dt).element_size()
    out = []
    for i in range(N):
        n = d * out_b[i] * out_b[i + 1]
        view = ws[out_o[i]: out_o[i] + n * es].view(dt).view(d, out_b[i], out_b[i + 1])
        out.append(view.clone())
    if stats is not None:
        stats.bonds = list(out_b)[1:N]
        stats.discarded = list(out_d)
        stats.log_norm = lnorm.value
        stats.norm_folded = bool(folded.value)
        stats.norm = float(np.exp(lnorm.value)) if abs(lnorm.value) < 700 else float("inf")
    return out


def apply_compress_host(sites, mpo, chi, precision="mixed", threshold=1e-15, stats=None):
    """The sweep for a caller that holds the state in host memory, as
    tncontract's users do: ``sites`` (phys, left, right) and ``mpo``
    (physout, physin, left, right) are host arrays (NumPy or CPU torch
    tensors; pinned tensors copy asynchronously) of any float / complex
    dtype.  On the current stream the inputs are copied to the device,
    balanced (``balance``) and cast to the storage dtype of ``precision``,
    the sweep runs as one native call (``apply_compress_native``; "mixed"
    finishes every bond core, ``MIXED_CORE``), and the result comes back as host
    arrays of the input's precision class (complex128 / float64 for double
    input) with the state's norm in the first site, as
    ``MatrixProductState.svd_compress`` leaves it (onedim_core.py:463-484)."""
    def dev(a):
        t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))
        return t.to(device=_ops.device(), non_blocking=True)
    d_sites = [dev(a) for a in sites]
    d_mpo = [dev(w) for w in mpo]
    cplx = any(t.is_complex() for t in d_sites + d_mpo)
    dt = compute_dtype(precision, cplx)
    out_dt = torch.complex128 if cplx else torch.float64
    bal, log_norm = balance(d_sites)
    st = stats if stats is not None else SweepStats()
    out = apply_compress_native([_ops.cast(a, dt) for a in bal], [_ops.cast(w, dt) for w in d_mpo], chi,
                                threshold=threshold, log_norm_in=log_norm, stats=st,
                                core=mixed_core(precision))
    res = [_ops.cast(o, out_dt) for o in out]
    if not st.norm_folded and abs(st.log_norm) < 700:
        # the factor did not fit the storage type; it fits the output's
        res[0] = _ops.scale(res[0], float(np.exp(st.log_norm - _log_norm_of(res))))
    return [r.cpu().numpy() for r in res]


def _log_norm_of(sites):
    """log of the norm of the state held by ``sites`` (device)."""
    v = inner_product(sites, sites).real
    return 0.5 * float(np.log(v)) if v > 0 else 0.0


def compress(sites, chi, threshold=1e-15, stats=None, log_norm_in=0.0, fold_norm=True):
    """``MatrixProductState.svd_compress(chi, threshold)`` on (phys, left,
    right) device sites (no MPO).  Returns (sites, log_norm): the state is
    exp(log_norm) times the returned sites; with ``fold_norm`` the factor is
    folded into the first site when it is representable (log_norm is then 0)."""
    P = [s for s in sites]
    log_norm = qr_left_sweep(P) + log_norm_in
    norm_acc = svd_right_sweep(P, chi, threshold, stats)
    if norm_acc > 0:
        log_norm += float(np.log(norm_acc))
        P[0] = _ops.scale(P[0], 1.0 / norm_acc)   # keep the returned sites normalised
    if fold_norm and abs(log_norm) <= _FOLD_LIMIT.get(P[0].dtype, 600.0):
        P[0] = _ops.scale(P[0], float(np.exp(log_norm)))
        log_norm = 0.0
    return P, log_norm


def run_batch(jobs, streams=None):
    """Run callables concurrently, each on its own CUDA stream and host
    thread (the native calls release the GIL); returns their results."""
    B = len(jobs)
    if streams is None:
        streams = [torch.cuda.Stream() for _ in range(B)]
    out = [None] * B
    errs = [None] * B
    dev = torch.cuda.current_device()
    cur = torch.cuda.current_stream()

    def run(b):
        try:
            torch.cuda.set_device(dev)
            streams[b % len(streams)].wait_stream(cur)
            with torch.cuda.stream(streams[b % len(streams)]):
                out[b] = jobs[b]()
        except BaseException as e:
            errs[b] = e

    threads = [threading.Thread(target=run, args=(b,)) for b in range(B)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for e in errs:
        if e is not None:
            raise e
    for s in streams:
        cur.wait_stream(s)
    return out


def run_queue(jobs, workers, streams=None, stagger=0.0):
    """Continuous batching: ``workers`` host threads, each on its own CUDA
    stream, take callables from one shared queue until it is empty, so an
    instance that finishes early picks up the next one instead of waiting
    for the slowest of a fixed batch (instances in different phases -- QR
    sweep, SVD sweep -- then share the GPU).  ``stagger`` (seconds): worker
    w takes its first job w * stagger late, so identical instances do not
    run their phases in lockstep.  Returns the results in job order."""
    n = len(jobs)
    workers = max(1, min(workers, n)) if n else 0
    if streams is None:
        streams = [torch.cuda.Stream() for _ in range(workers)]
    out = [None] * n
    errs = []
    nxt = [0]
    lock = threading.Lock()
    dev = torch.cuda.current_device()
    cur = torch.cuda.current_stream()

    def work(w):
        try:
            torch.cuda.set_device(dev)
            st = streams[w % len(streams)]
            st.wait_stream(cur)
            if stagger > 0 and w:
                time.sleep(w * stagger)
            with torch.cuda.stream(st):
                while True:
                    with lock:
                        if errs or nxt[0] >= n:
                            return
                        i = nxt[0]
                        nxt[0] += 1
                    out[i] = jobs[i]()
        except BaseException as e:  # surfaced below
            with lock:
                errs.append(e)

    threads = [threading.Thread(target=work, args=(w,)) for w in range(workers)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errs:
        raise errs[0]
    for s in streams[:workers]:
        cur.wait_stream(s)
    return out


def boundary_mps_contract(layer, chi, threshold=1e-14, precision="fp32"):
    """``SquareLatticeTensorNetwork.mps_contract`` with SVD compression
    (tncontract/twodim/square_lattice.py:130-203) on the engine: ``layer``
    is a 2-D list of double-layer tensors with legs (down, left, right, up)
    (device or host arrays).  Every site is balanced to unit norm, the
    column MPS is normalised after each compression and all scale factors are
    summed as natural logarithms on the host (the reference keeps the running
    norm in np.longdouble for the same reason: the 8x8 norm network is
    ~1e115, beyond FP32).  Returns (value as a Python complex or float when
    representable else None, log10 |value|, phase)."""
    nrows, ncols = len(layer), len(layer[0])
    first = layer[0][0]
    cplx = first.is_complex() if isinstance(first, torch.Tensor) else bool(np.iscomplexobj(first))
    dt = compute_dtype(precision, cplx)
    log_total = 0.0

    def prep(t, perm):
        a = _ops.to_device(t)
        n = _ops.nrm2(a)
        a = _ops.scale(a, 1.0 / n) if n > 0 else a
        return _ops.cast(_ops.permute(a, perm).contiguous(), dt), (float(np.log(n)) if n > 0 else 0.0)

    # column 0 -> MPS (phys=right, left=up, right=down); dummy 'left' leg dropped
    mps = []
    for i in range(nrows):
        t = layer[i][0]
        a, ln = prep(t, (2, 3, 0, 1))       # (right, up, down, left[1])
        mps.append(a.reshape(a.shape[0], a.shape[1], a.shape[2]))
        log_total += ln
    mps, ln = compress(mps, chi, threshold, fold_norm=False)
    log_total += ln
    for c in range(1, ncols - 1):
        mpo = []
        for i in range(nrows):
            a, ln = prep(layer[i][c], (2, 1, 3, 0))   # (physout=right, physin=left, up, down)
            mpo.append(a)
            log_total += ln
        mps = apply_mpo(mps, mpo)
        mps, ln = compress(mps, chi, threshold, fold_norm=False)
        log_total += ln
    last = []
    for i in range(nrows):
        a, ln = prep(layer[i][ncols - 1], (1, 3, 0, 2))  # (left, up, down, right[1])
        last.append(a.reshape(a.shape[0], a.shape[1], a.shape[2]))
        log_total += ln
    v = inner_product(mps, last, conj_bra=False)
    mag = abs(v)
    if mag == 0:
        return 0.0, float("-inf"), 1.0
    log10 = (log_total + math.log(mag)) / math.log(10.0)
    phase = v / mag
    value = None
    if abs(log10) < 300:
        value = phase * 10.0 ** log10
        if not cplx:
            value = value.real
    return value, log10, phase


def apply_compress_batch(batch, mpo, chi, threshold=1e-15, streams=None, stats=None, log_norms=None):
    """``apply_compress`` for several independent instances at once: instance
    b runs on its own CUDA stream from its own host thread.  ``batch`` is a
    list of site lists (``log_norms[b]``: their log norm factors, see
    ``balance``); returns the list of results (same order)."""
    B = len(batch)
    if streams is None:
        streams = [torch.cuda.Stream() for _ in range(B)]
    out = [None] * B
    errs = [None] * B
    dev = torch.cuda.current_device()
    cur = torch.cuda.current_stream()

    def run(b):
        try:
            torch.cuda.set_device(dev)
            streams[b].wait_stream(cur)
            with torch.cuda.stream(streams[b]):
                out[b] = apply_compress(batch[b], mpo, chi, threshold,
                                        stats[b] if stats is not None else None,
                                        log_norms[b] if log_norms is not None else 0.0)
        except BaseException as e:  # surfaced below
            errs[b] = e

    threads = [threading.Thread(target=run, args=(b,)) for b in range(B)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for e in errs:
        if e is not None:
            raise e
    for s in streams:
        cur.wait_stream(s)
    return out


def _unit_site(x):
    """(x / |x|_F, log |x|_F) for a device tensor whose squared norm may leave
    the FP64 range (|x| > 1e154 or < 1e-154): it is first scaled by a power
    of two, exactly."""
    n = _ops.nrm2(x)
    shift = 0.0
    for _ in range(4):
        if n > 0 and math.isfinite(n) and 1e-150 < n < 1e150:
            break
        if not math.isfinite(n):
            step = -600
        elif n == 0:
            return x, 0.0
        else:
            step = 600 if n < 1e-150 else -600
        x = _ops.scale(x, 2.0 ** step)
        shift -= step * math.log(2.0)
        n = _ops.nrm2(x)
    if not (n > 0) or not math.isfinite(n):
        return x, shift
    return _ops.scale(x, 1.0 / n), shift + math.log(n)


def inner_product(bra, ket, conj_bra=True, log_scale=False):
    """<bra|ket> of two (phys, left, right) site lists on the device, by the
    left-to-right environment sweep of ladder_contract (onedim_core.py:1587-1607).
    Returns a Python complex; with ``log_scale`` every site and the
    environment after every site are rescaled to unit norm and (mantissa,
    natural log of the scale) is returned, for states whose overlaps leave
    the FP64 range."""
    dt = torch.promote_types(bra[0].dtype, ket[0].dtype)
    C = None
    logs = 0.0
    for a, b in zip(bra, ket):
        a = _ops.cast(a, dt)
        b = _ops.cast(b, dt)
        if conj_bra:
            a = _ops.conj(a)
        if log_scale:  # sites to unit norm too (one of them may hold the state's whole norm)
            a, la_ = _unit_site(a)
            b, lb_ = _unit_site(b)
            logs += la_ + lb_
        d, la, ra = a.shape
        _, lb, rb = b.shape
        if C is None:
            # boundary legs have dimension 1
            Cn = _ops.empty((ra, rb), dt)
            _ops.gemm(L.OP_T, L.OP_N, ra, rb, d, a.reshape(d, ra), ra, b.reshape(d, rb), rb, Cn, rb)
            C = Cn
            continue
        # T[p][la? ...]: T = C^T-contract: T_p = C (la x lb) ; step 1: X_p = a_p^T C  (ra x lb)
        X = _ops.empty((d, ra, lb), dt)
        _ops.gemm(L.OP_T, L.OP_N, ra, lb, la, a, ra, C, lb, X, lb, batch=d, sA=la * ra, sB=0, sC=ra * lb)
        # C' = sum_p X_p b_p  (ra x rb): one GEMM with K = d * lb
        Cn = _ops.empty((ra, rb), dt)
        Xp = _ops.permute(X, (1, 0, 2)).reshape(ra, d * lb)
        _ops.gemm(L.OP_N, L.OP_N, ra, rb, d * lb, Xp, d * lb, b.reshape(d * lb, rb), rb, Cn, rb)
        C = Cn
        if log_scale:
            n = _ops.nrm2(C)
            if n > 0:
                C = _ops.scale(C, 1.0 / n)
                logs += math.log(n)
    v = C.reshape(-1)[0].item()
    return (complex(v), logs) if log_scale else complex(v)


def fidelity(a, b):
    """|<a|b>|^2 / (<a|a><b|b>) on the device, the overlaps carried as
    logarithms (``inner_product(log_scale=True)``): the norms of long chains
    leave the FP64 range."""
    ab, lab = inner_product(a, b, log_scale=True)
    aa, laa = inner_product(a, a, log_scale=True)
    bb, lbb = inner_product(b, b, log_scale=True)
    if ab == 0:
        return 0.0
    return math.exp(2.0 * (math.log(abs(ab)) + lab) - (math.log(aa.real) + laa) - (math.log(bb.real) + lbb))
