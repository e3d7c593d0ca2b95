"""ctypes binding of the native C ABI (``include/tncontract_gb300.h``).

The library is built in-tree by ``tncontract_gb300._build`` and loaded from
``tncontract_gb300/_lib/``.  There is no fallback: if the library is missing
or does not load, every device operation raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import _build

# C-ABI constants (include/tncontract_gb300.h)
F32, F64, C64, C128 = 0, 1, 2, 3
OK, ERR_ARG, ERR_NOT_CONVERGED, ERR_NONFINITE, ERR_CUDA, ERR_WORKSPACE, ERR_TIMEOUT, ERR_TOO_LARGE = range(8)
OP_N, OP_T, OP_C, OP_R = 0, 1, 2, 3
CORE_STORAGE, CORE_FP64, CORE_DF = 0, 1, 2
ROWS_GRAM = 32  # block_rows code of the Gram-form Jacobi update

_vp = C.c_void_p
_i64 = C.c_int64
_int = C.c_int
_dbl = C.c_double
_pdbl = C.POINTER(C.c_double)
_pi64 = C.POINTER(C.c_int64)
_pint = C.POINTER(C.c_int)
_psz = C.POINTER(C.c_size_t)

GEMM_GROUP_MAX = 16


class GemmProblem(C.Structure):
    """tnc_gemm_problem (include/tncontract_gb300.h)."""
    _fields_ = [("opA", C.c_int), ("opB", C.c_int), ("m", C.c_int64), ("n", C.c_int64), ("k", C.c_int64),
                ("A", C.c_void_p), ("lda", C.c_int64), ("B", C.c_void_p), ("ldb", C.c_int64),
                ("C", C.c_void_p), ("ldc", C.c_int64), ("alpha", C.c_double * 2), ("beta", C.c_double * 2)]


# name -> argtypes (restype int unless given)
SIGNATURES = {
    "tnc_abi_version": [],
    "tnc_status_string": [_int],
    "tnc_kernel_launches": [],
    "tnc_set_spin_limit": [C.c_longlong],
    "tnc_wait_selftest": [_int, _vp, C.c_size_t, _vp, _vp],
    "tnc_permute": [_int, _vp, _vp, _int, _pi64, _pint, _int, _vp],
    "tnc_scale": [_int, _i64, _pdbl, _vp, _vp, _int, _vp],
    "tnc_axpby": [_int, _i64, _pdbl, _vp, _pdbl, _vp, _vp],
    "tnc_cast": [_int, _int, _i64, _vp, _vp, _vp],
    "tnc_nrm2": [_int, _i64, _vp, _vp, _vp],
    "tnc_dot": [_int, _i64, _vp, _vp, _int, _vp, _vp],
    "tnc_trace": [_int, _int, _pi64, _int, _int, _vp, _vp, _vp],
    "tnc_scale_rows": [_int, _i64, _i64, _vp, _int, _vp, _i64, _vp],
    "tnc_scale_cols": [_int, _i64, _i64, _vp, _int, _vp, _i64, _vp],
    "tnc_diag_matrix": [_int, _i64, _vp, _vp, _vp],
    "tnc_copy2d": [_int, _i64, _i64, _vp, _i64, _vp, _i64, _vp],
    "tnc_gemm": [_int, _int, _int, _i64, _i64, _i64, _pdbl, _vp, _i64, _i64, _vp, _i64,
                 _i64, _pdbl, _vp, _i64, _i64, _i64, _vp],
    "tnc_gemm_grouped": [_int, _int, C.POINTER(GemmProblem), _vp],
    "tnc_mps_mpo_site": [_int, _i64, _i64, _i64, _i64, _i64, _i64, _vp, _vp, _vp, _int, _vp],
    "tnc_qr_workspace_size": [_int, _i64, _i64, _psz],
    "tnc_qr": [_int, _i64, _i64, _vp, _i64, _vp, _vp, _vp, C.c_size_t, _vp, _vp],
    "tnc_qr_r_workspace_size": [_int, _i64, _i64, _int, _psz],
    "tnc_sweep_workspace_size": [_int, _int, _i64, _pi64, _pi64, _int, _psz],
    "tnc_sweep_apply_compress": [_int, _int, _i64, C.POINTER(_vp), _pi64, C.POINTER(_vp), _pi64, _i64, C.c_double,
                                 _int, _int, C.c_double, _vp, C.c_size_t, _pi64, _pi64, _pdbl, _pdbl, _pint, _pdbl,
                                 _vp],
    "tnc_qr_r": [_int, _i64, _i64, _vp, _int, _vp, _vp, C.c_size_t, _vp, _vp],
    "tnc_svd_workspace_size": [_int, _i64, _i64, _psz],
    "tnc_svd": [_int, _i64, _i64, _vp, _i64, _vp, _vp, _vp, _int, _dbl, _vp, C.c_size_t, _vp, _vp],
    "tnc_truncation_rank": [_int, _i64, _vp, _i64, _dbl, _int, _vp, _vp, _vp],
    "tnc_svd_noalloc": [_int, _i64, _i64, _vp, _i64, _vp, _vp, _vp, _int, _dbl, _vp, _vp],
    "tnc_svd_rows_workspace_size": [_int, _i64, _i64, _psz],
    "tnc_svd_rows": [_int, _i64, _i64, _vp, _vp, _vp, _vp, _int, _dbl, _int, _vp, C.c_size_t, _vp, _vp],
    "tnc_svd_rows_keep": [_int, _i64, _i64, _vp, _vp, _vp, _vp, _int, _dbl, _int, _i64, _vp, C.c_size_t, _vp, _vp],
    "tnc_svd_rows_stage": [_int, _i64, _i64, _vp, _vp, _vp, _vp, _int, _dbl, _dbl, _int, _vp, C.c_size_t, _vp, _vp],
    "tnc_sort_rows": [_int, _i64, _i64, _vp, _vp, _vp, _vp, _vp, _vp],
    "tnc_permute_rows": [_int, _i64, _i64, _vp, _vp, _vp, _vp],
    "tnc_svd_rows_df": [_int, _i64, _i64, _vp, _vp, _vp, _vp, _int, _dbl, _int, _i64, _vp, C.c_size_t, _vp, _vp],
    "tnc_gather_rows": [_int, _vp, _i64, _vp, _vp, _i64, _vp, _int, _vp, _vp],
    "tnc_gemm_tc_workspace_size": [_int, _i64, _i64, _i64, _i64, _psz],
    "tnc_gemm_tc": [_int, _int, _int, _i64, _i64, _i64, _pdbl, _vp, _i64, _i64, _vp, _i64, _i64, _pdbl,
                    _vp, _i64, _i64, _i64, _vp, C.c_size_t, _vp],
    "tnc_gemm_tc_error": [],
    "tnc_dense_forward": [_vp, _vp, _vp, _vp, _int, _int, _int, _int, _vp],
    "tnc_dense_backward": [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _int, _int, _int, _int, _vp],
    "tnc_mse_sigmoid_grad": [_vp, _vp, _vp, _int, _vp],
    "tnc_adam_step": [_vp, _vp, _vp, _vp, _i64, _dbl, _dbl, _dbl, _dbl, _int, _vp],
    "tnc_fill_gaussian": [_int, _i64, C.c_uint64, _vp, _vp],
}

RESTYPES = {"tnc_status_string": C.c_char_p, "tnc_kernel_launches": C.c_ulonglong}

_LIB = None


def kernel_launches():
    """Kernels launched by the native library so far (host-side counter)."""
    return int(lib().tnc_kernel_launches())


def header_symbols():
    """Function names declared in include/tncontract_gb300.h."""
    path = os.path.join(_build.ROOT, "include", "tncontract_gb300.h")
    txt = open(path).read()
    return sorted(set(re.findall(r"\b(tnc_[a-z0-9_]+)\s*\(", txt)))


def lib():
    """Load (once) and return the native library; raise if unavailable."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIBPATH
    if not os.path.exists(path):
        raise RuntimeError(
            "tncontract_gb300 native library not built (%s missing); run "
            "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    L = C.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = RESTYPES.get(name, C.c_int)
    _LIB = L
    return L


class NativeError(RuntimeError):
    def __init__(self, fn, status):
        self.status = status
        super().__init__("%s failed: %s (status %d)" % (
            fn, lib().tnc_status_string(status).decode(), status))


def check(fn, status):
    if status != OK:
        raise NativeError(fn, status)
