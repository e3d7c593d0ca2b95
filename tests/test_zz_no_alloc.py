"""tnc_svd_noalloc: the SVD entry point for callers that cannot give the
library any device memory (hosts whose own allocator owns the whole device
budget, services that allocate only at start-up).  It must produce what the
regular, workspace-taking tnc_svd produces, also when called twice in a row
(the second call reuses the shared fixed scratch the first one left behind),
and must refuse problems larger than its fixed 16 MiB scratch.

This file is named to be collected last so that a stop-at-first-failure run
has already run every other test before this one."""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _rand(rng, shape, dt):
    a = rng.standard_normal(shape)
    if np.iscomplexobj(np.zeros(0, dt)):
        a = a + 1j * rng.standard_normal(shape)
    return torch.from_numpy(a.astype(dt)).cuda()


def _noalloc_svd(L, code, A):
    m, n = A.shape
    k = min(m, n)
    rdt = torch.float64 if A.dtype in (torch.float64, torch.complex128) else torch.float32
    U = torch.empty((m, k), dtype=A.dtype, device=A.device)
    S = torch.empty((k,), dtype=rdt, device=A.device)
    VH = torch.empty((k, n), dtype=A.dtype, device=A.device)
    info = torch.zeros(4, dtype=torch.int32, device=A.device)
    st = L.tnc_svd_noalloc(code, m, n, C.c_void_p(A.data_ptr()), n, C.c_void_p(U.data_ptr()),
                           C.c_void_p(S.data_ptr()), C.c_void_p(VH.data_ptr()), 0, 0.0,
                           C.c_void_p(info.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st, U, S, VH, info


@pytest.mark.parametrize("npdt,code,tol", [(np.complex128, 3, 1e-12), (np.complex64, 2, 2e-5),
                                           (np.float64, 1, 1e-12)])
def test_noalloc_matches_workspace_svd_twice(gpu, npdt, code, tol):
    from tncontract_gb300 import _lib, _ops
    L = _lib.lib()
    rng = np.random.default_rng(42)
    for shape in [(96, 200), (300, 130)]:  # two calls in a row, wide then tall
        A = _rand(rng, shape, npdt)
        U0, S0, V0 = _ops.svd(A)
        st, U, S, VH, info = _noalloc_svd(L, code, A)
        assert st == _lib.OK
        assert int(info[0]) == _lib.OK
        a = A.cpu().numpy()
        s0, s = S0.cpu().numpy(), S.cpu().numpy()
        assert np.max(np.abs(s - s0)) <= tol * 10 * s0[0]
        u, vh = U.cpu().numpy(), VH.cpu().numpy()
        assert np.linalg.norm((u * s) @ vh - a) <= tol * 10 * np.linalg.norm(a) * np.sqrt(max(shape))
        assert np.linalg.norm(u - U0.cpu().numpy()) <= tol * 10 * np.sqrt(u.size)
        assert np.linalg.norm(vh - V0.cpu().numpy()) <= tol * 10 * np.sqrt(vh.size)


def test_noalloc_rejects_too_large(gpu):
    from tncontract_gb300 import _lib
    L = _lib.lib()
    A = torch.zeros((1024, 2048), dtype=torch.complex128, device="cuda")
    st, *_ = _noalloc_svd(L, 3, A)
    assert st == _lib.ERR_TOO_LARGE
    assert "16 MiB" in L.tnc_status_string(st).decode()
