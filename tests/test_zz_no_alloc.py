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


def _ws_bytes(L, code, m, n):
    b = C.c_size_t()
    assert L.tnc_svd_workspace_size(code, m, n, C.byref(b)) == 0
    return b.value


# (dtype code, numpy dtype, largest accepted shape, one row or column more)
BOUNDARY = [(3, np.complex128, (433, 512), (434, 512)),
            (3, np.complex128, (450, 450), (451, 451)),
            (2, np.complex64, (1024, 531), (1024, 532))]


@pytest.mark.parametrize("code,npdt,fits,over", BOUNDARY)
def test_noalloc_size_boundary(gpu, code, npdt, fits, over):
    """At the edge of the 16 MiB scratch (the rule is tnc_svd_workspace_size
    <= 16 MiB): the largest accepted shape runs and matches tnc_svd; one row
    or column more is refused with TNC_ERR_TOO_LARGE, nothing is launched
    and U, S, VH and info keep what they held."""
    from tncontract_gb300 import _lib, _ops
    L = _lib.lib()
    limit = 16 << 20
    assert _ws_bytes(L, code, *fits) <= limit < _ws_bytes(L, code, *over)
    rng = np.random.default_rng(7)
    A = _rand(rng, fits, npdt)
    st, U, S, VH, info = _noalloc_svd(L, code, A)
    assert st == _lib.OK and int(info[0]) == _lib.OK
    s0 = _ops.svd(A)[1].cpu().numpy()
    tol = 1e-12 if code == 3 else 2e-5
    assert np.max(np.abs(S.cpu().numpy() - s0)) <= tol * 10 * s0[0]
    # one more row / column: refused before any launch or write
    A = _rand(rng, over, npdt)
    m, n = over
    k = min(m, n)
    rdt = torch.float64 if code == 3 else torch.float32
    U = torch.full((m, k), 7.0, dtype=A.dtype, device="cuda")
    S = torch.full((k,), 7.0, dtype=rdt, device="cuda")
    VH = torch.full((k, n), 7.0, dtype=A.dtype, device="cuda")
    info = torch.full((4,), 99, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    before = _lib.kernel_launches()
    st = L.tnc_svd_noalloc(code, m, n, C.c_void_p(A.data_ptr()), n, C.c_void_p(U.data_ptr()),
                           C.c_void_p(S.data_ptr()), C.c_void_p(VH.data_ptr()), 0, 0.0,
                           C.c_void_p(info.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert st == _lib.ERR_TOO_LARGE
    assert _lib.kernel_launches() == before
    assert bool((U == 7.0).all()) and bool((S == 7.0).all()) and bool((VH == 7.0).all())
    assert bool((info == 99).all())


def test_noalloc_rejects_too_large(gpu):
    from tncontract_gb300 import _lib
    L = _lib.lib()
    A = torch.zeros((1024, 2048), dtype=torch.complex128, device="cuda")
    st, *_ = _noalloc_svd(L, 3, A)
    assert st == _lib.ERR_TOO_LARGE
    assert "16 MiB" in L.tnc_status_string(st).decode()
