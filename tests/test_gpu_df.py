"""The double-float Jacobi finish (tnc_svd_rows_df) on the GPU against FP64
LAPACK of the same single-precision input.

One-sided Jacobi multiplies the rows by a unitary Q, so W^H W = A^H A must
hold to the arithmetic's precision (DF: about 2^-46 per operation; bound
1e-11 |A|_F^2 here), the rows must come out orthogonal to the tolerance
(1e-7 relative, x10 slack), and the row norms are A's singular values
(bound 1e-10 s_max, the orthogonality error entering at second order).
Cases: a from-scratch SVD (every rotation a large angle), rows already
orthogonal to FP32 level (the finish's use, small angles), exactly repeated
singular values (large angles between nearly equal norms), real rows, and
rows beyond nkeep."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-7


def rnd(rng, shape, cplx):
    a = rng.standard_normal(shape)
    return a + 1j * rng.standard_normal(shape) if cplx else a


def graded(rng, m, n, s, cplx):
    U = np.linalg.qr(rnd(rng, (m, m), cplx))[0]
    V = np.linalg.qr(rnd(rng, (n, m), cplx))[0]
    return (U * s) @ np.conj(V).T


def check(A32, W, S, order, info, nkeep=None, s_bound=1e-10):
    assert int(info[0].item()) == 0, info.cpu().numpy()
    A = A32.astype(np.complex128)
    Wn = W.cpu().numpy().astype(np.complex128)
    s = S.cpu().numpy()
    o = order.cpu().numpy()
    f2 = np.linalg.norm(A) ** 2
    # W = Q A with Q unitary
    assert np.linalg.norm(np.conj(Wn).T @ Wn - np.conj(A).T @ A) < 1e-11 * f2
    # S: the row norms, sorted, equal to A's singular values
    nrm = np.linalg.norm(Wn, axis=1)
    assert np.allclose(s, nrm[o], rtol=1e-12, atol=1e-14 * np.sqrt(f2))
    assert np.all(np.diff(s) <= 0)
    s_ref = np.linalg.svd(A, compute_uv=False)
    if nkeep is None:
        assert np.max(np.abs(s - s_ref)) < s_bound * s_ref[0]
    # orthogonality of the rows that must be orthogonal to every row
    rows = len(nrm) if nkeep is None else nkeep
    floor = (1.4e-14 ** 2) * f2  # rows at the noise floor take no rotation
    live = nrm ** 2 > floor
    G = np.abs(Wn[:rows] @ np.conj(Wn).T) / np.maximum(np.outer(nrm[:rows], nrm), 1e-300)
    G[np.arange(rows), np.arange(rows)] = 0.0
    G[~live[:rows], :] = 0.0
    G[:, ~live] = 0.0
    assert G.max() <= 10 * TOL, np.unravel_index(G.argmax(), G.shape)
    return s, s_ref


@pytest.mark.parametrize("cplx", [True, False])
@pytest.mark.parametrize("shape", [(2, 2), (3, 40), (33, 65), (96, 200), (256, 512), (512, 512)])
def test_df_from_scratch(gpu, cplx, shape):
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(5)
    A = rnd(rng, shape, cplx).astype(np.complex64 if cplx else np.float32)
    W, S, order, info = _ops.svd_rows_df(torch.from_numpy(A).cuda(), tol=TOL)
    check(A, W, S, order, info)


@pytest.mark.parametrize("cplx", [True, False])
def test_df_finish_of_fp32_rows(gpu, cplx):
    """The sweep's use: FP32 Jacobi rows (orthogonal to 3e-6), sorted, then
    the DF finish; against the FP64 finish of the same rows."""
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(7)
    m, n = 384, 512
    s_true = 10.0 ** (-8.0 * np.arange(m) / (m - 1))
    A = graded(rng, m, n, s_true, cplx).astype(np.complex64 if cplx else np.float32)
    W32, S32, o32, info32 = _ops.svd_rows(torch.from_numpy(A).cuda(), max_sweeps=14, tol=3e-6)
    rows = W32[o32].contiguous()
    W, S, order, info = _ops.svd_rows_df(rows, tol=TOL)
    s, s_ref = check(rows.cpu().numpy(), W, S, order, info)
    wide = torch.complex128 if cplx else torch.float64
    W64, S64, o64, info64 = _ops.svd_rows(rows.to(wide), tol=TOL)
    assert int(info64[0].item()) == 0
    assert np.max(np.abs(s - S64.cpu().numpy())) < 1e-10 * s_ref[0]


def test_df_repeated_singular_values(gpu):
    """Clusters of four equal singular values: inside a cluster a residual
    inner product d (<= TOL relative) moves the row norms by d/2, first
    order, so the norms are bound by TOL s_max there -- as for the FP64
    finish at the same tolerance, which the DF one is compared with."""
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(9)
    m, n = 200, 320
    s_true = np.repeat(10.0 ** (-6.0 * np.arange(m // 4) / (m // 4 - 1)), 4)
    A = graded(rng, m, n, s_true, True).astype(np.complex64)
    W, S, order, info = _ops.svd_rows_df(torch.from_numpy(A).cuda(), tol=TOL)
    s, s_ref = check(A, W, S, order, info, s_bound=TOL)
    W64, S64, o64, info64 = _ops.svd_rows(torch.from_numpy(A.astype(np.complex128)).cuda(), tol=TOL)
    assert int(info64[0].item()) == 0
    assert np.max(np.abs(S64.cpu().numpy() - s_ref)) < TOL * s_ref[0]


@pytest.mark.parametrize("nkeep", [1, 40, 64])
def test_df_nkeep(gpu, nkeep):
    """Rows beyond nkeep (whole half-blocks of 8) rotate only against the
    kept ones: the kept rows come out orthogonal to every row."""
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(13)
    m, n = 128, 256
    s_true = 10.0 ** (-6.0 * np.arange(m) / (m - 1))
    A = graded(rng, m, n, s_true, True).astype(np.complex64)
    W32, S32, o32, _ = _ops.svd_rows(torch.from_numpy(A).cuda(), max_sweeps=14, tol=3e-6)
    rows = W32[o32].contiguous()
    W, S, order, info = _ops.svd_rows_df(rows, tol=TOL, nkeep=nkeep)
    s, s_ref = check(rows.cpu().numpy(), W, S, order, info, nkeep=-(-nkeep // 8) * 8)
    k = -(-nkeep // 8) * 8
    assert np.max(np.abs(s[:k] - s_ref[:k])) < 1e-10 * s_ref[0]


def test_df_argument_errors(gpu):
    from tncontract_gb300 import _lib as L
    import ctypes as C
    lib = L.lib()
    A = torch.zeros((8, 4), dtype=torch.complex64, device="cuda")
    W = torch.zeros((8, 4), dtype=torch.complex128, device="cuda")
    S = torch.zeros(8, dtype=torch.float64, device="cuda")
    o = torch.zeros(8, dtype=torch.int64, device="cuda")
    info = torch.zeros(4, dtype=torch.int32, device="cuda")
    ws = torch.zeros(1 << 16, dtype=torch.uint8, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    args = (p(A), p(W), p(S), p(o), 0, 0.0, 0, 8, p(ws), 1 << 16, p(info), None)
    assert lib.tnc_svd_rows_df(L.C64, 8, 4, *args) == L.ERR_ARG          # tall
    assert lib.tnc_svd_rows_df(L.C128, 4, 8, *args) == L.ERR_ARG         # not single precision
    small = (p(A), p(W), p(S), p(o), 0, 0.0, 0, 4, p(ws), 16, p(info), None)
    assert lib.tnc_svd_rows_df(L.C64, 4, 8, *small) == L.ERR_WORKSPACE


def test_stage_stop_then_finish(gpu):
    """tnc_svd_rows_stage: with stop_tol the FP32 stage stops (status OK,
    info[3] = 1) after the first sweep whose rotations were all below it,
    in fewer sweeps than the full run; the double-float finish from those
    rows still meets every bound above, and the singular values match
    LAPACK's of the input to the FP32 stage's backward error (FP32-class,
    1e-4 of s_max; measured 1.4-5.4e-5 with or without the stop)."""
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(17)
    m, n = 256, 384
    s_true = 10.0 ** (-6.0 * np.arange(m) / (m - 1))
    A = torch.from_numpy(graded(rng, m, n, s_true, True).astype(np.complex64)).cuda()
    W0, S0, o0, i0 = _ops.svd_rows_stage(A, 40, 3e-6, 0.0)
    W1, S1, o1, i1 = _ops.svd_rows_stage(A, 40, 3e-6, 1e-3)
    i0, i1 = i0.cpu().numpy(), i1.cpu().numpy()
    assert i0[0] == 0 and i0[3] == 0
    assert i1[0] == 0 and i1[3] == 1 and i1[1] < i0[1], (i0, i1)
    kall = torch.tensor([m], dtype=torch.int64, device="cuda")
    rows = _ops.gather_rows(W1, o1, kall, m)
    W, S, order, info = _ops.svd_rows_df(rows, tol=TOL)
    s, _ = check(rows.cpu().numpy(), W, S, order, info)
    s_a = np.linalg.svd(A.cpu().numpy().astype(np.complex128), compute_uv=False)
    assert np.max(np.abs(s - s_a)) < 1e-4 * s_a[0]
    s0 = S0.cpu().numpy()
    assert np.max(np.abs(s - s0)) < 1e-4 * s_a[0]
