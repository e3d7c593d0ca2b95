"""Native kernels through the C ABI vs NumPy (same LAPACK/BLAS the reference
uses).  Tolerances: FP64 paths 1e-12 relative, FP32 paths 2e-5 relative."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DTYPES = [np.float32, np.float64, np.complex64, np.complex128]


def tol(dt):
    return 2e-5 if np.dtype(dt) in (np.float32, np.complex64) else 1e-12


def rnd(rng, shape, dt):
    a = rng.standard_normal(shape)
    if np.iscomplexobj(np.zeros(0, dt)):
        a = a + 1j * rng.standard_normal(shape)
    return a.astype(dt)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    return t.detach().cpu().numpy()


def relerr(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("dt", DTYPES)
def test_permute(gpu, dt):
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(1)
    cases = [((5,), [0]), ((3, 4), [1, 0]), ((33, 65), [1, 0]), ((2, 3, 4), [2, 0, 1]),
             ((7, 1, 9, 2), [3, 2, 1, 0]), ((4, 5, 6, 3), [0, 2, 1, 3]), ((2, 3, 2, 3, 2, 3), [5, 1, 3, 0, 4, 2]),
             ((64, 3, 96), [2, 1, 0]), ((1, 1, 5), [2, 0, 1]), ((130, 70), [1, 0])]
    for shape, perm in cases:
        a = rnd(rng, shape, dt)
        for conj in (False, True):
            out = host(_ops.permute(dev(a), perm, conj=conj))
            ref = np.transpose(a, perm)
            if conj:
                ref = np.conj(ref)
            assert out.shape == ref.shape
            assert np.array_equal(out, ref), (shape, perm, conj)


@pytest.mark.parametrize("dt", DTYPES)
def test_gemm_ops(gpu, dt):
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(2)
    opf = {0: lambda x: x, 1: lambda x: x.T, 2: lambda x: np.conj(x).T, 3: np.conj}
    for (m, n, k) in [(1, 1, 1), (5, 7, 3), (64, 64, 64), (65, 130, 17), (200, 33, 257), (3, 300, 2)]:
        for opA in range(4):
            for opB in range(4):
                A = rnd(rng, (k, m) if opA in (1, 2) else (m, k), dt)
                B = rnd(rng, (n, k) if opB in (1, 2) else (k, n), dt)
                out = host(_ops.matmul(dev(A), dev(B), opA, opB))
                ref = opf[opA](A) @ opf[opB](B)
                assert relerr(out, ref) < 10 * tol(dt), (m, n, k, opA, opB)


def test_gemm_batched_alpha_beta(gpu):
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(3)
    b, m, n, k = 3, 20, 30, 40
    A = rnd(rng, (b, m, k), np.complex128)
    B = rnd(rng, (b, k, n), np.complex128)
    Cm = rnd(rng, (b, m, n), np.complex128)
    Cd = dev(Cm)
    _ops.gemm(0, 0, m, n, k, dev(A), k, dev(B), n, Cd, n, alpha=2 - 1j, beta=0.5j, batch=b,
              sA=m * k, sB=k * n, sC=m * n)
    ref = (2 - 1j) * np.einsum("bmk,bkn->bmn", A, B) + 0.5j * Cm
    assert relerr(host(Cd), ref) < 1e-12
    # K == 0: C = beta * C
    Z = dev(np.zeros((0,)))
    Cz = dev(Cm[0])
    _ops.gemm(0, 0, m, n, 0, Z, 1, Z, 1, Cz, n, beta=0.0)
    assert np.all(host(Cz) == 0)


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("shape", [(1, 1), (1, 7), (7, 1), (6, 6), (40, 13), (13, 40), (130, 97), (256, 512),
                                   (700, 300), (300, 700), (1536, 768)])
def test_qr(gpu, dt, shape):
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(4)
    A = rnd(rng, shape, dt)
    Q, R = _ops.qr(dev(A))
    Q, R = host(Q), host(R)
    m, n = shape
    k = min(m, n)
    assert Q.shape == (m, k) and R.shape == (k, n)
    t = tol(dt) * max(m, n)
    assert relerr(Q @ R, A) < t
    assert np.linalg.norm(np.conj(Q).T @ Q - np.eye(k)) < t * np.sqrt(k)
    assert np.allclose(np.tril(R, -1), 0)
    # same Householder convention as LAPACK: |diag R| agrees, diag real
    _, Rn = np.linalg.qr(A.astype(np.complex128 if np.iscomplexobj(A) else np.float64))
    assert np.allclose(np.abs(np.diag(R)), np.abs(np.diag(Rn)), rtol=1e3 * t, atol=1e3 * t)
    assert np.allclose(np.imag(np.diag(R)), 0, atol=t)


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("shape", [(1, 1), (1, 7), (7, 1), (40, 13), (13, 40), (256, 512), (700, 300), (512, 768)])
def test_qr_r_only(gpu, dt, shape):
    """tnc_qr_r: R of A and of A^H equal the R of the full QR of the same
    matrix (same reflectors, Q not formed)."""
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(14)
    A = rnd(rng, shape, dt)
    for adjoint in (False, True):
        X = np.ascontiguousarray(np.conj(A).T) if adjoint else A
        R = host(_ops.qr_r(dev(A), adjoint=adjoint))
        _, Rfull = _ops.qr(dev(X))
        Rfull = host(Rfull)
        assert R.shape == Rfull.shape == (min(shape), X.shape[1])
        assert relerr(R, Rfull) < tol(dt)
        # R^H R = X^H X
        t = tol(dt) * max(shape)
        assert relerr(np.conj(R).T @ R, np.conj(X).T @ X) < t


@pytest.mark.parametrize("dt", DTYPES)
def test_qr_blocked_degenerate(gpu, dt):
    """Blocked QR (k >= 128) with a column already in triangular form (its
    reflector is the identity, tau = 0), a zero column and a repeated column."""
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(15)
    A = rnd(rng, (300, 200), dt)
    A[:, 0] = 0
    A[0, 0] = 2
    A[:, 70] = 0
    A[:, 150] = A[:, 5]
    Q, R = (host(x) for x in _ops.qr(dev(A)))
    t = tol(dt) * 300
    assert relerr(Q @ R, A) < t
    assert np.linalg.norm(np.conj(Q).T @ Q - np.eye(200)) < t * np.sqrt(200)


def test_qr_rank_deficient(gpu):
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(5)
    A = rnd(rng, (50, 4), np.float64) @ rnd(rng, (4, 30), np.float64)  # rank 4
    A[:, 7] = 0.0
    Q, R = (host(x) for x in _ops.qr(dev(A)))
    assert relerr(Q @ R, A) < 1e-12
    assert np.linalg.norm(Q.T @ Q - np.eye(30)) < 1e-11


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("shape", [(1, 1), (1, 9), (9, 1), (2, 2), (17, 5), (5, 17), (64, 64), (96, 200), (300, 130)])
def test_svd(gpu, dt, shape):
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(6)
    A = rnd(rng, shape, dt)
    U, S, VH = (host(x) for x in _ops.svd(dev(A)))
    m, n = shape
    k = min(m, n)
    assert U.shape == (m, k) and S.shape == (k,) and VH.shape == (k, n)
    s_ref = np.linalg.svd(A.astype(np.complex128), compute_uv=False)
    t = tol(dt) * np.sqrt(max(m, n))
    assert np.max(np.abs(S - s_ref)) < 10 * t * s_ref[0]
    assert np.all(np.diff(S) <= 0)
    assert relerr((U * S) @ VH, A) < 10 * t
    assert np.linalg.norm(np.conj(U).T @ U - np.eye(k)) < 10 * t * np.sqrt(k)
    assert np.linalg.norm(VH @ np.conj(VH).T - np.eye(k)) < 10 * t * np.sqrt(k)


def test_svd_rank_deficient_and_degenerate(gpu):
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(7)
    A = rnd(rng, (60, 5), np.complex128) @ rnd(rng, (5, 40), np.complex128)
    U, S, VH = (host(x) for x in _ops.svd(dev(A)))
    s_ref = np.linalg.svd(A, compute_uv=False)
    assert np.max(np.abs(S - s_ref)) < 1e-12 * s_ref[0]
    assert relerr((U * S) @ VH, A) < 1e-12
    # degenerate spectrum (isometry): all singular values 1
    Q, _ = np.linalg.qr(rnd(rng, (50, 20), np.float64))
    S2 = host(_ops.svd(dev(Q))[1])
    assert np.max(np.abs(S2 - 1)) < 1e-13


def test_svd_nonfinite_raises(gpu):
    from tncontract_gb300 import _ops
    A = np.ones((6, 4))
    A[2, 1] = np.nan
    with pytest.raises(ValueError):
        _ops.svd(dev(A))


def test_truncation_rank_rule(gpu):
    import tn_oracle as O
    from tncontract_gb300 import _ops
    s = np.array([5.0, 3.0, 1.0, 1e-3, 1e-15, 0.0])
    for chi in (0, 1, 2, 4, 10):
        for thr in (1e-15, 1e-4, 0.5, 2.0):
            for absolute in (True, False):
                k, disc = _ops.truncation_rank(dev(s), chi, thr, relative=not absolute)
                assert k == O.truncation_keep(s, chi, thr, absolute), (chi, thr, absolute)
                assert abs(disc - np.sum(s[k:] ** 2)) < 1e-14
            kc, _ = _ops.truncation_rank(dev(s), chi, thr, relative=True)
            assert kc == O.canonise_keep(s, chi, thr)


@pytest.mark.parametrize("dt", DTYPES)
def test_reductions_and_elementwise(gpu, dt):
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(8)
    a = rnd(rng, (3, 40, 7), dt)
    b = rnd(rng, (3, 40, 7), dt)
    t = tol(dt)
    assert abs(_ops.nrm2(dev(a)) - np.linalg.norm(a)) < t * np.linalg.norm(a)
    d = host(_ops.dot_device(dev(a), dev(b), conj_x=True))
    ref = np.vdot(a, b)
    assert abs(complex(d[0], d[1]) - ref) < 10 * t * np.linalg.norm(a) * np.linalg.norm(b)
    z = 0.5 - 2j if np.iscomplexobj(a) else -1.5
    assert relerr(host(_ops.scale(dev(a), z)), z * a) < t
    y = dev(b)
    _ops.axpby(z, dev(a), 2.0, y)
    assert relerr(host(y), z * a + 2.0 * b) < t
    sq = rnd(rng, (4, 6, 4, 3), dt)
    assert relerr(host(_ops.trace(dev(sq), 0, 2)), np.trace(sq, axis1=0, axis2=2)) < 10 * t
    M = rnd(rng, (9, 5), dt)
    sv = np.abs(rng.standard_normal(9)).astype(np.float32 if t > 1e-10 else np.float64)
    Md = dev(M)
    _ops.scale_rows(Md, dev(sv), 1)
    assert relerr(host(Md), np.sqrt(sv)[:, None] * M) < t
    out = host(_ops.slice_last(dev(a), 3))
    assert np.array_equal(out, a[..., :3])
    dm = host(_ops.diag_matrix(dev(sv[:5]), torch.from_numpy(np.zeros(0, dt)).dtype))
    assert np.array_equal(dm, np.diag(sv[:5]).astype(dt))


def test_cast(gpu):
    from tncontract_gb300 import _ops
    a = np.array([1.5, -2.25, 3.0])
    c = _ops.cast(dev(a), torch.complex64)
    assert np.array_equal(host(c), a.astype(np.complex64))
    r = _ops.cast(dev(np.array([1 + 2j, 3 - 4j])), torch.float64)
    assert np.array_equal(host(r), np.array([1.0, 3.0]))


@pytest.mark.parametrize("dt", [np.float64, np.complex128, np.complex64])
def test_mps_mpo_site(gpu, dt):
    import tn_oracle as O
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(9)
    A = rnd(rng, (2, 5, 7), dt)
    W = O.tfim_mpo(6)[2].astype(dt)
    ref = O.contract_mps_mpo([A], [W])[0]  # (phys, left, right)
    out1 = host(_ops.mps_mpo_site(dev(A), dev(W), 1))
    assert relerr(out1, ref) < tol(dt)
    out0 = host(_ops.mps_mpo_site(dev(A), dev(W), 0))
    assert relerr(out0, np.transpose(ref, (1, 0, 2))) < tol(dt)


@pytest.mark.parametrize("dt", [np.float32, np.complex64])
def test_gemm_tensor_core(gpu, dt):
    """tcgen05 GEMM (error-free BF16 digit split, exact level sums in tensor
    memory) against NumPy (FP64) at FP32-class tolerance, all op
    combinations, ragged sizes, batch and alpha/beta."""
    from tncontract_gb300 import _lib, _ops
    rng = np.random.default_rng(12)
    opf = {0: lambda x: x, 1: lambda x: x.T, 2: lambda x: np.conj(x).T, 3: np.conj}
    for (m, n, k) in [(128, 128, 32), (200, 136, 100), (512, 256, 768), (65, 300, 64)]:
        for opA in range(4):
            for opB in range(4):
                A = rnd(rng, (k, m) if opA in (1, 2) else (m, k), dt)
                B = rnd(rng, (n, k) if opB in (1, 2) else (k, n), dt)
                Cm = torch.empty((m, n), dtype=torch.from_numpy(np.zeros(0, dt)).dtype, device="cuda")
                _ops.gemm(opA, opB, m, n, k, dev(A), A.shape[1], dev(B), B.shape[1], Cm, n, tc=True)
                ref = opf[opA](A.astype(np.complex128)) @ opf[opB](B.astype(np.complex128))
                if not np.iscomplexobj(A):
                    ref = ref.real
                # inputs exact to their third 8-bit digit, FP32 round-to-nearest
                # sums of the chunks: FP32-class, ~1e-7 relative
                assert relerr(host(Cm), ref) < 2e-6, (m, n, k, opA, opB, relerr(host(Cm), ref))
    assert _lib.lib().tnc_gemm_tc_error() == 0
    # batched with alpha, beta
    b, m, n, k = 3, 130, 70, 96
    A = rnd(rng, (b, m, k), dt)
    B = rnd(rng, (b, k, n), dt)
    C0 = rnd(rng, (b, m, n), dt)
    Cd = dev(C0)
    al, be = (0.5 - 1j, 2j) if np.iscomplexobj(A) else (0.5, -2.0)
    _ops.gemm(0, 0, m, n, k, dev(A), k, dev(B), n, Cd, n, alpha=al, beta=be, batch=b,
              sA=m * k, sB=k * n, sC=m * n, tc=True)
    ref = al * np.einsum("bmk,bkn->bmn", A.astype(np.complex128), B) + be * C0
    if not np.iscomplexobj(A):
        ref = ref.real
    assert relerr(host(Cd), ref) < 3e-5
    assert _lib.lib().tnc_gemm_tc_error() == 0


@pytest.mark.parametrize("dt", [np.float32, np.float64, np.complex64, np.complex128])
def test_gemm_grouped(gpu, dt):
    """tnc_gemm_grouped: independent products of different shapes and
    operand layouts in one launch, each against NumPy."""
    from tncontract_gb300 import _lib as L
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(12)
    cplx = np.iscomplexobj(np.zeros(0, dt))

    def rnd(*shape):
        a = rng.standard_normal(shape)
        if cplx:
            a = a + 1j * rng.standard_normal(shape)
        return a.astype(dt)
    ops = {L.OP_N: lambda x: x, L.OP_T: lambda x: x.T, L.OP_C: lambda x: np.conj(x).T, L.OP_R: np.conj}
    cases = [(L.OP_N, L.OP_N, 70, 33, 129), (L.OP_T, L.OP_N, 5, 200, 17), (L.OP_N, L.OP_C, 64, 64, 64),
             (L.OP_C, L.OP_T, 130, 1, 300), (L.OP_R, L.OP_N, 1, 7, 3)]
    probs, want = [], []
    for opA, opB, m, n, k in cases:
        A = rnd(*((k, m) if opA in (L.OP_T, L.OP_C) else (m, k)))
        B = rnd(*((n, k) if opB in (L.OP_T, L.OP_C) else (k, n)))
        Cm = torch.empty((m, n), dtype=torch.from_numpy(A).dtype, device="cuda")
        probs.append((opA, opB, m, n, k, torch.from_numpy(A).cuda(), A.shape[1], torch.from_numpy(B).cuda(),
                      B.shape[1], Cm, n))
        want.append(ops[opA](A.astype(np.complex128)) @ ops[opB](B.astype(np.complex128)))
    before = L.kernel_launches()
    _ops.gemm_grouped(probs)
    torch.cuda.synchronize()
    assert L.kernel_launches() - before == 1
    tol = 1e-5 if dt in (np.float32, np.complex64) else 1e-12
    for p, w in zip(probs, want):
        assert np.linalg.norm(p[9].cpu().numpy() - w) <= tol * np.linalg.norm(w) + 1e-30


def test_con_wave_is_one_launch(gpu):
    """con's cost-ordered plan on the reference's 2x3 grid network issues one
    grouped GEMM launch per wave of independent pairwise contractions (no
    single-product GEMM), and the result is the reference's."""
    import api_cases as K
    import tncontract_gb300 as tn
    from tncontract_gb300 import _ops
    tensors, pairs, want, want_labels = K.con_fixture_network(tn, "grid_2x3_bfs")
    waves = K.con_waves(tn, tensors, pairs)
    assert max(len(w) for w in waves) >= 2
    _ops.PROFILE = {}
    try:
        r = tn.con(tensors, pairs)
        torch.cuda.synchronize()
        prof = _ops.PROFILE
    finally:
        _ops.PROFILE = None
    assert len(prof.get("tnc_gemm_grouped", [])) == len(waves)
    assert "tnc_gemm" not in prof and "tnc_gemm_tc" not in prof
    assert r.labels == want_labels and K.close(r.to_numpy(), want, 1e-12)


@pytest.mark.parametrize("dt", [np.float32, np.complex64])
def test_gemm_tensor_core_unbiased(gpu, dt):
    """The tensor-core GEMM keeps magnitudes: over many long-K products the
    mean relative change of |C| against the exact product is zero within the
    statistical scatter, and a chain of 64 products with unitary factors
    keeps the norm of a block to FP32 rounding (a truncating accumulation
    shrank it by ~1e-8 K per product)."""
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(31)
    m, n, k = 256, 256, 1536
    A = rnd(rng, (m, k), dt)
    B = rnd(rng, (k, n), dt)
    Cm = torch.empty((m, n), dtype=torch.from_numpy(np.zeros(0, dt)).dtype, device="cuda")
    _ops.gemm(0, 0, m, n, k, dev(A), k, dev(B), n, Cm, n, tc=True)
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    got = host(Cm).astype(np.complex128)
    rel = (np.abs(got) - np.abs(ref)) / np.abs(ref)
    rel = rel[np.abs(ref) > 0.1 * np.sqrt(k)]
    assert abs(rel.mean()) < 5 * rel.std() / np.sqrt(rel.size) + 1e-9, (rel.mean(), rel.std())
    # a chain of unitary products: X <- Q X, 64 times
    cplx = np.iscomplexobj(np.zeros(0, dt))
    Q = np.linalg.qr(rnd(rng, (512, 512), np.complex128 if cplx else np.float64))[0]
    Qd = dev(Q.astype(dt))
    X = rnd(rng, (512, 256), dt)
    Xd = dev(X)
    q_norm = np.linalg.norm(Q.astype(dt).astype(np.complex128), 2)
    for _ in range(64):
        Y = torch.empty_like(Xd)
        _ops.gemm(0, 0, 512, 256, 512, Qd, 512, Xd, 256, Y, 256, tc=True)
        Xd = Y
    drift = abs(np.linalg.norm(host(Xd)) / np.linalg.norm(X) - 1.0)
    assert drift < 64 * 2e-7, drift
