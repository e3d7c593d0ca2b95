"""Sweep engine and its Jacobi stage on the GPU, against the oracle and the
reference's fixtures.  Fidelity-error bounds: 1e-10 for FP64 storage, 1e-6
for FP32 storage (the tolerance of FP32-class paths)."""
import numpy as np
import pytest
import torch

import api_cases as K
import tn_oracle as O

pytestmark = pytest.mark.gpu


def rnd(rng, shape, dt):
    a = rng.standard_normal(shape)
    if np.iscomplexobj(np.zeros(0, dt)):
        a = a + 1j * rng.standard_normal(shape)
    return a.astype(dt)


@pytest.mark.parametrize("dt", [np.float32, np.float64, np.complex64, np.complex128])
@pytest.mark.parametrize("shape", [(2, 2), (3, 40), (40, 3), (33, 65), (96, 200), (260, 120), (512, 768)])
@pytest.mark.parametrize("block_rows", [None, 8, 16, 32])
def test_svd_rows(gpu, dt, shape, block_rows):
    """block_rows: None the autotuner's choice, 8 / 16 the row-by-row
    rotation kernel, 32 (TNC_ROWS_GRAM) the Gram-form block update (single
    precision; the other types run the row-by-row kernel)."""
    from tncontract_gb300 import _ops
    if np.dtype(dt).itemsize * (2 if np.iscomplexobj(np.zeros(0, dt)) else 1) >= 16 and max(shape) > 512:
        pytest.skip("FP64 complex rows above 512 use the accumulating SVD")
    rng = np.random.default_rng(11)
    A = rnd(rng, shape, dt)
    W, S, order, info = _ops.svd_rows(torch.from_numpy(A).cuda(), block_rows=block_rows)
    assert int(info[0].item()) == 0
    s = S.cpu().numpy()
    s_ref = np.linalg.svd(A.astype(np.complex128), compute_uv=False)
    tol = 2e-5 if np.dtype(dt) in (np.float32, np.complex64) else 1e-12
    assert np.max(np.abs(s - s_ref)) < 10 * tol * np.sqrt(max(shape)) * s_ref[0]
    Wh = W.cpu().numpy()[order.cpu().numpy()]
    G = Wh @ np.conj(Wh).T
    off = G - np.diag(np.diag(G))
    assert np.linalg.norm(off) < 10 * tol * np.sqrt(max(shape)) * s_ref[0] ** 2 * np.sqrt(min(shape))


@pytest.mark.parametrize("dt", [np.float32, np.complex64, np.float64, np.complex128])
@pytest.mark.parametrize("shape", [(200, 300), (300, 200), (256, 256), (600, 300)])
def test_factor_full_graded(gpu, dt, shape):
    """The sweep factorisation on a graded matrix whose spectrum falls from 1
    to 1e-40 (the boundary-MPS matrices of a PEPS norm network look like
    this): converges, U orthonormal for every direction the rank rule keeps,
    U (S V^H) = M up to the discarded weight, S against LAPACK.  FP64 with
    600 rows takes the accumulating-SVD branch."""
    from tncontract_gb300 import engine as E
    rng = np.random.default_rng(21)
    m, n = shape
    k = min(m, n)
    cplx = np.iscomplexobj(np.zeros(0, dt))
    Ux = np.linalg.qr(rnd(rng, (m, k), np.complex128 if cplx else np.float64))[0]
    Vx = np.linalg.qr(rnd(rng, (n, k), np.complex128 if cplx else np.float64))[0]
    s_true = 10.0 ** (-40.0 * np.arange(k) / (k - 1))
    M = ((Ux * s_true) @ np.conj(Vx).T).astype(dt)
    single = np.dtype(dt) in (np.float32, np.complex64)
    S, factors = E._factor_full(torch.from_numpy(M).cuda())
    s_ref = np.linalg.svd(M.astype(np.complex128), compute_uv=False)
    s = S.cpu().numpy().astype(np.float64)
    tol = 2e-5 if single else 1e-12
    assert np.max(np.abs(s - s_ref)) < 10 * tol * np.sqrt(max(shape)) * s_ref[0]
    # the engine's rule: the reference's threshold, capped at the noise floor
    kk = min(E.reference_rank(s, 0, 1e-14), E.noise_rank(s, torch.from_numpy(M).dtype))
    assert kk >= int(np.count_nonzero(s_ref > (1e-5 if single else 1e-13) * s_ref[0]))
    U, SV = factors(kk, torch.tensor([kk], dtype=torch.int64, device="cuda"))
    U = U.cpu().numpy().astype(np.complex128)
    SV = SV.cpu().numpy().astype(np.complex128)
    assert np.linalg.norm(np.conj(U).T @ U - np.eye(kk)) < 100 * tol * np.sqrt(kk)
    err = np.linalg.norm(U @ SV - M.astype(np.complex128)) / np.linalg.norm(M.astype(np.complex128))
    assert err < 10 * tol * np.sqrt(max(shape))


def _run_engine(tn_engine, sites, mpo, chi, precision, cplx=True):
    dt = tn_engine.compute_dtype(precision, cplx)
    bal, ln = tn_engine.balance(sites)
    S = tn_engine.to_sites(bal, dt)
    Mo = tn_engine.to_sites(mpo, dt)
    st = tn_engine.SweepStats()
    out = tn_engine.apply_compress(S, Mo, chi, stats=st, log_norm_in=ln)
    torch.cuda.synchronize()
    return [o.cpu().numpy().astype(np.complex128) for o in out], st


@pytest.mark.parametrize("precision,fid_tol", [("fp64", 1e-10), ("fp32", 1e-6)])
def test_engine_config2_small(gpu, precision, fid_tol):
    from tncontract_gb300 import engine as E
    g, m = K.load("config2_small")
    N, chi = 12, 16
    sites = O.random_mps(0, N, 2, chi, np.complex128, normalise=True)
    mpo = O.tfim_mpo(N)
    got, st = _run_engine(E, sites, mpo, chi, precision)
    assert [1] + [a.shape[2] for a in got] == m["c2s_m_bonds"]
    ref = O.apply_compress_sweep(sites, mpo, chi)
    assert 1 - O.fidelity(ref, got) < fid_tol
    assert abs(O.mps_norm(got) - float(np.real(g["c2s_norm_m"]))) < fid_tol ** 0.5 * 10
    for s, s_ref in zip(O.bond_spectra(got), K.unpack(g, "c2s_m_spectra")):
        assert K.close(s, s_ref, 1e-8 if precision == "fp64" else 1e-4)


@pytest.mark.parametrize("precision,fid_tol", [("fp64", 1e-10), ("fp32", 1e-6)])
def test_engine_config2_chi128(gpu, precision, fid_tol):
    """The benchmark unit at chi=128, N=64 (config 2) against the oracle."""
    from tncontract_gb300 import engine as E
    g, m = K.load("config2_chi128")
    N, chi = 64, 128
    sites = O.random_mps(0, N, 2, chi, np.complex128, normalise=True)
    mpo = O.tfim_mpo(N)
    got, st = _run_engine(E, sites, mpo, chi, precision)
    assert [1] + [a.shape[2] for a in got] == m["c2_m_bonds"]
    ref = O.apply_compress_sweep(sites, mpo, chi)
    err = 1 - O.fidelity(ref, got)
    assert err < fid_tol, err
    phi = O.contract_mps_mpo(sites, mpo)
    assert abs(O.fidelity(phi, got) - float(np.real(g["c2_fid_m_phi"]))) < 10 * fid_tol


def test_engine_real_config1(gpu):
    """Real float64 input (config 1 sizes) through the engine in FP64."""
    from tncontract_gb300 import engine as E
    sites = O.random_mps(0, 32, 2, 32, np.float64)
    lc = O.left_canonical_form_mps(sites)
    mpo = [np.eye(2).reshape(2, 2, 1, 1) for _ in range(32)]  # identity MPO
    got, _ = _run_engine(E, lc, mpo, 16, "fp64", cplx=False)
    ref = O.svd_compress_method(lc, 16)
    assert 1 - O.fidelity(ref, got) < 1e-10


def test_engine_batched(gpu):
    from tncontract_gb300 import engine as E
    N, chi = 16, 24
    mpo = O.tfim_mpo(N)
    batch_np = [O.random_mps(s, N, 2, chi, np.complex128, normalise=True) for s in range(4)]
    dt = E.compute_dtype("fp32", True)
    bal = [E.balance(b) for b in batch_np]
    batch = [E.to_sites(b, dt) for b, _ in bal]
    Mo = E.to_sites(mpo, dt)
    outs = E.apply_compress_batch(batch, Mo, chi, log_norms=[ln for _, ln in bal])
    torch.cuda.synchronize()
    for b, out in zip(batch_np, outs):
        got = [o.cpu().numpy().astype(np.complex128) for o in out]
        ref = O.apply_compress_sweep(b, mpo, chi)
        assert 1 - O.fidelity(ref, got) < 1e-6


@pytest.mark.parametrize("precision,fid_tol", [("fp64", 1e-10), ("fp32", 1e-6)])
@pytest.mark.parametrize("case", ["config2_small", "config2_chi128"])
def test_native_sweep(gpu, precision, fid_tol, case):
    """tnc_sweep_apply_compress (the whole sweep as one native call) against
    the oracle and the reference's bond dimensions."""
    from tncontract_gb300 import engine as E
    g, m = K.load(case)
    N, chi = (12, 16) if case == "config2_small" else (64, 128)
    key = "c2s_m_bonds" if case == "config2_small" else "c2_m_bonds"
    sites = O.random_mps(0, N, 2, chi, np.complex128, normalise=True)
    mpo = O.tfim_mpo(N)
    dt = E.compute_dtype(precision, True)
    bal, ln = E.balance(sites)
    st = E.SweepStats()
    out = E.apply_compress_native(E.to_sites(bal, dt), E.to_sites(mpo, dt), chi, log_norm_in=ln, stats=st)
    got = [o.cpu().numpy().astype(np.complex128) for o in out]
    assert [1] + [a.shape[2] for a in got] == m[key]
    ref = O.apply_compress_sweep(sites, mpo, chi)
    assert 1 - O.fidelity(ref, got) < fid_tol
    nr = O.mps_norm(ref)
    n_tol = 1e-9 if precision == "fp64" else 1e-5
    assert abs(O.mps_norm(got) * (1.0 if st.norm_folded else np.exp(st.log_norm - np.log(O.mps_norm(got)))) - nr) \
        < n_tol * nr


def test_native_sweep_real_and_batched(gpu):
    """Real float64 input through the native sweep, and native sweeps of
    several instances on the work queue."""
    from tncontract_gb300 import engine as E
    sites = O.random_mps(0, 32, 2, 32, np.float64)
    lc = O.left_canonical_form_mps(sites)
    ident = [np.eye(2).reshape(2, 2, 1, 1) for _ in range(32)]
    out = E.apply_compress_native(E.to_sites(lc, torch.float64), E.to_sites(ident, torch.float64), 16)
    got = [o.cpu().numpy() for o in out]
    assert 1 - O.fidelity(O.svd_compress_method(lc, 16), got) < 1e-10
    N, chi = 16, 24
    mpo = O.tfim_mpo(N)
    batch_np = [O.random_mps(s, N, 2, chi, np.complex128, normalise=True) for s in range(5)]
    dt = E.compute_dtype("fp32", True)
    bal = [E.balance(b) for b in batch_np]
    Mo = E.to_sites(mpo, dt)
    outs = E.run_queue([(lambda b=b: E.apply_compress_native(E.to_sites(bal[b][0], dt), Mo, chi,
                                                             log_norm_in=bal[b][1])) for b in range(5)], 2)
    torch.cuda.synchronize()
    for b, out in zip(batch_np, outs):
        got = [o.cpu().numpy().astype(np.complex128) for o in out]
        assert 1 - O.fidelity(O.apply_compress_sweep(b, mpo, chi), got) < 1e-6


@pytest.mark.parametrize("d,chi,cut,dt", [(3, 20, 10, np.float32), (4, 12, 40, np.complex64), (2, 16, 8, np.float64)])
def test_native_sweep_shapes(gpu, d, chi, cut, dt):
    """The native sweep on other physical dimensions and dtypes (the uneven
    batch's shapes), with chi below (truncating) and above (keeping every
    direction) the applied bonds, against the oracle's svd_compress."""
    from tncontract_gb300 import engine as E
    N = 10
    cplx = np.iscomplexobj(np.zeros(0, dt))
    sites = O.random_mps(3, N, d, chi, np.complex128 if cplx else np.float64, normalise=True)
    ident = [np.eye(d).reshape(d, d, 1, 1) for _ in range(N)]
    tdt = {np.float32: torch.float32, np.complex64: torch.complex64, np.float64: torch.float64}[dt]
    bal, ln = E.balance(sites)
    st = E.SweepStats()
    out = E.apply_compress_native(E.to_sites(bal, tdt), E.to_sites(ident, tdt), cut, log_norm_in=ln, stats=st)
    got = [o.cpu().numpy().astype(np.complex128) for o in out]
    ref = O.svd_compress_method(O.left_canonical_form_mps(sites), cut)
    tol = 1e-10 if dt == np.float64 else 1e-6
    assert 1 - O.fidelity(ref, got) < tol
    assert [a.shape[2] for a in got[:-1]] == [a.shape[2] for a in ref[:-1]]
    assert max(a.shape[2] for a in got) <= cut


def test_native_sweep_zero_state(gpu):
    from tncontract_gb300 import engine as E
    sites = [np.zeros((2, 1, 4)), np.zeros((2, 4, 4)), np.zeros((2, 4, 1))]
    ident = [np.eye(2).reshape(2, 2, 1, 1) for _ in range(3)]
    with pytest.raises(ValueError):
        E.apply_compress_native(E.to_sites(sites, torch.float64), E.to_sites(ident, torch.float64), 4)


def test_engine_run_queue(gpu):
    """Continuous batching: 6 sweep jobs on 3 worker streams give the same
    results as the oracle, in job order."""
    from tncontract_gb300 import engine as E
    N, chi = 12, 16
    mpo = O.tfim_mpo(N)
    batch_np = [O.random_mps(s, N, 2, chi, np.complex128, normalise=True) for s in range(6)]
    dt = E.compute_dtype("fp32", True)
    bal = [E.balance(b) for b in batch_np]
    Mo = E.to_sites(mpo, dt)
    jobs = [(lambda b=b: E.apply_compress(E.to_sites(bal[b][0], dt), Mo, chi, log_norm_in=bal[b][1]))
            for b in range(6)]
    outs = E.run_queue(jobs, 3)
    torch.cuda.synchronize()
    for b, out in zip(batch_np, outs):
        got = [o.cpu().numpy().astype(np.complex128) for o in out]
        assert 1 - O.fidelity(O.apply_compress_sweep(b, mpo, chi), got) < 1e-6


def test_engine_inner_product(gpu):
    from tncontract_gb300 import engine as E
    a = O.random_mps(5, 10, 3, 7, np.complex128)
    b = O.random_mps(6, 10, 3, 7, np.complex128)
    da = E.to_sites(a, torch.complex128)
    db = E.to_sites(b, torch.complex128)
    assert abs(E.inner_product(da, db) - O.inner_product(a, b)) < 1e-10 * abs(O.inner_product(a, b))


@pytest.mark.parametrize("dt", [np.float32, np.complex64, np.float64, np.complex128])
def test_sort_rows(gpu, dt):
    """tnc_sort_rows: decreasing norm, equal norms in their original order, a
    NaN row last; tnc_permute_rows with the rank restores the rows exactly."""
    from tncontract_gb300 import _ops
    rng = np.random.default_rng(3)
    A = rnd(rng, (37, 19), dt)
    A[9] = A[5]
    A[20] = 0
    A[30, 2] = np.nan
    Ms, order, rank = _ops.sort_rows(torch.from_numpy(A).cuda())
    o, r = order.cpu().numpy(), rank.cpu().numpy()
    nrm = (np.abs(A.astype(np.complex128)) ** 2).sum(1)
    assert list(o) == list(np.argsort(-nrm, kind="stable"))
    assert o[-1] == 30 and o[-2] == 20
    assert np.array_equal(r[o], np.arange(37))
    assert np.array_equal(Ms.cpu().numpy(), A[o], equal_nan=True)
    back = _ops.permute_rows(Ms, rank).cpu().numpy()
    assert np.array_equal(back, A, equal_nan=True)
