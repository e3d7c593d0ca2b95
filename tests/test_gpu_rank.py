"""Learned rank predictor on the GPU: the MLP's forward/backward/Adam kernels
against the float64 oracle (oracle/mlp_oracle.py), the Gaussian sketch
generator, and what the trained predictor gains in the truncating sweep
(randomized SVD sized by the prediction, the full SVD as fallback when the
sketch fails its residual check)."""
import numpy as np
import pytest
import torch

import mlp_oracle as MO
import tn_oracle as O

pytestmark = pytest.mark.gpu


def test_mlp_forward_backward_adam_vs_oracle(gpu):
    from tncontract_gb300 import rank_model as RM
    m = RM.RankMLP(seed=3)
    rng = np.random.default_rng(0)
    X = rng.random((200, RM.N_FEATURES)).astype(np.float32)
    T = rng.random(200).astype(np.float32)
    y, _ = m.forward(torch.from_numpy(X).cuda())
    y_ref, _ = MO.forward(m.params.cpu().numpy(), X, RM.N_FEATURES, 128)
    assert np.max(np.abs(y.cpu().numpy() - y_ref)) < 1e-5
    m.backward(torch.from_numpy(X).cuda(), torch.from_numpy(T).cuda())
    g = m.grads.cpu().numpy()
    g_ref = MO.grads(m.params.cpu().numpy(), X, T, RM.N_FEATURES, 128)
    assert np.linalg.norm(g - g_ref) < 1e-4 * np.linalg.norm(g_ref)
    p0 = m.params.cpu().numpy().astype(np.float64)
    m.adam(lr=1e-2)
    p_ref, _, _ = MO.adam(p0, g_ref, np.zeros_like(p0), np.zeros_like(p0), 1e-2, 0.9, 0.999, 1e-8, 1)
    assert np.max(np.abs(m.params.cpu().numpy() - p_ref)) < 1e-5


def test_gaussian_fill(gpu):
    from tncontract_gb300 import _ops
    a = _ops.fill_gaussian((1000, 500), torch.complex64, 7).cpu().numpy()
    assert abs(a.real.mean()) < 0.01 and abs(a.imag.mean()) < 0.01
    assert abs(a.real.var() - 1) < 0.02 and abs(a.imag.var() - 1) < 0.02
    b = _ops.fill_gaussian((1000, 500), torch.complex64, 7).cpu().numpy()
    assert np.array_equal(a, b)


def _sweep(E, sites, mpo_np, precision, **kw):
    dt = E.compute_dtype(precision, True)
    bal, ln = E.balance(sites)
    rs = E.RankStats()
    out = E.apply_compress(E.to_sites(bal, dt), E.to_sites(mpo_np, dt), 0, log_norm_in=ln, rank_stats=rs, **kw)
    torch.cuda.synchronize()
    return [o.cpu().numpy().astype(np.complex128) for o in out], rs


def test_learned_rank_gain(gpu):
    """XXZ (D=5) MPO on random MPS, discarded-weight tolerance 1e-8: the
    predictor trained on spectra of plain sweeps sizes randomized SVDs that
    cover the bonds with less factorisation work than the full SVD, at the
    same fidelity bound (<= 1e-6 against the FP64 oracle)."""
    from tncontract_gb300 import engine as E
    from tncontract_gb300 import rank_model as RM
    N, chi, tol = 24, 64, 1e-8
    mpo = O.xxz_mpo(N)
    feats, targets = [], []
    for seed in range(4):
        sites = O.random_mps(seed, N, 2, chi, np.complex128, normalise=True)
        _, rs = _sweep(E, sites, mpo, "fp32", dw_tol=tol)
        feats += rs.features
        targets += rs.targets
    model = RM.RankMLP(seed=0)
    hist = model.fit(np.array(feats), np.array(targets), steps=400)
    assert hist[-1] < 0.1 * hist[0]
    sites = O.random_mps(11, N, 2, chi, np.complex128, normalise=True)
    ref = MO.svd_compress_dw(O.contract_mps_mpo(sites, mpo), 0, tol)
    plain, rs_plain = _sweep(E, sites, mpo, "fp32", dw_tol=tol)
    learned, rs_learn = _sweep(E, sites, mpo, "fp32", dw_tol=tol, rank_model=model)
    assert 1 - O.fidelity(ref, plain) < 1e-6
    assert 1 - O.fidelity(ref, learned) < 1e-6
    assert rs_learn.sketched > 0
    assert rs_learn.rows_factored < rs_plain.rows_factored
