"""Config 5 at full size on the GPU: a random MPS (N=128, d=2, chi=512,
float32 storage) under the XXZ MPO (Delta=0.8, D=5), compressed with the
discarded-weight rule (1e-8, at most chi), with and without the learned rank
predictor (trained here by the library's MLP kernels on spectra of configs
1-3).  Wherever the predictor's randomized SVD is accepted its result must
hold the same fidelity bound as the full SVD's: the learned sweep agrees
with the plain one to 1e-6 in fidelity and keeps the same bond dimensions,
and every bond's outcome (sketch accepted, fallback, sketch declined because
the bond cap sets the rank, full SVD) is counted."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_config5_full_size_learned_vs_plain(gpu):
    from tncontract_gb300 import engine as E
    from tncontract_gb300 import learned as LR
    tol = 1e-8
    model, hist, ntrain = LR.train_rank_model(tol, steps=300)
    assert ntrain > 50 and hist[-1] < hist[0]
    sites, mpo = LR.config5_inputs(128, 2, 512)
    plain, t_plain, rs_plain, _ = LR.config5(sites, mpo, 512, tol)
    learn, t_learn, rs_learn, _ = LR.config5(sites, mpo, 512, tol, model=model)
    assert [a.shape[2] for a in learn] == [a.shape[2] for a in plain]
    assert max(a.shape[2] for a in plain) == 512
    f = E.fidelity([x.to(torch.float64) for x in plain], [x.to(torch.float64) for x in learn])
    assert 1.0 - f < 1e-6
    # every one of the 127 bonds either took an accepted sketch or the full
    # SVD (fallbacks are full SVDs after a rejected sketch)
    assert rs_learn.sketched + rs_learn.full == 127
    assert rs_learn.fallbacks + rs_learn.declined <= rs_learn.full
    assert LR.fallback_rate(rs_learn) is None or 0.0 <= LR.fallback_rate(rs_learn) <= 1.0
