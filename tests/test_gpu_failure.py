"""Failure paths on the GPU, in the forms that leave the GPU usable: a
bounded device-side wait that runs out (a barrier, step counter or flag that
nothing completes, with the wait limit shortened for the test) returns
TNC_ERR_TIMEOUT to the host; a Jacobi held to one sweep returns
TNC_ERR_NOT_CONVERGED, which the host maps to LinAlgError; the drop-in
tensor_svd keeps the reference's failure contract (tncontract/tensor.py:
914-929: warn, retry once, re-raise).  Nothing here traps or faults."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_bounded_wait_runs_out(gpu, kind):
    from tncontract_gb300 import _lib as L
    from tncontract_gb300 import _ops
    try:
        _ops.set_spin_limit(1 << 12)
        assert _ops.wait_selftest(kind) == L.ERR_TIMEOUT
    finally:
        _ops.set_spin_limit(0)
    # the context is intact: a factorisation right after is correct
    A = torch.from_numpy(np.random.default_rng(0).standard_normal((40, 30))).cuda()
    _u, S, _vh = _ops.svd(A)
    assert np.allclose(S.cpu().numpy(), np.linalg.svd(A.cpu().numpy(), compute_uv=False), rtol=1e-12, atol=1e-12)


def test_jacobi_sweep_cap_raises(gpu):
    from tncontract_gb300 import _lib as L
    from tncontract_gb300 import _ops
    from tncontract_gb300 import engine as E
    A = torch.from_numpy(np.random.default_rng(1).standard_normal((64, 64))).cuda()
    infos = []
    with pytest.raises(_ops.LinAlgError):
        _ops.svd(A, max_sweeps=1, info_out=infos)
    assert int(infos[0][0].item()) == L.ERR_NOT_CONVERGED and int(infos[0][1].item()) == 1
    _w, _s, _o, info = _ops.svd_rows(A, max_sweeps=1, block_rows=8)
    assert int(info[0].item()) == L.ERR_NOT_CONVERGED
    with pytest.raises(_ops.LinAlgError):
        E._check_info(info)


def test_tensor_svd_retry_contract(gpu, monkeypatch):
    import tncontract_gb300 as tn
    from tncontract_gb300 import _ops
    from tncontract_gb300 import tensor as T
    rng = np.random.default_rng(2)
    t = tn.Tensor(rng.standard_normal((8, 6, 10)), ["a", "b", "c"])
    # first attempt capped at one sweep: warn, retry with the default cap, succeed
    monkeypatch.setattr(T, "SVD_SWEEPS", 1)
    with pytest.warns(UserWarning, match="retrying"):
        U, S, V = tn.tensor_svd(t, ["a", "b"])
    s_ref = np.linalg.svd(t.to_numpy().reshape(48, 10), compute_uv=False)
    assert np.allclose(np.diag(S.to_numpy()), s_ref, rtol=1e-12)
    # the retry capped too: LinAlgError after the warning
    monkeypatch.setattr(T, "SVD_RETRY_SWEEPS", 1)
    with pytest.warns(UserWarning, match="retrying"):
        with pytest.raises(_ops.LinAlgError):
            tn.tensor_svd(t, ["a", "b"])


def test_tensor_svd_nonfinite_reports(gpu, capsys):
    import tncontract_gb300 as tn
    a = np.ones((4, 5))
    a[1, 2] = np.nan
    with pytest.warns(UserWarning):
        with pytest.raises(ValueError):
            tn.tensor_svd(tn.Tensor(a, ["r", "c"]), ["r"])
    out = capsys.readouterr().out
    assert "Matrix contains inf's: False. Matrix contains nan's: True" in out
