"""The other workloads on the GPU: the 2-D boundary-MPS contraction of a PEPS
norm network (drop-in FP64 path and FP32 engine) against the values the
reference computed, and a slice of the uneven batch (left-canonise,
svd_compress to chi/2, norm) against the oracle."""
import numpy as np
import pytest
import torch

import api_cases as K
import tn_oracle as O

pytestmark = pytest.mark.gpu


def _peps(tn, rows):
    return tn.twodim.SquareLatticePEPS(
        [[tn.Tensor(a, ["phys", "up", "right", "down", "left"]) for a in r] for r in rows])


def test_peps_4x4_dropin_and_engine(gpu):
    from tncontract_gb300 import engine as E
    from tncontract_gb300 import workloads as W
    g, m = K.load("peps")
    rows = O.random_peps(2, 4, 4, 2, 2)
    tn = gpu
    v = tn.twodim.inner_product_peps(_peps(tn, rows), _peps(tn, rows), exact_contract=False, chi=4)
    ref = float(g["p4_value"])
    assert abs(float(v) - ref) < 1e-10 * ref
    ex = tn.twodim.inner_product_peps(_peps(tn, rows), _peps(tn, rows), exact_contract=True)
    assert abs(float(ex.data.item()) - float(g["p4_exact"])) < 1e-10 * abs(float(g["p4_exact"]))
    val, log10, _ = E.boundary_mps_contract(W.double_layer_arrays(rows), 4, precision="fp32")
    assert abs(val - ref) < 1e-5 * ref


def test_peps_8x8_dropin_chi16(gpu):
    g, m = K.load("peps")
    rows = O.random_peps(2, 8, 8, 4, 2)
    tn = gpu
    v = tn.twodim.inner_product_peps(_peps(tn, rows), _peps(tn, rows), exact_contract=False, chi=16)
    ref = float(g["p8c16_value"])
    assert abs(float(v) - ref) < 1e-9 * ref


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-4), ("fp64", 1e-9)])
def test_peps_8x8_engine_chi64(gpu, precision, tol):
    """Config 4: 8x8 PEPS norm, D=4, d=2, boundary chi=64 (the reference:
    4.831813278736701e115); relative error of the scalar."""
    from tncontract_gb300 import engine as E
    from tncontract_gb300 import workloads as W
    g, m = K.load("peps")
    rows = W.random_peps_arrays(2, 8, 8, 4, 2)
    val, log10, phase = E.boundary_mps_contract(W.double_layer_arrays(rows), 64, precision=precision)
    ref = float(g["p8c64_value"])
    assert abs(log10 - m["p8c64_log10"]) < tol
    assert abs(val - ref) < 3 * tol * ref


def test_uneven_batch_slice(gpu):
    """A few instances of the uneven batch (sizes scaled down): left-canonise,
    svd_compress(chi // 2), norm; fidelity and norm against the oracle."""
    from tncontract_gb300 import engine as E
    from tncontract_gb300 import workloads as W
    specs = [(N // 4, d, chi // 4, dt, s) for (N, d, chi, dt, s) in W.config3_specs(1, 6)]
    jobs, refs = [], []
    for (N, d, chi, dt, s) in specs:
        sites = W.random_mps_arrays(s, max(N, 4), d, max(chi, 4), dt)
        lc = O.left_canonical_form_mps([a.astype(np.complex128 if np.iscomplexobj(a) else np.float64)
                                        for a in sites])
        ref = O.svd_compress_method(lc, max(chi, 4) // 2)
        refs.append(ref)
        bal, ln = E.balance(sites)
        dsites = E.to_sites(bal, torch.complex64 if np.iscomplexobj(sites[0]) else torch.float32)
        jobs.append((lambda ds=dsites, c=max(chi, 4) // 2, l0=ln: E.compress(ds, c, log_norm_in=l0)))
    outs = E.run_batch(jobs)
    for (sites_out, ln), ref in zip(outs, refs):
        got = [o.cpu().numpy().astype(np.complex128) for o in sites_out]
        assert 1 - O.fidelity(ref, got) < 1e-6
        nr = O.mps_norm(ref)
        assert abs(O.mps_norm(got) * np.exp(ln) - nr) < 1e-5 * nr
